"""Pickup (checkpoint) files in the reference's format: byte layout against the oracle's restatement of
WritePickup, and read-back of every field."""
import os

import numpy as np


def test_shallow_water_pickup_bytes_and_read_back(oracle, tmp_path):
    from self_gb300.dgsem import read_pickup, write_pickup
    rng = np.random.default_rng(11)
    N, nEl = 5, 7
    nn = (N + 1) ** 2
    q, h, f = rng.normal(size=3 * nn * nEl), rng.normal(size=nn * nEl), rng.normal(size=nn * nEl)
    path = str(tmp_path / "ShallowWater.0000000042.pickup")
    write_pickup(path, N, nEl, [(q, 3), (h, 1), (f, 1)])
    data = open(path, "rb").read()
    assert len(data) == 5 * 8 * nn * nEl
    assert data == oracle.pickup_bytes(N, nEl, [(q, 3), (h, 1), (f, 1)])
    q2, h2, f2 = np.zeros_like(q), np.zeros_like(h), np.zeros_like(f)
    read_pickup(path, N, nEl, [(q2, 3), (h2, 1), (f2, 1)])
    assert np.array_equal(q, q2) and np.array_equal(h, h2) and np.array_equal(f, f2)
    q3 = np.zeros_like(q)
    read_pickup(path, N, nEl, [(q3, 3), (None, 1), (None, 1)])  # skipped fields
    assert np.array_equal(q, q3)


def test_advection_pickup_layout(oracle, tmp_path):
    from self_gb300.dgsem import write_pickup
    rng = np.random.default_rng(12)
    N, nEl, nEq = 3, 4, 2
    nn = (N + 1) ** 2
    fields = [(rng.normal(size=nEq * nn * nEl), nEq), (rng.normal(size=nEq * nn * nEl), nEq),
              (rng.normal(size=nEq * nn * nEl), nEq), (rng.normal(size=nn * nEl), 1), (rng.normal(size=nn * nEl), 1)]
    path = str(tmp_path / "Advection.0000000001.pickup")
    write_pickup(path, N, nEl, fields)
    assert open(path, "rb").read() == oracle.pickup_bytes(N, nEl, fields)


def test_truncated_pickup_is_an_error(tmp_path):
    import pytest
    from self_gb300 import _native as nat
    from self_gb300.dgsem import read_pickup, write_pickup
    N, nEl = 2, 3
    nn = (N + 1) ** 2
    path = str(tmp_path / "p.pickup")
    write_pickup(path, N, nEl, [(np.ones(nn * nEl), 1)])
    with open(path, "r+b") as fh:
        fh.truncate(os.path.getsize(path) - 8)
    with pytest.raises(nat.SelfError):
        read_pickup(path, N, nEl, [(np.zeros(nn * nEl), 1)])
