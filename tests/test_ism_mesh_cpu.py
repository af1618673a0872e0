"""ISM-V2 (SpecMesh) mesh files: the product reader against the oracle's restatement of ReadSpecMeshFile on the
reference's example meshes (tests/golden/square.mesh: curved boundary records of degree 5, Dirichlet sides;
tests/golden/box.mesh: 448 straight-sided elements, no-normal-flow walls)."""
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
MESHES = [("square.mesh", 64, 144, 81, 5, -200, 32), ("box.mesh", 448, 936, 489, 1, -100, 80)]


@pytest.mark.parametrize("name,nel,ned,nno,gdeg,flag,nbnd", MESHES)
@pytest.mark.parametrize("N,quad", [(4, -1), (7, 1)])
def test_ism_reader_matches_oracle(oracle, name, nel, ned, nno, gdeg, flag, nbnd, N, quad):
    import self_gb300 as sg
    path = os.path.join(HERE, "golden", name)
    m = sg.read_ism_mesh(path, N, quad)
    o = oracle.IsmMesh(path, N, quad)
    assert (m.nEl, m.nEdges, m.nNodes, m.geomDegree) == (nel, ned, nno, gdeg)
    for f in ("edges", "elemNodes", "nodeType", "n2e_ptr", "n2e_elem", "n2e_local"):
        assert np.array_equal(getattr(m, f), getattr(o, f)), f
    for f in ("x", "y", "dxds", "dxdp", "dyds", "dydp", "J", "nhx", "nhy", "nlen", "bx", "by"):
        a, b = getattr(m, f), getattr(o, f)
        assert np.abs(a - b).max() <= 1e-12 * max(1.0, np.abs(b).max()), f  # rounding of the curve interpolants
    e = m.edges.reshape(-1, 6)
    assert (e[:, 2] < 0).sum() == nbnd and set(e[e[:, 2] < 0, 2]) == {flag}
    assert (m.J > 0).all()


def test_ism_geometry_properties():
    """Areas add up to the unit square; at every matched interior edge node the two elements' normals are
    opposite and their length elements agree."""
    import self_gb300 as sg
    N = 5
    nod = sg.NodalStorage_2D(N, sg._native.GAUSS_LOBATTO, sg._native.CG)
    for name in ("square.mesh", "box.mesh"):
        m = sg.read_ism_mesh(os.path.join(HERE, "golden", name), N, sg._native.GAUSS_LOBATTO)
        W = np.outer(nod.w, nod.w).ravel()
        assert abs((m.J.reshape(m.nEl, -1) * W).sum() - 1.0) < 1e-12
        n = N + 1
        nh = np.stack([m.nhx, m.nhy]).reshape(2, m.nEl, 4, n)
        ln = m.nlen.reshape(m.nEl, 4, n)
        for e1, s1, e2, s2, st, inc in m.edges.reshape(-1, 6):
            if e2 <= 0:
                continue
            for i in range(n):
                k = (st - inc + i * inc) if N > 1 else i
                k = i if inc > 0 else N - i
                a = nh[:, e1 - 1, s1 - 1, i]
                b = nh[:, e2 - 1, abs(s2) - 1, k]
                assert np.abs(a + b).max() < 1e-12
                assert abs(ln[e1 - 1, s1 - 1, i] - ln[e2 - 1, abs(s2) - 1, k]) < 1e-12 * ln[e1 - 1, s1 - 1, i]


def test_ism_reader_rejects_a_truncated_file(tmp_path):
    import self_gb300 as sg
    src = open(os.path.join(HERE, "golden", "square.mesh")).read().splitlines()
    bad = tmp_path / "cut.mesh"
    bad.write_text("\n".join(src[:200]) + "\n")
    with pytest.raises(sg._native.SelfError):
        sg.read_ism_mesh(str(bad), 4, -1)
