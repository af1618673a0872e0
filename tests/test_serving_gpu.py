"""Continuous-batching serving loop: every result computed in the mix equals the same request served alone."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _reqs(sg, seed=5):
    from self_gb300 import serving as S
    reqs = S.make_requests(sg, 9, rate=1e6, seed=seed, sw_nx=8, sw_N=5, sw_steps=20, helmholtz_nmax=10)
    assert any(r.kind == "sw" for r in reqs) and any(r.kind == "helmholtz" for r in reqs)
    return reqs


def test_results_identical_alone_and_in_the_mix(gpu_ctx):
    import self_gb300 as sg
    from self_gb300 import serving as S
    reqs = _reqs(sg)
    srv = S.Server(gpu_ctx, sw_streams=2, sw_chunk=5)
    srv.run(reqs)
    stats = S.latency_stats(reqs)
    assert stats["requests"] == len(reqs) and stats["p99_ms"] >= stats["p50_ms"] > 0
    srv.close()
    for r in reqs:
        assert r.finished is not None and r.result is not None
        if r.kind == "helmholtz":
            assert r.report["rel_residual"] < 1e-10
        alone = S.Request(r.rid, r.kind, 0.0, r.payload)
        solo = S.Server(gpu_ctx, sw_streams=1, sw_chunk=5)
        solo.run([alone])
        solo.close()
        assert np.array_equal(alone.result, r.result), (r.rid, r.kind)


def test_admission_respects_the_budget(gpu_ctx):
    """With a budget that fits one request at a time, requests still complete (queued, then admitted)."""
    import self_gb300 as sg
    from self_gb300 import serving as S
    reqs = _reqs(sg, seed=7)[:4]
    srv = S.Server(gpu_ctx, sw_streams=1, sw_chunk=5)
    srv.budget = max(srv.footprint(r) for r in reqs)
    srv.run(reqs)
    srv.close()
    assert all(r.finished is not None for r in reqs)
    # with room for a single request the service is sequential: admissions follow completions
    order = sorted(reqs, key=lambda r: r.admitted)
    for a, b in zip(order, order[1:]):
        assert b.admitted >= a.finished - 1e-9 or srv.footprint(a) + srv.footprint(b) <= srv.budget
