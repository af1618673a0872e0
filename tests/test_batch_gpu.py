"""Batched uneven CGSEM solves against the single-problem solver (GPU)."""
import numpy as np
import pytest

from helpers import rel_inf

pytestmark = pytest.mark.gpu


def _problems(sg, specs):
    from self_gb300 import workloads as W
    return [W.batched_problem(sg, nx, N, seed) for nx, N, seed in specs]


@pytest.mark.parametrize("precision", ["fp32", "fp64"])
def test_batch_matches_single_solves(gpu_ctx, precision, tmp_path):
    import self_gb300 as sg
    specs = [(4, 3, 11), (6, 5, 12), (5, 7, 13), (3, 9, 14), (7, 4, 15), (4, 8, 16)]
    probs = _problems(sg, specs)
    B = sg.CGBatch(gpu_ctx, probs)
    tune = B.autotune(str(tmp_path / "tune.json"))
    assert all(v >= 1 for v in tune.values())
    reps = B.Solve(precision=precision, tolerance=1e-10)
    for p, pr in enumerate(probs):
        assert reps[p]["ioerr"] == 0 and reps[p]["rel_residual"] < 1e-10, reps[p]
        cg = sg.CGsemElliptic_2D(gpu_ctx, pr["nodal"], pr["mesh"], pr["k"], lam=pr["lam"])
        ref, rr = cg.Solve(pr["source"], method="pcg", tolerance=1e-10)
        assert rel_inf(B.GetSolution(p), ref) < 1e-8
        if precision == "fp64":
            assert abs(reps[p]["iterations"] - rr["iterations"]) <= max(2, 0.02 * rr["iterations"])
    # a second tuner pass reads the cache
    B2 = sg.CGBatch(gpu_ctx, probs[:2])
    t2 = B2.autotune(str(tmp_path / "tune.json"))
    assert t2[(3, 0)] == tune[(3, 0)]


@pytest.mark.parametrize("precision", ["fp32", "fp64"])
def test_batch_resolve_after_short_solve(gpu_ctx, precision):
    """A solve capped at a few iterations, then a full solve of the same pool: the second one converges and
    equals a solve on a fresh pool (the iteration cap is not left behind in the captured iteration graph)."""
    import self_gb300 as sg
    specs = [(5, 4, 21), (6, 6, 22), (4, 7, 23)]
    probs = _problems(sg, specs)
    B = sg.CGBatch(gpu_ctx, probs)
    short = B.Solve(precision=precision, tolerance=1e-10, maxIters=8)
    assert all(r["ioerr"] == -1 for r in short)
    reps = B.Solve(precision=precision, tolerance=1e-10)
    fresh = sg.CGBatch(gpu_ctx, probs)
    reps_f = fresh.Solve(precision=precision, tolerance=1e-10)
    for p in range(len(probs)):
        assert reps[p]["ioerr"] == 0 and reps[p]["rel_residual"] < 1e-10, reps[p]
        assert reps[p]["iterations"] == reps_f[p]["iterations"]
        assert np.array_equal(B.GetSolution(p), fresh.GetSolution(p))
