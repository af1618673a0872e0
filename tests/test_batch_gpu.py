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


def test_pool_growth_keeps_running_solves(gpu_ctx):
    """Continuous batching through the C ABI: one problem is stepped for a few ticks, then 20 more join (the slot
    arrays grow past their first capacity of 16 while the first solve runs on the device); every problem converges
    and the first one's solution is bit-identical to a pool that never grew."""
    import ctypes as C

    import self_gb300 as sg
    from self_gb300 import _native as nat
    from self_gb300.cgsem import SolveOpts, SolveReport, cg2d_desc
    L = nat.lib()
    specs = [(6, 5, 31)] + [(4 + (i % 3), 3 + (i % 5), 40 + i) for i in range(20)]
    probs = _problems(sg, specs)
    o = SolveOpts()
    o.method, o.precision, o.maxIters, o.tolerance = 1, nat.PREC_FP32, 20000, 1e-10
    o.inner_tolerance, o.max_outer = 1e-4, 30

    def run(batch_from):
        bp = C.c_void_p()
        nat.check(L.self_cgbatch_create(gpu_ctx.ptr, 0, None, C.byref(bp)), gpu_ctx.ptr)
        keep, slots = [], []
        try:
            for i, pr in enumerate(probs[:batch_from]):
                d, k = cg2d_desc(pr["nodal"], pr["mesh"], pr["k"], pr["lam"])
                src = np.ascontiguousarray(pr["source"])
                keep.append((d, k, src))
                s = C.c_int()
                nat.check(L.self_cgbatch_add(bp, C.byref(d), nat.d(src), C.byref(s)), gpu_ctx.ptr)
                slots.append(s.value)
                if i == 0:
                    for _ in range(3):  # the first solve is under way before the pool grows
                        nat.check(L.self_cgbatch_step(bp, C.byref(o), C.byref(C.c_int())), gpu_ctx.ptr)
            for _ in range(100000):
                nfin = C.c_int()
                nat.check(L.self_cgbatch_step(bp, C.byref(o), C.byref(nfin)), gpu_ctx.ptr)
                if nfin.value == len(slots):
                    break
            reps, sols = [], []
            for s, pr in zip(slots, probs):
                rep, fin = SolveReport(), C.c_int()
                nat.check(L.self_cgbatch_report(bp, s, C.byref(rep), C.byref(fin)))
                reps.append((rep.as_dict(), fin.value))
                out = np.zeros(pr["mesh"].nEl * (pr["nodal"].N + 1) ** 2)
                nat.check(L.self_cgbatch_get_solution(bp, s, nat.d(out)))
                sols.append(out)
            return reps, sols
        finally:
            L.self_cgbatch_destroy(bp)

    reps, sols = run(len(probs))
    for rep, fin in reps:
        assert fin == 1 and rep["r0"] > 0 and rep["rel_residual"] < 1e-10 and rep["outer_iterations"] >= 1, rep
    alone_reps, alone_sols = run(1)
    assert alone_reps[0][0]["iterations"] == reps[0][0]["iterations"]
    assert np.array_equal(alone_sols[0], sols[0])
