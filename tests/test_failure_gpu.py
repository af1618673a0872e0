"""Failure detection without a GPU fault: each failure is made on the host or by a bounded wait that is made to
run out, and the library must report it as a status while the CUDA context stays usable.

* Bounded waits: the fused FP32 shallow-water stage's bulk-copy waits are bounded; the time-out test hook makes the
  first wait of every warp poll a barrier nothing arrives on, so the call returns SELF_ERR_TIMEOUT, leaves the
  state unchanged, and the next call on the same handle (and a fresh handle) steps normally.
* Non-finite residuals: a NaN or Inf in the source or the initial guess makes self_cg2d_solve return
  SELF_ERR_NONFINITE (ioerr -7 in the report) for PCG, FP32-refined PCG, GMRES and FP32-inner GMRES, before any
  iteration.
* Unsupported options return SELF_ERR_UNSUPPORTED.
The reference signals solver failure through ioerr (IterativeSolvers_Class.f90:357,402) and stops on fatal errors.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TIMEOUT, NONFINITE, UNSUPPORTED = -5, -7, -4


def _sw32(sg, W, gpu_ctx, precision):
    N, nx = 7, 8
    nod = sg.NodalStorage_2D(N)
    mesh = sg.QuadMesh(nx, nx, N, warp=W.SW_WARP, scale=(W.SW_L, W.SW_L))
    q, h, fcor, dt = W.shallow_water(mesh, N, nx, seed=2)
    dhdx, dhdy = sg.bathymetry_gradient(nod, mesh, h)
    sw = sg.ShallowWater(gpu_ctx, nod, mesh, h, fcor, dt, dhdx=dhdx, dhdy=dhdy, precision=precision)
    sw.SetSolution(q)
    return sw, q


def test_fused_stage_wait_timeout_is_reported_and_recoverable(gpu_ctx):
    import self_gb300 as sg
    from self_gb300 import _native as nat
    from self_gb300 import workloads as W
    L = nat.lib()
    sw, q = _sw32(sg, W, gpu_ctx, nat.PREC_FP32)
    before = sw.GetSolution()
    nat.check(L.self_dg2d_test_wait_timeout(sw.ptr, C.c_int(16)), gpu_ctx.ptr)
    with pytest.raises(nat.SelfError) as ei:
        sw.ForwardStepRK3(0.0, 1)
    assert ei.value.status == TIMEOUT
    assert "ran out" in str(ei.value)
    assert np.array_equal(sw.GetSolution(), before)  # no warp wrote anything
    # the hook applied to one call: the same handle and a fresh handle now step identically
    sw.ForwardStepRK3(0.0, 3)
    got = sw.GetSolution()
    fresh, _ = _sw32(sg, W, gpu_ctx, nat.PREC_FP32)
    fresh.ForwardStepRK3(0.0, 3)
    assert np.array_equal(got, fresh.GetSolution())
    assert np.all(np.isfinite(got)) and not np.array_equal(got, before)
    sw.Trash()
    fresh.Trash()


def test_wait_timeout_hook_unsupported_outside_fused_stage(gpu_ctx):
    import self_gb300 as sg
    from self_gb300 import _native as nat
    from self_gb300 import workloads as W
    sw, _ = _sw32(sg, W, gpu_ctx, nat.PREC_FP64)
    assert nat.lib().self_dg2d_test_wait_timeout(sw.ptr, C.c_int(16)) == UNSUPPORTED
    sw.ForwardStepRK3(0.0, 1)  # the handle is unaffected
    sw.Trash()


@pytest.mark.parametrize("method,precision", [("pcg", "fp64"), ("pcg", "fp32"), ("gmres", "fp64"), ("gmres", "fp32"),
                                              ("cg", "fp64")])
def test_nonfinite_source_is_reported(gpu_ctx, method, precision):
    import self_gb300 as sg
    from self_gb300 import _native as nat
    from self_gb300 import workloads as W
    N, nx = 5, 6
    nod = sg.NodalStorage_2D(N, nat.GAUSS_LOBATTO, nat.CG)
    mesh = sg.QuadMesh(nx, nx, N, nat.GAUSS_LOBATTO, boundary_flag=nat.DIRICHLET)
    k, f, source = W.helmholtz(mesh, N)
    cg = sg.CGsemElliptic_2D(gpu_ctx, nod, mesh, k, lam=0.1)
    bad = source.copy()
    bad[bad.size // 2 + 3] = np.nan
    with pytest.raises(nat.SelfError) as ei:
        cg.Solve(bad, method=method, precision=precision, tolerance=1e-10, maxIters=500)
    assert ei.value.status == NONFINITE
    guess = np.zeros(cg.nl)
    n = N + 1
    guess[10 * n * n + 2 + 2 * n] = np.inf  # an element-interior node (no other copy overwrites it)
    with pytest.raises(nat.SelfError) as ei:
        cg.Solve(source, solution=guess, method=method, precision=precision, tolerance=1e-10, maxIters=500)
    assert ei.value.status == NONFINITE
    # the handle and the context stay usable
    sol, rep = cg.Solve(source, method="pcg", tolerance=1e-10, maxIters=2000)
    assert rep["ioerr"] == 0 and np.all(np.isfinite(sol))
    cg.Trash()


def test_unsupported_options(gpu_ctx):
    import self_gb300 as sg
    from self_gb300 import _native as nat
    from self_gb300 import workloads as W
    N, nx = 3, 4
    nod = sg.NodalStorage_2D(N)
    mesh = sg.QuadMesh(nx, nx, N, warp=0.0, scale=(W.SW_L, W.SW_L))
    q, h, fcor, dt = W.shallow_water(mesh, N, nx, seed=2)
    with pytest.raises(nat.SelfError) as ei:  # the FP32 form covers the conservative and advection models
        sg.ShallowWater(gpu_ctx, nod, mesh, h, fcor, dt, precision=nat.PREC_FP32, formulation="linear")
    assert ei.value.status == UNSUPPORTED
