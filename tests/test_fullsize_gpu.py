"""Size-independent properties at the benchmark sizes (the oracle is too slow there).

* 128x128 quads, N = 7 shallow water (3,145,728 DOF): total mass sum(w_i w_j J H) is conserved by the LLF flux with
  mirror walls, in the FP64 drop-in (to 1e-13 relative over 100 steps) and in the FP32 perturbation form (to the
  FP32 rounding of eta, 1e-9 of the total); from a lake at rest both forms drift the same way (the discrete
  h^2/2 derivative is not exactly h times the discrete dh/dx, and the FP32 form carries that FP64 lake-at-rest
  tendency): after 20 steps the FP32 heights equal the FP64 ones to 1e-9 of max H and the velocities to 1e-3
  of the FP64 drift.
* 256x256 quads, N = 7 Helmholtz (4,194,304 local nodes): the operator is symmetric, <A u, v> = <u, A v> to 1e-12
  relative, and the FP32-refined and FP64 PCG solutions agree to 1e-8.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _sw(sg, W):
    N, nx = 7, 128
    nod = sg.NodalStorage_2D(N)
    mesh = sg.QuadMesh(nx, nx, N, warp=W.SW_WARP, scale=(W.SW_L, W.SW_L))
    q, h, fcor, dt = W.shallow_water(mesh, N, nx, seed=2)
    dhdx, dhdy = sg.bathymetry_gradient(nod, mesh, h)
    return nod, mesh, q, h, fcor, dt, dhdx, dhdy


def test_fullsize_sw_mass_conservation(gpu_ctx):
    import self_gb300 as sg
    from self_gb300 import workloads as W
    nod, mesh, q, h, fcor, dt, dhdx, dhdy = _sw(sg, W)
    n2 = nod.n * nod.n
    w2 = np.outer(nod.w, nod.w).ravel()
    J = mesh.J.reshape(mesh.nEl, n2)

    def mass(state):
        return float(np.sum(w2 * J * state.reshape(mesh.nEl, 3, n2)[:, 2]))

    m0 = mass(q)
    for prec, tol in ((sg._native.PREC_FP64, 1e-13), (sg._native.PREC_FP32, 1e-9)):
        sw = sg.ShallowWater(gpu_ctx, nod, mesh, h, fcor, dt, dhdx=dhdx, dhdy=dhdy, precision=prec)
        sw.SetSolution(q)
        sw.ForwardStepRK3(0.0, 100)
        m1 = mass(sw.GetSolution())
        sw.Trash()
        assert abs(m1 - m0) <= tol * abs(m0), (prec, m1, m0)


def test_fullsize_lake_at_rest(gpu_ctx):
    import self_gb300 as sg
    from self_gb300 import workloads as W
    nod, mesh, q, h, fcor, dt, dhdx, dhdy = _sw(sg, W)
    n2 = nod.n * nod.n
    rest = np.zeros((mesh.nEl, 3, n2))
    rest[:, 2] = h.reshape(mesh.nEl, n2)
    rest = rest.ravel()
    out = {}
    for prec in (sg._native.PREC_FP64, sg._native.PREC_FP32):
        sw = sg.ShallowWater(gpu_ctx, nod, mesh, h, fcor, dt, dhdx=dhdx, dhdy=dhdy, precision=prec)
        sw.SetSolution(rest)
        sw.ForwardStepRK3(0.0, 20)
        out[prec] = sw.GetSolution().reshape(mesh.nEl, 3, n2)
        sw.Trash()
    a, b = out[sg._native.PREC_FP64], out[sg._native.PREC_FP32]
    assert np.abs(b[:, 2] - a[:, 2]).max() <= 1e-9 * np.abs(a[:, 2]).max()
    for v in (0, 1):
        drift = np.abs(a[:, v]).max()
        assert np.abs(b[:, v] - a[:, v]).max() <= 1e-3 * drift + 1e-12


def test_fullsize_helmholtz_symmetry_and_fp32_refinement(gpu_ctx):
    import self_gb300 as sg
    from self_gb300 import workloads as W
    nat = sg._native
    N, nx = 7, 256
    nod = sg.NodalStorage_2D(N, nat.GAUSS_LOBATTO, nat.CG)
    mesh = sg.QuadMesh(nx, nx, N, nat.GAUSS_LOBATTO, boundary_flag=nat.DIRICHLET)
    k, f, source = W.helmholtz(mesh, N, seed=3)
    cg = sg.CGsemElliptic_2D(gpu_ctx, nod, mesh, k, lam=0.1)
    rng = np.random.default_rng(11)
    u = cg.UnMask(cg.Mask(rng.normal(size=cg.nl)))
    v = cg.UnMask(cg.Mask(rng.normal(size=cg.nl)))
    a, b = cg.DotProduct(cg.MatrixAction(u), v), cg.DotProduct(u, cg.MatrixAction(v))
    assert abs(a - b) <= 1e-12 * max(abs(a), abs(b))
    s64, r64 = cg.Solve(source, method="pcg", tolerance=1e-10)
    s32, r32 = cg.Solve(source, method="pcg", precision="fp32", tolerance=1e-10)
    assert r64["ioerr"] == 0 and r32["ioerr"] == 0
    assert np.abs(s32 - s64).max() <= 1e-8 * np.abs(s64).max()
    cg.Trash()
