"""Parity with the oracle and size-independent properties at the benchmark sizes.

Parity (the drop-in against the oracle, both fed the oracle's own set-up: oracle.Nodal, oracle.Mesh and the
oracle's bathymetry gradient; the oracle runs OpenMP over all host cores):
* 128x128 quads, N = 7 shallow water (3,145,728 DOF, seed 2): one GlobalTimeDerivative of the same state with a
  seeded velocity field <= 1e-12 per variable (||gpu - oracle||_inf / ||oracle||_inf); of the configured state
  (zero velocity: an ill-conditioned lake-at-rest cancellation) within 4x the oracle's own spread under a one-ulp
  change of its inputs; 100 ForwardStepRK3 steps from the configured state <= 1e-11 per variable or within 4x the
  oracle's one-ulp spread, whichever is larger.
* 256x256 quads, N = 7 Helmholtz (4,194,304 local nodes, seed 3): MatrixAction and Residual <= 1e-12; the first
  20 PCG-Jacobi residuals <= 1e-9 relative; the converged FP64 and FP32-refined solutions <= 1e-8 of max |u| against
  the oracle's converged solve (minutes on a host, so kept as a fixture of 8192 sampled nodes made by
  tests/golden/make_helmholtz256_fixture.py), iteration count within 2 %.
Properties:
* shallow water: total mass sum(w_i w_j J H) is conserved by the LLF flux with mirror walls, in the FP64 drop-in
  (to 1e-13 relative over 100 steps) and in the FP32 perturbation form (to the FP32 rounding of eta, 1e-9 of the
  total); from a lake at rest both forms drift the same way (the discrete h^2/2 derivative is not exactly h times
  the discrete dh/dx, and the FP32 form carries that FP64 lake-at-rest tendency): after 20 steps the FP32 heights
  equal the FP64 ones to 1e-9 of max H and the velocities to 1e-3 of the FP64 drift.
* Helmholtz: the operator is symmetric, <A u, v> = <u, A v> to 1e-12 relative, and the FP32-refined and FP64 PCG
  solutions agree to 1e-8.
"""
import os

import numpy as np
import pytest

from helpers import per_var_rel, rel_inf

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))


def _sw_oracle(oracle):
    """The 128x128 N=7 shallow-water workload built by the oracle's set-up routines."""
    from self_gb300 import workloads as W
    oracle.set_threads(os.cpu_count())
    N, nx = 7, 128
    nod = oracle.Nodal(N, oracle.GAUSS, oracle.DG)
    mesh = oracle.Mesh(nx, nx, N, oracle.GAUSS, warp=W.SW_WARP, scale=(W.SW_L, W.SW_L))
    q, h, fcor, dt = W.shallow_water(mesh, N, nx, seed=2)
    dhdx, dhdy = oracle.DGProblem(nod, mesh, 1, 3, dt, h=h).bathymetry_gradient()
    P = oracle.DGProblem(nod, mesh, 1, 3, dt, h=h, dhdx=dhdx, dhdy=dhdy, fcor=fcor)
    return nod, mesh, q, h, fcor, dhdx, dhdy, dt, P


def _ulp_spread(fn, q, nvar, n2, seeds=(0, 1)):
    """The oracle's own spread on this input: max change per variable of fn(q) when every input value moves by at
    most one ulp (seeded signs).  At the configured state (zero velocity, a 1 m free surface on 1000 m of water) the
    conservative form cancels gH^2/2 fluxes of ~5e6 against the bathymetry source to leave tendencies of ~0.1, and
    the height tendency is the LLF dissipation of trace jumps that are themselves rounding (~2e-12): there a 1-ulp
    input change moves the oracle's momentum tendency by ~4e-10 and its height tendency by ~20 % relative, so no
    FP64 evaluation in another order can be closer than that."""
    base = fn(q).reshape(-1, nvar, n2)
    spread = np.zeros(nvar)
    for seed in seeds:
        rng = np.random.default_rng(seed)
        qp = q * (1.0 + 2.0 ** -52 * rng.choice([-1.0, 0.0, 1.0], q.size))
        d = np.abs(fn(qp).reshape(-1, nvar, n2) - base)
        spread = np.maximum(spread, [d[:, v].max() for v in range(nvar)])
    return base, spread


def _within(got, base, spread, nvar, n2, tol):
    """per variable: |gpu - oracle|_inf <= max(tol |oracle|_inf, 4 x the oracle's one-ulp spread)"""
    got = got.reshape(-1, nvar, n2)
    out = []
    for v in range(nvar):
        err = np.abs(got[:, v] - base[:, v]).max()
        bound = max(tol * np.abs(base[:, v]).max(), 4.0 * spread[v])
        out.append((err, bound))
    return out


def test_fullsize_sw_tendency_parity(oracle, gpu_ctx):
    """The configured state (ill-conditioned, bar = the oracle's own one-ulp spread) and the same state with a
    seeded 50 m/s velocity field (well-conditioned, bar 1e-12 per variable)."""
    import self_gb300 as sg
    nod, mesh, q, h, fcor, dhdx, dhdy, dt, P = _sw_oracle(oracle)
    n2 = nod.n * nod.n
    flow = q.reshape(mesh.nEl, 3, n2).copy()
    rng = np.random.default_rng(21)
    flow[:, 0] = rng.normal(0, 50.0, (mesh.nEl, n2))
    flow[:, 1] = rng.normal(0, 50.0, (mesh.nEl, n2))
    flow = flow.ravel()
    sw = sg.ShallowWater(gpu_ctx, nod, mesh, h, fcor, dt, dhdx=dhdx, dhdy=dhdy)
    sw.SetSolution(q)
    got = sw.GlobalTimeDerivative(0.0)
    base, spread = _ulp_spread(P.tendency, q, 3, n2)
    res = _within(got, base, spread, 3, n2, 1e-12)
    assert all(e <= b for e, b in res), res
    sw.SetSolution(flow)
    errs = per_var_rel(sw.GlobalTimeDerivative(0.0), P.tendency(flow), 3, n2)
    assert max(errs) <= 1e-12, errs
    sw.Trash()


def test_fullsize_sw_rk3_100_steps_parity(oracle, gpu_ctx):
    """100 LSRK3 steps from the configured state: <= 1e-11 per variable, or 4 x the oracle's own spread under a
    one-ulp change of the initial state where that is larger (the momentum grows from zero out of the
    ill-conditioned tendency above)."""
    import self_gb300 as sg
    nod, mesh, q, h, fcor, dhdx, dhdy, dt, P = _sw_oracle(oracle)
    n2 = nod.n * nod.n
    sw = sg.ShallowWater(gpu_ctx, nod, mesh, h, fcor, dt, dhdx=dhdx, dhdy=dhdy)
    sw.SetSolution(q)
    sw.ForwardStepRK3(0.0, 100)
    got = sw.GetSolution()
    sw.Trash()
    base, spread = _ulp_spread(lambda x: P.rk3(x, 100), q, 3, n2, seeds=(0,))
    res = _within(got, base, spread, 3, n2, 1e-11)
    assert all(e <= b for e, b in res), res


def _helmholtz256_oracle(oracle):
    from self_gb300 import workloads as W
    oracle.set_threads(os.cpu_count())
    N, nx = 7, 256
    nod = oracle.Nodal(N, oracle.GAUSS_LOBATTO, oracle.CG)
    mesh = oracle.Mesh(nx, nx, N, oracle.GAUSS_LOBATTO, boundary_flag=oracle.DIRICHLET)
    k, f, source = W.helmholtz(mesh, N, seed=3)
    return nod, mesh, k, source, oracle.CGProblem(nod, mesh, k, lam=0.1)


def test_fullsize_helmholtz_operator_and_pcg_parity(oracle, gpu_ctx):
    import self_gb300 as sg
    nod, mesh, k, source, P = _helmholtz256_oracle(oracle)
    cg = sg.CGsemElliptic_2D(gpu_ctx, nod, mesh, k, lam=0.1)
    rng = np.random.default_rng(31)
    u = rng.normal(size=cg.nl)
    assert rel_inf(cg.MatrixAction(u), P.matrix_action(u)) <= 1e-12
    sol = rng.normal(size=cg.nl)
    assert rel_inf(cg.Residual(source, sol), P.residual(source, sol)) <= 1e-12
    _, rep = cg.Solve(source, method="pcg", tolerance=1e-30, maxIters=20, return_resi=True)
    _, _, _, oresi = P.solve_pcg(source, maxIters=20, tol=1e-30, precond=1)
    assert rel_inf(rep["resi"][:21], oresi[:21]) <= 1e-9
    cg.Trash()


def test_fullsize_helmholtz_converged_solutions_vs_oracle(oracle, gpu_ctx):
    import self_gb300 as sg
    fx = np.load(os.path.join(HERE, "golden", "helmholtz256_n7_pcg.npz"))
    idx, uref, umax, oit = fx["idx"], fx["u"], float(fx["umax"]), int(fx["iterations"])
    nod, mesh, k, source, P = _helmholtz256_oracle(oracle)
    cg = sg.CGsemElliptic_2D(gpu_ctx, nod, mesh, k, lam=0.1)
    s64, r64 = cg.Solve(source, method="pcg", tolerance=1e-10, maxIters=50000)
    assert r64["ioerr"] == 0 and abs(r64["iterations"] - oit) <= max(2, 0.02 * oit), (r64, oit)
    assert np.abs(s64[idx] - uref).max() <= 1e-8 * umax
    assert abs(np.abs(s64).max() - umax) <= 1e-8 * umax
    s32, r32 = cg.Solve(source, method="pcg", precision="fp32", tolerance=1e-10)
    assert r32["ioerr"] == 0
    assert np.abs(s32[idx] - uref).max() <= 1e-8 * umax
    cg.Trash()


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
