"""GPU CGSEM 2-D operator and solvers against the CPU oracle (restated CGsemElliptic_2D / IterativeSolvers).

Tolerances: MatrixAction / Residual / DotProduct 1e-12 relative (per array, infinity norm); solver residual
histories agree to 1e-9 relative over the first 20 iterations (rounding differences grow with the Krylov
recurrence); converged solutions agree to 1e-8 relative; iteration counts within 2%.
"""
import numpy as np
import pytest

from helpers import rel_inf

pytestmark = pytest.mark.gpu


def _problem(oracle, N, nx, warp=0.0, lam=0.1, op=0, vel=(0.0, 0.0), kappa=None):
    import self_gb300 as sg
    from self_gb300 import workloads as W
    nod = sg.NodalStorage_2D(N, sg._native.GAUSS_LOBATTO, sg._native.CG)
    mesh = sg.QuadMesh(nx, nx, N, sg._native.GAUSS_LOBATTO, warp=warp, boundary_flag=sg._native.DIRICHLET)
    k, f, source = W.helmholtz(mesh, N)
    if kappa is not None:
        k = np.full_like(k, kappa)
    P = oracle.CGProblem(nod, mesh, k, lam=lam, op=op, vel=vel)
    return nod, mesh, k, source, P


@pytest.mark.parametrize("N,nx,warp,op", [(3, 4, 0.0, 0), (7, 8, 0.05, 0), (5, 6, 0.03, 1), (9, 3, 0.0, 0),
                                          (6, 5, 0.03, 0), (8, 4, 0.02, 1)])
def test_matrix_action_residual_dot_parity(oracle, gpu_ctx, N, nx, warp, op):
    import self_gb300 as sg
    vel = (1.0, 0.5) if op == 1 else (0.0, 0.0)
    nod, mesh, k, source, P = _problem(oracle, N, nx, warp, op=op, vel=vel)
    cg = sg.CGsemElliptic_2D(gpu_ctx, nod, mesh, k, lam=0.1, op=op, vel=vel)
    rng = np.random.default_rng(5)
    u = rng.normal(size=cg.nl)
    assert rel_inf(cg.MatrixAction(u), P.matrix_action(u)) <= 1e-12
    sol = rng.normal(size=cg.nl)
    assert rel_inf(cg.Residual(source, sol), P.residual(source, sol)) <= 1e-12
    v = rng.normal(size=cg.nl)
    a, b = cg.DotProduct(u, v), P.dot(u, v)
    assert abs(a - b) <= 1e-12 * abs(b) * 10
    um = u.copy()
    P.mask(um)
    assert np.array_equal(cg.Mask(u), um)
    uu = um.copy()
    P.unmask(uu)
    assert np.array_equal(cg.UnMask(um), uu)


def test_jacobi_diagonal_matches_unit_vector_application(oracle):
    """The closed-form assembled diagonal equals the operator applied to unit vectors (small mesh, oracle)."""
    nod, mesh, k, source, P = _problem(oracle, 3, 3, warp=0.05)
    d = P.jacobi_diagonal()
    nl = P.nl
    e = np.zeros(nl)
    um = np.ones(nl)
    P.mask(um)
    for idx in range(nl):
        if um[idx] == 0:
            assert d[idx] == 1.0
            continue
        e[:] = 0
        e[idx] = 1.0
        P.unmask(e)
        Ae = P.matrix_action(e)
        assert abs(Ae[idx] - d[idx]) <= 1e-12 * abs(d[idx])


@pytest.mark.parametrize("method,precond,N,nx", [("cg", 0, 5, 6), ("pcg", 1, 5, 6), ("pcg", 1, 6, 5), ("pcg", 1, 7, 4),
                                                 ("pcg", 1, 8, 4)])
def test_pcg_parity_with_oracle(oracle, gpu_ctx, method, precond, N, nx):
    import self_gb300 as sg
    nod, mesh, k, source, P = _problem(oracle, N, nx, warp=0.03)
    cg = sg.CGsemElliptic_2D(gpu_ctx, nod, mesh, k, lam=0.1)
    sol, rep = cg.Solve(source, method=method, tolerance=1e-10, maxIters=3000, return_resi=True)
    osol, ioerr, oit, oresi = P.solve_pcg(source, maxIters=3000, tol=1e-10, precond=precond)
    assert rep["ioerr"] == 0 and ioerr == 0
    assert abs(rep["iterations"] - oit) <= max(2, 0.02 * oit)
    r = rep["resi"]
    assert rel_inf(r[:20], oresi[:20]) <= 1e-9
    assert rel_inf(sol, osol) <= 1e-8
    assert rep["rel_residual"] < 1e-10


def test_fp32_refinement_reaches_fp64_accuracy(oracle, gpu_ctx):
    import self_gb300 as sg
    N, nx = 7, 8
    nod, mesh, k, source, P = _problem(oracle, N, nx, warp=0.03)
    cg = sg.CGsemElliptic_2D(gpu_ctx, nod, mesh, k, lam=0.1)
    s64, r64 = cg.Solve(source, method="pcg", tolerance=1e-10)
    s32, r32 = cg.Solve(source, method="pcg", precision="fp32", tolerance=1e-10)
    assert r32["ioerr"] == 0 and r32["rel_residual"] < 1e-10 and r32["outer_iterations"] >= 2
    # true FP64 residual of the refined solution, recomputed by the oracle
    res = P.residual(source, s32)
    r0 = P.residual(source, np.zeros_like(s32))
    assert np.sqrt(P.dot(res, res)) / np.sqrt(P.dot(r0, r0)) < 1.5e-10
    assert rel_inf(s32, s64) < 1e-8


@pytest.mark.parametrize("N,nx", [(4, 6), (4, 5)])
def test_gmres_advection_diffusion_parity(oracle, gpu_ctx, N, nx):
    """GMRES(30) against the oracle's: 6x6 N=4 (900 local nodes) runs the on-chip Gram-Schmidt, 5x5 N=4 (625, not a
    multiple of 4) the streaming one."""
    import self_gb300 as sg
    nod, mesh, k, source, P = _problem(oracle, N, nx, lam=0.0, op=1, vel=(1.0, 0.5), kappa=1e-2)
    cg = sg.CGsemElliptic_2D(gpu_ctx, nod, mesh, k, lam=0.0, op=1, vel=(1.0, 0.5))
    sol, rep = cg.Solve(source, method="gmres", m=30, tolerance=1e-10, maxIters=2000, return_resi=True)
    osol, ioerr, oit, oresi = P.solve_gmres(source, m=30, maxIters=2000, tol=1e-10)
    assert rep["ioerr"] == 0 and ioerr == 0
    assert abs(rep["iterations"] - oit) <= max(2, 0.02 * oit)
    assert rel_inf(rep["resi"][:20], oresi[:20]) <= 1e-9
    assert rel_inf(sol, osol) <= 1e-8


def test_pgmres_jacobi_advection_diffusion_parity(oracle, gpu_ctx):
    """Solve_PCGMRES with the Jacobi preconditioner: same residual history (first 20 Arnoldi steps), iteration
    count and solution as the oracle."""
    import self_gb300 as sg
    N, nx = 4, 6
    nod, mesh, k, source, P = _problem(oracle, N, nx, warp=0.03, lam=0.0, op=1, vel=(1.0, 0.5), kappa=1e-2)
    cg = sg.CGsemElliptic_2D(gpu_ctx, nod, mesh, k, lam=0.0, op=1, vel=(1.0, 0.5))
    sol, rep = cg.Solve(source, method="pgmres", m=30, tolerance=1e-10, maxIters=2000, return_resi=True)
    osol, ioerr, oit, oresi = P.solve_pgmres(source, m=30, maxIters=2000, tol=1e-10)
    assert rep["ioerr"] == 0 and ioerr == 0
    assert abs(rep["iterations"] - oit) <= max(2, 0.02 * oit)
    assert rel_inf(rep["resi"][:20], oresi[:20]) <= 1e-9
    assert rel_inf(sol, osol) <= 1e-8


@pytest.mark.parametrize("method", ["gmres", "pgmres"])
def test_fp32_inner_gmres_reaches_fp64_accuracy(oracle, gpu_ctx, method):
    """FP32-inner GMRES(m) under FP64 refinement (one FP32 cycle per refinement step, Gram-Schmidt dots in FP64,
    Givens in FP64, FP64 residual at every restart): ||r||/||r0|| < 1e-10 recomputed by the oracle, solution
    within 1e-8 of the FP64 GMRES solution, Arnoldi steps within 10 % of FP64 (the refinement step is the
    restart)."""
    import self_gb300 as sg
    N, nx = 5, 8
    nod, mesh, k, source, P = _problem(oracle, N, nx, warp=0.03, lam=0.0, op=1, vel=(1.0, 0.5), kappa=1e-2)
    cg = sg.CGsemElliptic_2D(gpu_ctx, nod, mesh, k, lam=0.0, op=1, vel=(1.0, 0.5))
    s64, r64 = cg.Solve(source, method=method, m=30, tolerance=1e-10, maxIters=5000)
    s32, r32 = cg.Solve(source, method=method, precision="fp32", m=30, tolerance=1e-10, maxIters=5000,
                        return_resi=True)
    assert r64["ioerr"] == 0 and r32["ioerr"] == 0 and r32["rel_residual"] < 1e-10
    assert r32["outer_iterations"] >= 2
    assert abs(r32["iterations"] - r64["iterations"]) <= 0.1 * r64["iterations"] + 30
    res = P.residual(source, s32)
    r0 = P.residual(source, np.zeros_like(s32))
    assert np.sqrt(P.dot(res, res)) / np.sqrt(P.dot(r0, r0)) < 1.5e-10
    assert rel_inf(s32, s64) < 1e-8
    h = r32["resi"][: r32["outer_iterations"] + 1]
    assert np.all(h[1:] > 0) and h[-1] / h[0] < 1e-10  # FP64 residual per refinement step


def test_manufactured_solution_converges(gpu_ctx):
    """u = sin(pi x) sin(pi y), k = 1, lam = 0.1: spectral accuracy of the solved field."""
    import self_gb300 as sg
    errs = []
    for N in (3, 5, 7):
        nod = sg.NodalStorage_2D(N, sg._native.GAUSS_LOBATTO, sg._native.CG)
        mesh = sg.QuadMesh(4, 4, N, sg._native.GAUSS_LOBATTO, boundary_flag=sg._native.DIRICHLET)
        ue = np.sin(np.pi * mesh.x) * np.sin(np.pi * mesh.y)
        f = (2 * np.pi ** 2 + 0.1) * ue
        cg = sg.CGsemElliptic_2D(gpu_ctx, nod, mesh, np.ones_like(ue), lam=0.1)
        sol, rep = cg.Solve(-f, method="pcg", tolerance=1e-12)
        errs.append(np.abs(sol - ue).max())
    assert errs[2] < 1e-6 and errs[2] < errs[0] * 1e-3
