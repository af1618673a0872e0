"""GPU linear-FEM preconditioner (SELF_SOLVE_PCG_LINEAR, self_cg2d_precondition) against the CPU oracle.

The reference's own CGsemElliptic_2D %Solve: PCG whose preconditioner is an inner CG on the N = 1 mesh of the GLL
nodes (CGsemPreconditioner_2D_Class.f90).  Tolerances: one preconditioner application 1e-11 relative (infinity
norm) with the same inner iteration count; solver residual histories 1e-8 relative over the first 10 iterations;
converged solutions 1e-9 relative; outer iteration counts within 1.
"""
import ctypes as C
import os

import numpy as np
import pytest

from helpers import connectivity_ids, rel_inf

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _problem(oracle, N, nx, warp, lam=0.1, flag=None, ism=None):
    import self_gb300 as sg
    from self_gb300 import workloads as W
    nat = sg._native
    nod = sg.NodalStorage_2D(N, nat.GAUSS_LOBATTO, nat.CG)
    if ism:
        mesh = sg.read_ism_mesh(os.path.join(ROOT, "tests", "golden", ism), N, nat.GAUSS_LOBATTO)
    else:
        mesh = sg.QuadMesh(nx, nx, N, nat.GAUSS_LOBATTO, warp=warp,
                           boundary_flag=nat.DIRICHLET if flag is None else flag)
    k, f, source = W.helmholtz(mesh, N)
    return nod, mesh, k, source, oracle.CGProblem(nod, mesh, k, lam=lam)


# (N, nx, warp, inner iterations, inner tolerance, boundary flag, ISM mesh file, node identification)
CASES = [(5, 8, 0.03, 20, 1e-4, None, None, "position"), (3, 4, 0.0, 50, 1e-4, None, None, "position"),
         (9, 3, 0.05, 10, 0.0, None, None, "position"), (2, 6, 0.0, 7, 1e-4, None, None, "position"),
         (4, 5, 0.02, 15, 1e-4, -100, None, "position"), (4, 0, 0.0, 12, 1e-4, None, "square.mesh", "position"),
         (4, 0, 0.0, 12, 1e-4, None, "square.mesh", "connectivity"),
         (3, 0, 0.0, 9, 1e-4, None, "box.mesh", "connectivity"), (6, 5, 0.02, 9, 1e-4, None, None, "connectivity")]


@pytest.mark.parametrize("N,nx,warp,its,tol,flag,ism,nodes", CASES)
def test_precondition_parity(oracle, gpu_ctx, N, nx, warp, its, tol, flag, ism, nodes):
    import self_gb300 as sg
    lam = 1.0 if flag is not None else 0.1
    nod, mesh, k, source, P = _problem(oracle, N, nx, warp, lam, flag, ism)
    cg = sg.CGsemElliptic_2D(gpu_ctx, nod, mesh, k, lam=lam)
    rng = np.random.default_rng(7)
    r = rng.normal(size=cg.nl)
    P.mask(r)
    P.unmask(r)
    ids = connectivity_ids(mesh, N) if nodes == "connectivity" else None
    w_ref, it_ref = P.pc_linear_apply(r, pcIters=its, pcTol=tol, ids=ids)
    w, it = cg.Precondition(r, pc_iterations=its, pc_tolerance=tol, pc_nodes=nodes)
    assert it == it_ref
    assert rel_inf(w, w_ref) <= 1e-11
    w0, it0 = cg.Precondition(r, pc_iterations=0)
    assert it0 == 0
    np.testing.assert_array_equal(w0, r)
    cg.Trash()


# the reference's preconditioner stalls the PCG where its linear mesh has Dirichlet nodes the problem does not: a
# Neumann boundary, or nodes of a SpecMesh file its position search leaves split ("stall": both stop at maxIters
# with ioerr -1 and the same residual history)
SOLVES = [(5, 8, 0.03, 20, None, None, "position", "converge"), (3, 6, 0.0, 50, None, None, "position", "converge"),
          (4, 5, 0.02, 15, -100, None, "position", "stall"), (4, 0, 0.0, 12, None, "square.mesh", "position", "stall"),
          (4, 0, 0.0, 12, None, "square.mesh", "connectivity", "converge"),
          (4, 0, 0.0, 12, None, "box.mesh", "position", "stall")]


@pytest.mark.parametrize("N,nx,warp,its,flag,ism,nodes,expect", SOLVES)
def test_solve_pcg_linear_parity(oracle, gpu_ctx, N, nx, warp, its, flag, ism, nodes, expect):
    import self_gb300 as sg
    lam = 1.0 if flag is not None else 0.1
    nod, mesh, k, source, P = _problem(oracle, N, nx, warp, lam, flag, ism)
    cg = sg.CGsemElliptic_2D(gpu_ctx, nod, mesh, k, lam=lam)
    ids = connectivity_ids(mesh, N) if nodes == "connectivity" else None
    max_iters = 40 if expect == "stall" else 600
    s_ref, e_ref, it_ref, r_ref = P.solve_pcg_linear(source, maxIters=max_iters, tol=1e-10, pcIters=its, pcTol=1e-4,
                                                     ids=ids)
    sol, rep = cg.Solve(source, method="pcg_linear", maxIters=max_iters, tolerance=1e-10, pc_iterations=its,
                        pc_tolerance=1e-4, pc_nodes=nodes, return_resi=True)
    if expect == "stall":
        assert e_ref == -1 and rep["ioerr"] == -1 and rep["iterations"] == it_ref == max_iters
        assert r_ref[-1] / r_ref[0] > 1e-3
        assert rel_inf(rep["resi"], r_ref) <= 1e-7
    else:
        assert e_ref == 0 and rep["ioerr"] == 0
        assert abs(rep["iterations"] - it_ref) <= 1
        m = min(10, it_ref)
        assert rel_inf(rep["resi"][: m + 1], r_ref[: m + 1]) <= 1e-8
        assert rel_inf(sol, s_ref) <= 1e-9
    cg.Trash()


def test_pcg_linear_fp32_refinement(oracle, gpu_ctx):
    """FP32 inner PCG with the FP32 linear-FEM preconditioner under FP64 refinement reaches the FP64 solution."""
    import self_gb300 as sg
    nod, mesh, k, source, P = _problem(oracle, 7, 12, 0.03)
    cg = sg.CGsemElliptic_2D(gpu_ctx, nod, mesh, k, lam=0.1)
    s64, r64 = cg.Solve(source, method="pcg_linear", tolerance=1e-10, pc_iterations=20)
    s32, r32 = cg.Solve(source, method="pcg_linear", precision="fp32", tolerance=1e-10, pc_iterations=20)
    assert r64["ioerr"] == 0 and r32["ioerr"] == 0 and r32["rel_residual"] < 1e-10
    assert rel_inf(s32, s64) <= 1e-8
    sj, rj = cg.Solve(source, method="pcg", tolerance=1e-10)
    assert rel_inf(sj, s64) <= 1e-8
    assert r64["iterations"] < rj["iterations"] / 4
    cg.Trash()


def test_zero_preconditioner_iterations_is_plain_cg(oracle, gpu_ctx):
    import self_gb300 as sg
    nod, mesh, k, source, P = _problem(oracle, 4, 6, 0.0)
    cg = sg.CGsemElliptic_2D(gpu_ctx, nod, mesh, k, lam=0.1)
    s1, r1 = cg.Solve(source, method="pcg_linear", tolerance=1e-10, pc_iterations=0)
    s2, r2 = cg.Solve(source, method="cg", tolerance=1e-10)
    assert r1["iterations"] == r2["iterations"]
    np.testing.assert_array_equal(s1, s2)
    cg.Trash()


def test_pcg_linear_needs_positions(gpu_ctx):
    """A descriptor without x, y cannot build the preconditioner mesh: the solve fails with an error, no fallback."""
    import self_gb300 as sg
    from self_gb300 import workloads as W
    from self_gb300.cgsem import CG2DDesc
    nat = sg._native
    N, nx = 3, 4
    nod = sg.NodalStorage_2D(N, nat.GAUSS_LOBATTO, nat.CG)
    mesh = sg.QuadMesh(nx, nx, N, nat.GAUSS_LOBATTO, boundary_flag=nat.DIRICHLET)
    k, f, source = W.helmholtz(mesh, N)
    d = CG2DDesc()
    d.N, d.nEl, d.nEdges, d.nNodes = N, mesh.nEl, mesh.nEdges, mesh.nNodes
    d.dmat, d.qweight = nat.d(nod.dmatS), nat.d(nod.w)
    d.edges, d.nodeType = nat.i(mesh.edges), nat.i(mesh.nodeType)
    d.n2e_ptr, d.n2e_elem, d.n2e_local = nat.i(mesh.n2e_ptr), nat.i(mesh.n2e_elem), nat.i(mesh.n2e_local)
    d.dxds, d.dxdp, d.dyds, d.dydp, d.J = (nat.d(getattr(mesh, q)) for q in ("dxds", "dxdp", "dyds", "dydp", "J"))
    d.fluxCoeff, d.lam = nat.d(k), 0.1
    p = C.c_void_p()
    nat.check(nat.lib().self_cg2d_create(gpu_ctx.ptr, C.byref(d), C.byref(p)), gpu_ctx.ptr)
    cg = sg.CGsemElliptic_2D.__new__(sg.CGsemElliptic_2D)
    cg.ptr, cg.ctx, cg.nl = p, gpu_ctx, (N + 1) ** 2 * mesh.nEl
    with pytest.raises(nat.SelfError):
        cg.Solve(source, method="pcg_linear", pc_iterations=5)
    sol, rep = cg.Solve(source, method="pcg", tolerance=1e-10)  # the handle still works for the other methods
    assert rep["ioerr"] == 0
    cg.Trash()
