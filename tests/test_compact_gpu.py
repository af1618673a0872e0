"""FP32 inner PCG on the compact node layout against the element-local layout (GPU).

Both layouts run the same FP32 element operator and the same direct-stiffness sums: the assembled operator output is
bit-identical (MatrixAction32, compact vs local) where both use the line kernel, and agrees to FP32 rounding (1e-6)
for the warp-per-element kernel of N = 7.  In the solves only the order of the grid-wide dot-product sums
differs.  Bars: both converge to 1e-10, solutions within 1e-8 relative, inner iteration totals within 2 % (+2) for
Jacobi PCG on Dirichlet problems (10 % for plain CG, 15 % on the Neumann problem: there the FP32 iteration count
moves with the rounding of the dot sums); the compact solve issues two kernels per inner iteration (the element-local one three), which shows the
compact path ran.
"""
import numpy as np
import pytest

from helpers import rel_inf

pytestmark = pytest.mark.gpu


def _solve_both(gpu_ctx, N, nx, warp=0.0, periodic=(False, False), bflag=None, method="pcg", lam=0.1, its=0.02):
    import self_gb300 as sg
    from self_gb300 import workloads as W
    nod = sg.NodalStorage_2D(N, sg._native.GAUSS_LOBATTO, sg._native.CG)
    mesh = sg.QuadMesh(nx, nx, N, sg._native.GAUSS_LOBATTO, warp=warp, periodic=periodic,
                       boundary_flag=sg._native.DIRICHLET if bflag is None else bflag)
    k, f, source = W.helmholtz(mesh, N)
    cg = sg.CGsemElliptic_2D(gpu_ctx, nod, mesh, k, lam=lam)
    rng = np.random.default_rng(N + nx)
    u = cg.Mask(rng.normal(size=cg.nl))
    a_loc, a_cpt = cg.MatrixAction32(u, form="local"), cg.MatrixAction32(u, form="compact")
    if N == 7:  # warp-per-element kernel: same sums, its own FMA contraction of the flux and mass terms
        assert rel_inf(a_cpt, a_loc) <= 1e-6
    else:  # line kernel shared with the element-local form: bit-identical
        assert np.array_equal(a_cpt, a_loc), rel_inf(a_cpt, a_loc)
    out = {"its": its}
    for layout in ("local", "compact"):
        l0 = gpu_ctx.kernel_launches()
        sol, rep = cg.Solve(source, method=method, precision="fp32", tolerance=1e-10, inner_layout=layout)
        out[layout] = (sol, rep, gpu_ctx.kernel_launches() - l0)
    return out


def _check(out):
    (sl, rl, ll), (sc, rc, lc) = out["local"], out["compact"]
    for rep in (rl, rc):
        assert rep["ioerr"] == 0 and rep["rel_residual"] < 1e-10, rep
    assert rel_inf(sc, sl) < 1e-8
    assert abs(rc["iterations"] - rl["iterations"]) <= out["its"] * rl["iterations"] + 2, (rl, rc)
    # kernels per inner iteration: 2 (compact) vs 3 (element-local), plus the per-refinement-step launches
    assert lc < ll and lc <= 2 * rc["iterations"] + 40 * rc["outer_iterations"] + 64, (ll, lc, rl, rc)


@pytest.mark.parametrize("N,nx,warp", [(7, 12, 0.05), (4, 9, 0.0), (3, 5, 0.03), (2, 6, 0.0), (9, 4, 0.02)])
def test_compact_matches_local_dirichlet_box(gpu_ctx, N, nx, warp):
    _check(_solve_both(gpu_ctx, N, nx, warp))


def test_compact_matches_local_periodic_x(gpu_ctx):
    """Periodic in x (edges and corners paired across the domain), Dirichlet in y."""
    _check(_solve_both(gpu_ctx, 5, 8, 0.0, periodic=(True, False)))


def test_compact_matches_local_no_dirichlet(gpu_ctx):
    """No Dirichlet nodes (boundary edges are one-sided unknowns, boundary corners have one or two copies);
    lambda > 0 keeps the Helmholtz operator definite."""
    import self_gb300 as sg
    _check(_solve_both(gpu_ctx, 6, 7, 0.02, bflag=sg._native.NO_NORMAL_FLOW, lam=1.0, its=0.15))


def test_compact_plain_cg(gpu_ctx):
    """Unpreconditioned: the FP32 iteration count moves with the rounding of the dot sums (10 % bar)."""
    _check(_solve_both(gpu_ctx, 7, 6, 0.03, method="cg", its=0.10))


@pytest.mark.parametrize("N,nx,warp", [(7, 12, 0.05), (5, 9, 0.03), (3, 6, 0.0)])
def test_compact_fp64_pcg_matches_local(gpu_ctx, N, nx, warp):
    """FP64 Jacobi PCG on the compact layout (CG on the correction from the residual of the initial guess; N >= 5:
    the even-odd FP64 operator; N = 3 runs the element-local form under the same option) against the element-local
    solve: residual histories within 1e-9 over the first 20 iterations, iterations within 2 % (+2), solutions within
    1e-10; the compact solve launches two kernels per iteration."""
    import self_gb300 as sg
    from self_gb300 import workloads as W
    nod = sg.NodalStorage_2D(N, sg._native.GAUSS_LOBATTO, sg._native.CG)
    mesh = sg.QuadMesh(nx, nx, N, sg._native.GAUSS_LOBATTO, warp=warp, boundary_flag=sg._native.DIRICHLET)
    k, f, source = W.helmholtz(mesh, N)
    cg = sg.CGsemElliptic_2D(gpu_ctx, nod, mesh, k, lam=0.1)
    x0 = np.random.default_rng(N).normal(size=cg.nl) * 1e-3  # a nonzero initial guess
    out = {}
    for layout in ("local", "compact"):
        l0 = gpu_ctx.kernel_launches()
        sol, rep = cg.Solve(source, solution=x0, method="pcg", tolerance=1e-10, return_resi=True,
                            inner_layout=layout)
        out[layout] = (sol, rep, gpu_ctx.kernel_launches() - l0)
    (sl, rl, ll), (sc, rc, lc) = out["local"], out["compact"]
    for rep in (rl, rc):
        assert rep["ioerr"] == 0 and rep["rel_residual"] < 1e-10, rep
    assert abs(rc["iterations"] - rl["iterations"]) <= 0.02 * rl["iterations"] + 2
    assert rel_inf(rc["resi"][:20], rl["resi"][:20]) <= 1e-9
    assert rel_inf(sc, sl) < 1e-10
    if N >= 5:
        assert lc < ll, (ll, lc)
