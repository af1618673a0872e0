"""The CPU oracle against the reference's own golden vectors and analytic known answers (no GPU)."""
import os

import numpy as np
import pytest

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _read_curve(path):
    rows = []
    for line in open(path):
        line = line.strip()
        if not line or line.startswith("#"):
            continue
        rows.append([float(t) for t in line.split()])
    return np.array(rows)


def test_elliptic1d_residual_history_matches_reference(oracle):
    """examples/elliptic1d/parabola/run/residual.curve: N=5, 10 elements, tol 1e-8, abstract CG."""
    ref = _read_curve(os.path.join(GOLD, "elliptic1d_residual.curve"))
    x, u, resi, iters, ioerr = oracle.elliptic1d(N=5, nEl=10, maxIters=1000, tol=1e-8, cg_quirk=1)
    assert iters == 81 and ioerr == 0
    nz = ref[:, 1] != 0
    # the curve holds 8 significant digits
    rel = np.abs(resi[: len(ref)][nz] - ref[nz, 1]) / np.abs(ref[nz, 1])
    assert rel.max() < 6e-8
    assert np.all(resi[82:] == 0.0)


def test_elliptic1d_solution_matches_reference_bitwise(oracle):
    ref = _read_curve(os.path.join(GOLD, "elliptic1d_solution.curve"))
    x, u, resi, iters, ioerr = oracle.elliptic1d()
    assert np.array_equal(ref[:, 0], x)
    assert np.array_equal(ref[:, 1], u)


def test_true_relative_residual_stops_earlier(oracle):
    # decision: the product stops on ||r||/||r0|| (the CGSEM PCG test), not sqrt(||r||)/||r0||
    _, _, resi, iters, ioerr = oracle.elliptic1d(cg_quirk=0)
    assert ioerr == 0 and iters < 81 and resi[iters] / resi[0] < 1e-8


@pytest.mark.parametrize("quad", [1, -1])
def test_derivative_matrix_spectral_convergence(oracle, quad):
    """testing/interp/Lagrange1D_Convergence: derivative of exp(-s^2) converges spectrally."""
    errs = []
    for N in range(2, 18):
        x, w = oracle.quadrature(N, quad)
        D = oracle.derivative_matrix(N, x)
        f = np.exp(-x ** 2)
        errs.append(np.abs(D @ f - (-2 * x * f)).max())
    # geometric (spectral) decay: eight orders of magnitude from degree 2 to degree 17
    assert errs[-1] < 1e-8 and errs[-1] < errs[0] * 1e-7
    assert all(errs[k + 2] < errs[k] for k in range(len(errs) - 2))


def test_quadrature_exactness(oracle):
    for N in range(1, 12):
        x, w = oracle.quadrature(N, 1)  # Gauss: exact to degree 2N+1
        assert abs(np.sum(w * x ** (2 * N)) - 2.0 / (2 * N + 1)) < 1e-13
        x, w = oracle.quadrature(N, -1)  # Gauss-Lobatto: exact to degree 2N-1
        if N >= 1:
            assert abs(np.sum(w * x ** (2 * N - 2)) - 2.0 / (2 * N - 1)) < 1e-13


def test_dg_matrix_quirk_is_the_transpose(oracle):
    ok = oracle.Nodal(7, oracle.GAUSS, oracle.DG, 0)
    qk = oracle.Nodal(7, oracle.GAUSS, oracle.DG, 1)
    n = 8
    S = ok.dmatS.reshape(n, n, order="F")
    P = qk.dmatP.reshape(n, n, order="F")
    assert np.array_equal(ok.dmatS, ok.dmatP)
    assert np.allclose(P, S.T, rtol=0, atol=0)
    # the corrected matrix differentiates: -D^T weak form reproduces -f' for f = x^3 up to the lift
    assert not np.allclose(P, S)


def test_advection_translation_known_answer(oracle):
    from self_gb300 import workloads as W
    N, nx = 5, 8
    nod = oracle.Nodal(N, oracle.GAUSS, oracle.DG)
    m = oracle.Mesh(nx, nx, N, oracle.GAUSS, periodic=(True, True))
    c0, u, v, dt = W.advection_periodic(m, N, nx)
    P = oracle.DGProblem(nod, m, 2, 1, dt, u=u, v=v)
    steps = 100
    q = P.rk3(c0, steps)
    ex = W.advection_exact(m.x, m.y, steps * dt)
    assert np.abs(q - ex).max() < 2e-4


def test_lake_at_rest_flat_bottom_is_steady(oracle):
    # straight-sided elements satisfy the discrete metric identities exactly, so a flat lake stays at rest
    N = 5
    nod = oracle.Nodal(N, oracle.GAUSS, oracle.DG)
    m = oracle.Mesh(4, 4, N, oracle.GAUSS, warp=0.0, scale=(2e6, 2e6))
    n2 = (N + 1) ** 2
    h = np.full(m.nEl * n2, 1000.0)
    z = np.zeros_like(h)
    P = oracle.DGProblem(nod, m, 1, 3, 1.0, h=h, dhdx=z, dhdy=z, fcor=1e-4 + z)
    q = np.zeros((m.nEl, 3, n2))
    q[:, 2, :] = 1000.0
    td = P.tendency(q.ravel()).reshape(m.nEl, 3, n2)
    scale = 9.81 * 1000.0 ** 2 / (2e6 / 4)  # g H^2 / dx
    assert np.abs(td[:, :2]).max() < 1e-9 * scale
    assert np.abs(td[:, 2]).max() == 0.0


def test_oracle_pgmres_solves_what_gmres_solves(oracle):
    """The restated Solve_PCGMRES (Jacobi) reaches the same solution as the restated GMRES on a small
    advection-diffusion problem (both to 1e-10)."""
    import numpy as np
    import self_gb300 as sg
    N, nx = 3, 4
    nod = sg.NodalStorage_2D(N, sg._native.GAUSS_LOBATTO, sg._native.CG)
    mesh = sg.QuadMesh(nx, nx, N, sg._native.GAUSS_LOBATTO, warp=0.03, boundary_flag=sg._native.DIRICHLET)
    from self_gb300 import workloads as W
    _, f, source = W.helmholtz(mesh, N)
    P = oracle.CGProblem(nod, mesh, np.full(mesh.x.shape, 1e-2), lam=0.0, op=1, vel=(1.0, 0.5))
    s1, e1, it1, _ = P.solve_gmres(source, m=20, maxIters=500, tol=1e-10)
    s2, e2, it2, _ = P.solve_pgmres(source, m=20, maxIters=500, tol=1e-10)
    assert e1 == 0 and e2 == 0
    assert np.abs(s1 - s2).max() <= 1e-7 * np.abs(s1).max()
