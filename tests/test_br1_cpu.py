"""Known answers of the restated BR1 advection-diffusion (AdvectionClass.f90 with kappa > 0; oracle only)."""
import numpy as np


def _periodic(oracle, N=7, nx=8, warp=0.0, kappa=1e-2, velocity=(0.0, 0.0), seed=None):
    import self_gb300 as sg
    nod = sg.NodalStorage_2D(N)
    mesh = sg.QuadMesh(nx, nx, N, periodic=(True, True), warp=warp)
    u = np.full(mesh.x.size, velocity[0])
    v = np.full(mesh.x.size, velocity[1])
    c = np.sin(2 * np.pi * mesh.x) * np.sin(2 * np.pi * mesh.y)
    if seed is not None:
        c = c + 0.1 * np.random.default_rng(seed).normal(size=c.size)
    dt = 0.02 * (1.0 / nx) ** 2 / (kappa * (N + 1) ** 4) if kappa > 0 else 1e-3
    P = oracle.DGProblem(nod, mesh, 2, 1, dt, u=u, v=v, kappa=kappa)
    return nod, mesh, c, u, v, dt, P


def test_pure_diffusion_is_kappa_laplacian(oracle):
    """u = v = 0, c = sin(2 pi x) sin(2 pi y) on the periodic unit square: the BR1 tendency is
    kappa * Laplacian(c) = -8 pi^2 kappa c to spectral accuracy."""
    nod, mesh, c, u, v, dt, P = _periodic(oracle)
    t = P.tendency(c)
    exact = -8 * np.pi ** 2 * 1e-2 * c
    assert np.abs(t - exact).max() <= 1e-5 * np.abs(exact).max()


def test_diffusion_conserves_the_mean_and_decays_the_variance(oracle):
    nod, mesh, c, u, v, dt, P = _periodic(oracle, N=5, nx=6, warp=0.03, velocity=(1.0, 0.5), seed=3)
    n = nod.n
    w2 = np.outer(nod.w, nod.w).ravel()
    J = mesh.J.reshape(mesh.nEl, n * n)
    t = P.tendency(c).reshape(mesh.nEl, n * n)
    mass = np.sum(w2 * J * c.reshape(mesh.nEl, n * n))
    assert abs(np.sum(w2 * J * t)) <= 1e-12 * max(1.0, abs(mass)) * 1e3
    q = P.rk3(c, 20)
    var = lambda z: np.sum(w2 * J * z.reshape(mesh.nEl, n * n) ** 2)  # noqa: E731
    assert var(q) < var(c)


def test_kappa_zero_matches_the_advection_path(oracle):
    """kappa = 0 through the BR1 code path equals the plain advection tendency."""
    import self_gb300 as sg
    nod, mesh, c, u, v, dt, P = _periodic(oracle, kappa=0.0, velocity=(1.0, 0.5), seed=1)
    Q = oracle.DGProblem(nod, mesh, 2, 1, dt, u=u, v=v, kappa=1e-30)
    assert np.abs(Q.tendency(c) - P.tendency(c)).max() <= 1e-20 * 1e10
