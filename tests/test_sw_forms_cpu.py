"""Known answers of the restated alternate shallow-water forms (oracle only, no GPU).

ShallowWaterClass.f90 with ModelFormulation LINEAR (state u, v, eta about the resting depth h) and
SKEW_SYMMETRIC (u, v, eta and the relative vorticity zeta as a 4th variable).
"""
import numpy as np


def _linear_problem(oracle, N=5, nx=6, warp=0.05, drag=0.0, relax=False, seed=3):
    import self_gb300 as sg
    from self_gb300 import workloads as W
    nod = sg.NodalStorage_2D(N)
    mesh = sg.QuadMesh(nx, nx, N, warp=warp, scale=(W.SW_L, W.SW_L))
    q, h, fcor, dt = W.shallow_water(mesh, N, nx, seed=seed)
    n2 = (N + 1) ** 2
    qq = q.reshape(mesh.nEl, 3, n2).copy()
    eta = qq[:, 2] - h.reshape(mesh.nEl, n2)
    rng = np.random.default_rng(seed + 1)
    lin = np.stack([rng.normal(0, 0.05, eta.shape), rng.normal(0, 0.05, eta.shape), eta], axis=1).ravel()
    rl = ts = None
    if relax:
        rl = lin + rng.normal(0, 0.01, lin.size)
        ts = np.full(h.size, 1e-4)
    P = oracle.DGProblem(nod, mesh, 3, 3, dt, g=9.81, drag=drag, h=h, fcor=fcor, relax=rl, rfac=ts)
    return nod, mesh, lin, h, fcor, dt, P, rl, ts


def test_linear_lake_at_rest(oracle):
    """u = v = eta = 0 is a steady state of the linear form: the tendency is exactly zero."""
    _, mesh, lin, h, fcor, dt, P, _, _ = _linear_problem(oracle)
    assert np.abs(P.tendency(np.zeros_like(lin))).max() == 0.0


def test_linear_energy_does_not_grow(oracle):
    """With mirror walls, no drag and no forcing, the discrete energy 1/2 sum w J (h (u^2 + v^2) + g eta^2) of
    the linear form cannot grow: the central part of the flux conserves it, the jump penalty dissipates."""
    nod, mesh, lin, h, fcor, dt, P, _, _ = _linear_problem(oracle)
    n = nod.n
    w2 = np.outer(nod.w, nod.w).ravel()
    J = mesh.J.reshape(mesh.nEl, n * n)
    hh = h.reshape(mesh.nEl, n * n)

    def energy(q):
        qq = q.reshape(mesh.nEl, 3, n * n)
        return 0.5 * np.sum(w2 * J * (hh * (qq[:, 0] ** 2 + qq[:, 1] ** 2) + 9.81 * qq[:, 2] ** 2))

    e0 = energy(lin)
    q = P.rk3(lin, 40)
    assert np.isfinite(q).all()
    assert energy(q) <= e0 * (1 + 1e-12)


def test_linear_tendency_is_linear_in_the_state(oracle):
    _, _, lin, _, _, _, P, _, _ = _linear_problem(oracle, relax=False)
    rng = np.random.default_rng(9)
    other = rng.normal(0, 0.05, lin.size)
    a, b = P.tendency(lin), P.tendency(other)
    ab = P.tendency(2.0 * lin - 3.0 * other)
    assert np.abs(ab - (2.0 * a - 3.0 * b)).max() <= 1e-12 * np.abs(ab).max()


def _skew_problem(oracle, N=5, nx=6, warp=0.05, drag=0.0, relax=False, seed=3, zeta=True):
    nod, mesh, lin, h, fcor, dt, _, rl3, ts = _linear_problem(oracle, N, nx, warp, drag, relax, seed)
    n2 = (N + 1) ** 2
    rng = np.random.default_rng(seed + 7)
    z = rng.normal(0, 1e-5, (mesh.nEl, 1, n2)) if zeta else np.zeros((mesh.nEl, 1, n2))
    q = np.concatenate([lin.reshape(mesh.nEl, 3, n2), z], axis=1).ravel()
    rl = None
    if relax:
        rl = np.concatenate([rl3.reshape(mesh.nEl, 3, n2), np.zeros((mesh.nEl, 1, n2))], axis=1).ravel()
    P = oracle.DGProblem(nod, mesh, 4, 4, dt, g=9.81, drag=drag, h=h, fcor=fcor, relax=rl, rfac=ts)
    return nod, mesh, q, h, fcor, dt, P, rl, ts


def test_skew_lake_at_rest(oracle):
    """u = v = eta = zeta = 0 is steady in the skew-symmetric form."""
    _, _, q, _, _, _, P, _, _ = _skew_problem(oracle)
    assert np.abs(P.tendency(np.zeros_like(q))).max() == 0.0


def test_skew_uniform_absolute_vorticity_flux_is_divergence_free(oracle):
    """With u = v = 0 and any zeta the vorticity fluxes u (zeta + f) vanish: zeta does not change, and the
    momentum tendency is that of eta alone."""
    _, mesh, q, _, _, _, P, _, _ = _skew_problem(oracle)
    n2 = P.nq // (4 * mesh.nEl)
    qq = q.reshape(mesh.nEl, 4, n2).copy()
    qq[:, 0] = qq[:, 1] = 0.0
    t = P.tendency(qq.ravel()).reshape(mesh.nEl, 4, n2)
    assert np.abs(t[:, 3]).max() == 0.0


def test_skew_reduces_to_linear_for_small_amplitude(oracle):
    """From rest (u = v = zeta = 0) with a tiny eta the skew-symmetric tendency of (u, v, eta) approaches the
    linear one: the fluxes differ only through KE and eta (h + eta), and the wave-speed estimates through
    sqrt(g (h + eta)) - all quadratic in the amplitude.  (With velocity the two dissipate differently already at
    first order: the skew flux penalises the whole velocity jump, the linear one its normal part.)"""
    nod, mesh, q, h, fcor, dt, P, _, _ = _skew_problem(oracle, zeta=False)
    _, _, lin, _, _, _, PL, _, _ = _linear_problem(oracle)
    n2 = P.nq // (4 * mesh.nEl)
    qs = q.reshape(mesh.nEl, 4, n2).copy()
    qs[:, :2] = 0.0
    ql = lin.reshape(mesh.nEl, 3, n2).copy()
    ql[:, :2] = 0.0
    d = []
    for amp in (1e-2, 1e-3):
        ts_ = P.tendency(amp * qs.ravel()).reshape(mesh.nEl, 4, n2)[:, :3].ravel()
        tl_ = PL.tendency(amp * ql.ravel())
        d.append(np.abs(ts_ - tl_).max() / np.abs(tl_).max())
    assert d[1] < d[0] / 5
