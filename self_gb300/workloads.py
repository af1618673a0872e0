"""Seeded synthetic inputs with the shapes of the benchmark configurations.

The reference ships no datasets for these configurations; every input here is generated from a seed so
the GPU path and the CPU oracle see identical arrays.  Functions take any mesh object exposing the
MappedGeometry_2D node positions (x, y flat arrays in element order).

* advection_periodic: periodic [0,1]^2, velocity (1, 0.5), Gaussian exp(-r^2/(2*0.1^2)) at (0.5,0.5).
* shallow_water: [0, L]^2 with L = 2e6 m, beta-plane f = f0 + beta*y, depth 1000 m minus a 200 m Gaussian
  seamount (sigma 2e5 m) at the centre, free surface = 16 Gaussian bumps with amplitudes U(0.5, 1) m, centres
  uniform in the domain and widths U(5e4, 1.5e5) m, zero velocity.
Time steps: advection dt = CFL * dx / ((2N+1) (|u|+|v|)); shallow water dt = CFL * 2 / ((2N+1) max over nodes of
sqrt(g H) (|grad s| + |grad p|)), the contravariant gravity-wave speed of the mapped element (reduces to
CFL * dx / ((2N+1) 2 sqrt(g H)) on uniform squares, and shrinks where the warp compresses the mesh).
"""
import numpy as np

SW_L = 2.0e6
SW_F0, SW_BETA, SW_G = 1.0e-4, 2.0e-11, 9.81
SW_WARP = 0.05  # x + 0.05 L sin(2 pi x/L) sin(2 pi y/L) (applied to both coordinates)


def advection_periodic(mesh, N, nx, cfl=0.5, vel=(1.0, 0.5)):
    x, y = mesh.x, mesh.y
    c0 = np.exp(-((x - 0.5) ** 2 + (y - 0.5) ** 2) / (2 * 0.1 ** 2))
    u = np.full_like(x, vel[0])
    v = np.full_like(x, vel[1])
    dt = cfl * (1.0 / nx) / ((2 * N + 1) * (abs(vel[0]) + abs(vel[1])))
    return c0, u, v, dt


def advection_exact(x, y, t, vel=(1.0, 0.5)):
    """Periodic translate of the initial Gaussian (sum over the nearest images)."""
    X = np.mod(x - vel[0] * t, 1.0)
    Y = np.mod(y - vel[1] * t, 1.0)
    out = np.zeros_like(x)
    for sx in (-1, 0, 1):
        for sy in (-1, 0, 1):
            out += np.exp(-((X + sx - 0.5) ** 2 + (Y + sy - 0.5) ** 2) / (2 * 0.1 ** 2))
    return out


def shallow_water(mesh, N, nx, seed=2, cfl=0.5, L=SW_L, nbumps=16):
    rng = np.random.default_rng(seed)
    x, y = mesh.x, mesh.y
    h = 1000.0 - 200.0 * np.exp(-((x - L / 2) ** 2 + (y - L / 2) ** 2) / (2 * (2.0e5) ** 2))
    amp = rng.uniform(0.5, 1.0, nbumps)
    cx = rng.uniform(0.0, L, nbumps)
    cy = rng.uniform(0.0, L, nbumps)
    wid = rng.uniform(5.0e4, 1.5e5, nbumps)
    eta = np.zeros_like(x)
    for k in range(nbumps):
        eta += amp[k] * np.exp(-((x - cx[k]) ** 2 + (y - cy[k]) ** 2) / (2 * wid[k] ** 2))
    fcor = SW_F0 + SW_BETA * y
    nEl = x.size // ((N + 1) ** 2)
    n2 = (N + 1) ** 2
    q = np.zeros((nEl, 3, n2))
    q[:, 2, :] = (h + eta).reshape(nEl, n2)
    dt = sw_dt(mesh, N, h + eta, cfl)
    return q.ravel(), h, fcor, dt


def sw_dt(mesh, N, H, cfl=0.5, g=SW_G):
    """CFL time step from the contravariant gravity-wave speeds: |grad s| = |(dydp, -dxdp)| / |J|,
    |grad p| = |(-dyds, dxds)| / |J| on the reference element [-1, 1]^2."""
    J = np.abs(mesh.J)
    gs = np.hypot(mesh.dydp, mesh.dxdp) / J
    gp = np.hypot(mesh.dyds, mesh.dxds) / J
    lam = np.sqrt(g * H) * (gs + gp)
    return float(cfl * 2.0 / ((2 * N + 1) * lam.max()))


def sw_ensemble_member(mesh, N, nx, seed, cfl=0.5, L=SW_L):
    """Shallow-water ensemble member: same set-up, initial heights perturbed by the member's seed."""
    return shallow_water(mesh, N, nx, seed=seed, cfl=cfl, L=L)


def helmholtz(mesh, N, seed=3, nmodes=32, kmax=16):
    """Variable-coefficient Helmholtz on [0,1]^2: k = 1 + 0.5 sin(4 pi x) cos(4 pi y), f = seeded sum of 32
    Fourier modes (wavenumbers |k| <= 16 per direction, N(0,1) amplitudes, random sin/cos phase).  Returns
    (k, f, source) with source = -f: the operator -(K + lam M) of the reference's sign convention solves
    -div(k grad u) + lam u = f with load source*J*w*w."""
    rng = np.random.default_rng(seed)
    x, y = mesh.x, mesh.y
    k = 1.0 + 0.5 * np.sin(4 * np.pi * x) * np.cos(4 * np.pi * y)
    f = np.zeros_like(x)
    kx = rng.integers(-kmax, kmax + 1, nmodes)
    ky = rng.integers(-kmax, kmax + 1, nmodes)
    amp = rng.normal(0.0, 1.0, nmodes)
    ph = rng.uniform(0.0, 2 * np.pi, nmodes)
    for m in range(nmodes):
        f += amp[m] * np.cos(2 * np.pi * (kx[m] * x + ky[m] * y) + ph[m])
    return k, f, -f


def batched_specs(nprob=512, seed0=4, nmin=8, nmax=64, Nmin=3, Nmax=9):
    """Mesh size n (n x n quads) uniform in [nmin, nmax] and degree N uniform in {Nmin..Nmax}, seed seed0 + i."""
    specs = []
    for i in range(nprob):
        rng = np.random.default_rng(seed0 + i)
        specs.append((int(rng.integers(nmin, nmax + 1)), int(rng.integers(Nmin, Nmax + 1)), seed0 + i))
    return specs


def batched_problem(mod, nx, N, seed, lam=0.1):
    """One Helmholtz problem of the batched configuration: unit square, Dirichlet walls, its own coefficient
    field k = 1 + 0.5 sin(4 pi x + a) cos(4 pi y + b) (seeded phases) and seeded Fourier right-hand side."""
    nod = mod.NodalStorage_2D(N, -1, 2001)
    mesh = mod.QuadMesh(nx, nx, N, -1, boundary_flag=-200)
    rng = np.random.default_rng(seed + 100000)
    a, b = rng.uniform(0, 2 * np.pi, 2)
    k = 1.0 + 0.5 * np.sin(4 * np.pi * mesh.x + a) * np.cos(4 * np.pi * mesh.y + b)
    _, f, source = helmholtz(mesh, N, seed=seed)
    return {"nodal": nod, "mesh": mesh, "k": k, "source": source, "lam": lam}
