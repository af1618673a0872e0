"""GPU DGSEM 2-D (plain FP64 drop-in) against the CPU oracle on identical seeded inputs.

Tolerance: per-variable relative error ||gpu - oracle||_inf / ||oracle||_inf <= 1e-12 for one tendency
evaluation, <= 1e-11 for RK3 trajectories (10 to 1000 steps): FMA contraction and the 1/J, 1/H
multiplications on the GPU round differently from the Fortran-order oracle, and the difference grows
with the number of stages.
"""
import numpy as np
import pytest

from helpers import per_var_rel, rel_inf

pytestmark = pytest.mark.gpu

TOL1 = 1e-12
TOLLONG = 1e-11


def _sw_problem(oracle, N, nx, warp=0.05, seed=7, drag=0.0, relax=False, flow=True):
    import self_gb300 as sg
    from self_gb300 import workloads as W
    nod = sg.NodalStorage_2D(N)
    mesh = sg.QuadMesh(nx, nx, N, warp=warp, scale=(W.SW_L, W.SW_L))
    q, h, fcor, dt = W.shallow_water(mesh, N, nx, seed=seed)
    n2 = (N + 1) ** 2
    if flow:  # give the state a velocity so every flux and source term is exercised
        rng = np.random.default_rng(seed + 100)
        qq = q.reshape(mesh.nEl, 3, n2)
        qq[:, 0] = rng.normal(0, 50.0, (mesh.nEl, n2))
        qq[:, 1] = rng.normal(0, 50.0, (mesh.nEl, n2))
        q = qq.ravel()
    dhdx, dhdy = sg.bathymetry_gradient(nod, mesh, h)
    rl = ts = None
    if relax:
        rng = np.random.default_rng(seed + 200)
        rl = (q + rng.normal(0, 1.0, q.size)).copy()
        ts = np.full(h.size, 1e-4)
    P = oracle.DGProblem(nod, mesh, 1, 3, dt, g=9.81, drag=drag, h=h, dhdx=dhdx, dhdy=dhdy, fcor=fcor, relax=rl,
                         rfac=ts)
    return nod, mesh, q, h, fcor, dhdx, dhdy, dt, P, rl, ts


@pytest.mark.parametrize("N,nx,warp,drag,relax", [(3, 4, 0.05, 0.0, False), (7, 16, 0.05, 0.0, False),
                                                  (5, 6, 0.0, 1e-3, True), (9, 3, 0.05, 0.0, False),
                                                  (6, 5, 0.05, 0.0, False), (8, 4, 0.05, 1e-3, True)])
def test_sw_tendency_parity(oracle, gpu_ctx, N, nx, warp, drag, relax):
    import self_gb300 as sg
    nod, mesh, q, h, fcor, dhdx, dhdy, dt, P, rl, ts = _sw_problem(oracle, N, nx, warp, drag=drag, relax=relax)
    sw = sg.ShallowWater(gpu_ctx, nod, mesh, h, fcor, dt, linear_drag=drag, dhdx=dhdx, dhdy=dhdy, relax=rl,
                         timescale=ts)
    sw.SetSolution(q)
    got = sw.GlobalTimeDerivative(0.0)
    ref = P.tendency(q)
    errs = per_var_rel(got, ref, 3, (N + 1) ** 2)
    assert max(errs) <= TOL1, errs
    assert np.array_equal(sw.GetSolution(), q)


def test_sw_rk3_parity_10_steps(oracle, gpu_ctx):
    import self_gb300 as sg
    N, nx = 7, 8
    nod, mesh, q, h, fcor, dhdx, dhdy, dt, P, _, _ = _sw_problem(oracle, N, nx)
    sw = sg.ShallowWater(gpu_ctx, nod, mesh, h, fcor, dt, dhdx=dhdx, dhdy=dhdy)
    sw.SetSolution(q)
    sw.ForwardStepRK3(0.0, 10)
    got = sw.GetSolution()
    ref = P.rk3(q, 10)
    errs = per_var_rel(got, ref, 3, (N + 1) ** 2)
    assert max(errs) <= TOLLONG, errs


def test_sw_lake_at_rest_flat_bottom(gpu_ctx):
    import self_gb300 as sg
    N, nx = 5, 4
    nod = sg.NodalStorage_2D(N)
    mesh = sg.QuadMesh(nx, nx, N, scale=(2e6, 2e6))
    h = np.full(mesh.x.size, 1000.0)
    sw = sg.ShallowWater(gpu_ctx, nod, mesh, h, np.full_like(h, 1e-4), 1.0)
    q = np.zeros((mesh.nEl, 3, (N + 1) ** 2))
    q[:, 2] = 1000.0
    sw.SetSolution(q.ravel())
    td = sw.GlobalTimeDerivative().reshape(mesh.nEl, 3, -1)
    assert np.abs(td[:, :2]).max() < 1e-9 * 9.81 * 1000.0 ** 2 / (2e6 / nx)
    assert np.abs(td[:, 2]).max() == 0.0


@pytest.mark.parametrize("nEq", [1, 3])
def test_advection_tendency_parity(oracle, gpu_ctx, nEq):
    import self_gb300 as sg
    from self_gb300 import workloads as W
    N, nx = 7, 6
    nod = sg.NodalStorage_2D(N)
    mesh = sg.QuadMesh(nx, nx, N, periodic=(True, True), warp=0.03)
    c0, u, v, dt = W.advection_periodic(mesh, N, nx)
    rng = np.random.default_rng(3)
    u = u + 0.2 * np.sin(2 * np.pi * mesh.y)
    q = np.concatenate([c0.reshape(mesh.nEl, 1, -1) * (k + 1) for k in range(nEq)], axis=1).ravel()
    rl = rng.normal(size=q.size)
    rf = np.abs(rng.normal(size=q.size))
    P = oracle.DGProblem(nod, mesh, 2, nEq, dt, u=u, v=v, relax=rl, rfac=rf)
    adv = sg.Advection(gpu_ctx, nod, mesh, u, v, dt, nTracers=nEq, relax=rl, rfac=rf)
    adv.SetSolution(q)
    got = adv.GlobalTimeDerivative(0.0)
    errs = per_var_rel(got, P.tendency(q), nEq, (N + 1) ** 2)
    assert max(errs) <= TOL1, errs


def test_advection_inflow_boundaries(oracle, gpu_ctx):
    """Non-periodic mesh with InflowOne edges: tanh(t) external state (AdvectionClass.f90:1851-1886)."""
    import self_gb300 as sg
    from self_gb300 import workloads as W
    N, nx = 4, 5
    nod = sg.NodalStorage_2D(N)
    mesh = sg.QuadMesh(nx, nx, N, boundary_flag=sg._native.INFLOW_ONE)
    c0, u, v, dt = W.advection_periodic(mesh, N, nx)
    P = oracle.DGProblem(nod, mesh, 2, 1, dt, u=u, v=v)
    adv = sg.Advection(gpu_ctx, nod, mesh, u, v, dt)
    adv.SetSolution(c0)
    assert max(per_var_rel(adv.GlobalTimeDerivative(0.7), P.tendency(c0, 0.7), 1, (N + 1) ** 2)) <= TOL1
    adv.ForwardStepRK3(0.3, 5)
    ref = P.rk3(c0, 5, tn=0.3)
    assert rel_inf(adv.GetSolution(), ref) <= TOLLONG


def test_advection_config1_1000_steps(oracle, gpu_ctx):
    """16x16 periodic, N=7, velocity (1, 0.5), Gaussian, CFL 0.5, 1000 LSRK3 steps: oracle and analytic."""
    import self_gb300 as sg
    from self_gb300 import workloads as W
    N, nx, steps = 7, 16, 1000
    nod = sg.NodalStorage_2D(N)
    mesh = sg.QuadMesh(nx, nx, N, periodic=(True, True))
    c0, u, v, dt = W.advection_periodic(mesh, N, nx)
    adv = sg.Advection(gpu_ctx, nod, mesh, u, v, dt)
    adv.SetSolution(c0)
    adv.ForwardStepRK3(0.0, steps)
    got = adv.GetSolution()
    ref = oracle.DGProblem(nod, mesh, 2, 1, dt, u=u, v=v).rk3(c0, steps)
    assert rel_inf(got, ref) <= TOLLONG
    ex = W.advection_exact(mesh.x, mesh.y, steps * dt)
    assert np.abs(got - ex).max() < 1e-4


# ---------------------------------------------------------------------------------------------- FP32 form
def test_fp32_sw_tendency_close_to_fp64(oracle, gpu_ctx):
    """FP32 perturbation form: one tendency within 1e-4 relative (per variable) of the FP64 oracle."""
    import self_gb300 as sg
    N, nx = 7, 8
    nod, mesh, q, h, fcor, dhdx, dhdy, dt, P, _, _ = _sw_problem(oracle, N, nx, flow=False)
    rng = np.random.default_rng(11)
    qq = q.reshape(mesh.nEl, 3, -1)
    qq[:, 0] = 20.0 * np.sin(2 * np.pi * mesh.y / 2e6).reshape(mesh.nEl, -1)
    qq[:, 1] = 10.0 * np.cos(2 * np.pi * mesh.x / 2e6).reshape(mesh.nEl, -1)
    q = qq.ravel()
    sw = sg.ShallowWater(gpu_ctx, nod, mesh, h, fcor, dt, dhdx=dhdx, dhdy=dhdy, precision=sg._native.PREC_FP32)
    sw.SetSolution(q)
    back = sw.GetSolution().reshape(mesh.nEl, 3, -1)
    assert np.abs(back[:, 2] - qq[:, 2]).max() < 1e-6  # eta = H - h stored in FP32
    got = sw.GlobalTimeDerivative(0.0)
    errs = per_var_rel(got, P.tendency(q), 3, (N + 1) ** 2)
    assert max(errs) <= 1e-4, errs


def test_fp32_sw_height_error_after_1000_steps(gpu_ctx):
    """North-star accuracy of the FP32 step: shallow-water height error <= 1e-6 relative to FP64 after 1000
    steps on the 128x128, N=7 curvilinear workload."""
    import self_gb300 as sg
    from self_gb300 import workloads as W
    N, nx, steps = 7, 128, 1000
    nod = sg.NodalStorage_2D(N)
    mesh = sg.QuadMesh(nx, nx, N, warp=W.SW_WARP, scale=(W.SW_L, W.SW_L))
    q, h, fcor, dt = W.shallow_water(mesh, N, nx, seed=2)
    dhdx, dhdy = sg.bathymetry_gradient(nod, mesh, h)
    out = {}
    for prec in (sg._native.PREC_FP64, sg._native.PREC_FP32):
        sw = sg.ShallowWater(gpu_ctx, nod, mesh, h, fcor, dt, dhdx=dhdx, dhdy=dhdy, precision=prec)
        sw.SetSolution(q)
        sw.ForwardStepRK3(0.0, steps)
        out[prec] = sw.GetSolution().reshape(mesh.nEl, 3, -1)
        sw.Trash()
    H64, H32 = out[0][:, 2], out[1][:, 2]
    err = np.abs(H32 - H64).max() / np.abs(H64).max()
    assert err <= 1e-6, err
    eta_err = np.abs(H32 - H64).max() / np.abs(H64 - h.reshape(mesh.nEl, -1)).max()
    assert eta_err <= 1e-3, eta_err
    for v in (0, 1):
        assert rel_inf(out[1][:, v], out[0][:, v]) <= 1e-3


def test_fp32_advection_1000_steps(gpu_ctx):
    import self_gb300 as sg
    from self_gb300 import workloads as W
    N, nx, steps = 7, 16, 1000
    nod = sg.NodalStorage_2D(N)
    mesh = sg.QuadMesh(nx, nx, N, periodic=(True, True))
    c0, u, v, dt = W.advection_periodic(mesh, N, nx)
    res = []
    for prec in (0, 1):
        adv = sg.Advection(gpu_ctx, nod, mesh, u, v, dt, precision=prec)
        adv.SetSolution(c0)
        adv.ForwardStepRK3(0.0, steps)
        res.append(adv.GetSolution())
    assert rel_inf(res[1], res[0]) <= 1e-5



# ---------------------------------------------------------------------------------------------- exact FP64 mode
@pytest.mark.parametrize("N,nx,warp,drag,relax", [(3, 4, 0.05, 0.0, False), (7, 16, 0.05, 0.0, False),
                                                  (5, 6, 0.0, 1e-3, True)])
def test_sw_exact_mode_is_bitwise_oracle(oracle, gpu_ctx, N, nx, warp, drag, relax):
    """SELF_PREC_FP64_EXACT (no FMA contraction, true divisions, the reference's statement order) reproduces the
    Fortran-order oracle bit for bit: tendency and a 10-step RK3 trajectory."""
    import self_gb300 as sg
    nod, mesh, q, h, fcor, dhdx, dhdy, dt, P, rl, ts = _sw_problem(oracle, N, nx, warp, drag=drag, relax=relax)
    sw = sg.ShallowWater(gpu_ctx, nod, mesh, h, fcor, dt, linear_drag=drag, dhdx=dhdx, dhdy=dhdy, relax=rl,
                         timescale=ts, precision=sg._native.PREC_FP64_EXACT)
    sw.SetSolution(q)
    assert np.array_equal(sw.GlobalTimeDerivative(0.0), P.tendency(q))
    sw.ForwardStepRK3(0.0, 10)
    assert np.array_equal(sw.GetSolution(), P.rk3(q, 10))


def test_advection_exact_mode_1000_steps_bitwise(oracle, gpu_ctx):
    import self_gb300 as sg
    from self_gb300 import workloads as W
    N, nx, steps = 7, 16, 1000
    nod = sg.NodalStorage_2D(N)
    mesh = sg.QuadMesh(nx, nx, N, periodic=(True, True))
    c0, u, v, dt = W.advection_periodic(mesh, N, nx)
    adv = sg.Advection(gpu_ctx, nod, mesh, u, v, dt, precision=sg._native.PREC_FP64_EXACT)
    adv.SetSolution(c0)
    adv.ForwardStepRK3(0.0, steps)
    assert np.array_equal(adv.GetSolution(), oracle.DGProblem(nod, mesh, 2, 1, dt, u=u, v=v).rk3(c0, steps))


def test_fp32_sw_rk3_close_to_oracle(oracle, gpu_ctx):
    """FP32 form through the fused TMA-staged stage kernel (N = 7): 20 RK3 steps within 1e-5 of the FP64 oracle
    per variable (heights relative to the perturbation eta)."""
    import self_gb300 as sg
    N, nx = 7, 8
    nod, mesh, q, h, fcor, dhdx, dhdy, dt, P, _, _ = _sw_problem(oracle, N, nx, flow=False)
    qq = q.reshape(mesh.nEl, 3, -1)
    qq[:, 0] = 20.0 * np.sin(2 * np.pi * mesh.y / 2e6).reshape(mesh.nEl, -1)
    qq[:, 1] = 10.0 * np.cos(2 * np.pi * mesh.x / 2e6).reshape(mesh.nEl, -1)
    q = qq.ravel()
    sw = sg.ShallowWater(gpu_ctx, nod, mesh, h, fcor, dt, dhdx=dhdx, dhdy=dhdy, precision=sg._native.PREC_FP32)
    sw.SetSolution(q)
    sw.ForwardStepRK3(0.0, 20)
    got = sw.GetSolution().reshape(mesh.nEl, 3, -1)
    ref = P.rk3(q, 20).reshape(mesh.nEl, 3, -1)
    hh = h.reshape(mesh.nEl, -1)
    assert rel_inf(got[:, 0], ref[:, 0]) < 1e-5 and rel_inf(got[:, 1], ref[:, 1]) < 1e-5
    assert rel_inf(got[:, 2] - hh, ref[:, 2] - hh) < 1e-5


def test_fp32_state_through_mapped_host_buffer_matches_staged_path(oracle, gpu_ctx):
    """A state in a self_host_alloc block is converted on the device straight from / into host memory; the
    result of set -> 5 steps -> get is bit-identical to the staged path with ordinary host arrays."""
    import ctypes as C
    import self_gb300 as sg
    nat = sg._native
    N, nx = 7, 6
    nod, mesh, q, h, fcor, dhdx, dhdy, dt, P, _, _ = _sw_problem(oracle, N, nx, flow=True)
    sw = sg.ShallowWater(gpu_ctx, nod, mesh, h, fcor, dt, dhdx=dhdx, dhdy=dhdy, precision=nat.PREC_FP32)
    sw.SetSolution(q)
    sw.ForwardStepRK3(0.0, 5)
    staged = sw.GetSolution()
    L = nat.lib()
    ptrs = []
    try:
        for _ in range(2):
            p = C.c_void_p()
            nat.check(L.self_host_alloc(C.c_size_t(q.size * 8), C.byref(p)))
            ptrs.append(p)
        hin = np.ctypeslib.as_array((C.c_double * q.size).from_address(ptrs[0].value))
        hout = np.ctypeslib.as_array((C.c_double * q.size).from_address(ptrs[1].value))
        hin[:] = q
        hout[:] = np.nan
        nat.check(L.self_dg2d_set_state(sw.ptr, C.cast(ptrs[0], nat.dp)), gpu_ctx.ptr)
        nat.check(L.self_dg2d_rk3(sw.ptr, C.c_double(0.0), 5), gpu_ctx.ptr)
        nat.check(L.self_dg2d_get_state(sw.ptr, C.cast(ptrs[1], nat.dp)), gpu_ctx.ptr)
        assert np.array_equal(hout, staged)
    finally:
        for p in ptrs:
            L.self_host_free(p)


def test_pickup_restart_continues_bit_identically(oracle, gpu_ctx, tmp_path):
    """10 RK3 steps in one go equal 5 steps, WritePickup, a fresh handle's ReadPickup and 5 more steps (FP64
    form): the pickup carries the state exactly."""
    import self_gb300 as sg
    N, nx = 5, 6
    nod, mesh, q, h, fcor, dhdx, dhdy, dt, P, _, _ = _sw_problem(oracle, N, nx, flow=True)
    a = sg.ShallowWater(gpu_ctx, nod, mesh, h, fcor, dt, dhdx=dhdx, dhdy=dhdy)
    a.SetSolution(q)
    a.ForwardStepRK3(0.0, 10)
    ref = a.GetSolution()
    b = sg.ShallowWater(gpu_ctx, nod, mesh, h, fcor, dt, dhdx=dhdx, dhdy=dhdy)
    b.SetSolution(q)
    b.ForwardStepRK3(0.0, 5)
    b.WritePickup(5, directory=str(tmp_path))
    c = sg.ShallowWater(gpu_ctx, nod, mesh, h, fcor, dt, dhdx=dhdx, dhdy=dhdy)
    q5, h5, f5 = c.ReadPickup(5, directory=str(tmp_path))
    assert np.array_equal(h5, np.ravel(h)) and np.array_equal(f5, np.ravel(fcor))
    c.ForwardStepRK3(0.0, 5)
    assert np.array_equal(c.GetSolution(), ref)
