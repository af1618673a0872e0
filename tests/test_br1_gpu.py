"""GPU advection-diffusion with kappa > 0 (BR1 passes of AdvectionClass.f90) against the CPU oracle.

Tolerances as for plain advection: one tendency 1e-12, 20 RK3 steps 1e-11; the bit-faithful FP64 mode equals the
oracle bit for bit.
"""
import numpy as np
import pytest

from helpers import per_var_rel, rel_inf
from test_br1_cpu import _periodic

pytestmark = pytest.mark.gpu


def _inflow_problem(oracle, N, nx, nEq, kappa, seed=5):
    """Non-periodic box with inflow on the west (tracer 1) and south (tracer 2) sides, velocity (1, 0.5)."""
    import self_gb300 as sg
    nat = sg._native
    nod = sg.NodalStorage_2D(N)
    mesh = sg.QuadMesh(nx, nx, N, warp=0.03)
    E = mesh.edges.reshape(-1, 6)
    rng = np.random.default_rng(seed)
    for k in range(E.shape[0]):
        if E[k, 2] < 0:
            E[k, 2] = nat.INFLOW_ONE if E[k, 1] in (4, 1) and rng.uniform() < 0.7 else nat.INFLOW_TWO
    mesh.edges = E.ravel().copy()
    u = np.full(mesh.x.size, 1.0)
    v = np.full(mesh.x.size, 0.5)
    c = np.concatenate([rng.normal(size=(mesh.nEl, 1, nod.n ** 2)) for _ in range(nEq)], axis=1).ravel()
    dt = 0.02 * (1.0 / nx) ** 2 / (kappa * (N + 1) ** 4)
    P = oracle.DGProblem(nod, mesh, 2, nEq, dt, u=u, v=v, kappa=kappa)
    return nod, mesh, c, u, v, dt, P


@pytest.mark.parametrize("N,nx,warp,vel", [(7, 8, 0.0, (0.0, 0.0)), (5, 6, 0.03, (1.0, 0.5)), (3, 4, 0.05, (0.3, -1.0))])
def test_br1_periodic_parity(oracle, gpu_ctx, N, nx, warp, vel):
    import self_gb300 as sg
    nod, mesh, c, u, v, dt, P = _periodic(oracle, N, nx, warp, 1e-2, vel, seed=2)
    adv = sg.Advection(gpu_ctx, nod, mesh, u, v, dt, kappa=1e-2)
    adv.SetSolution(c)
    assert rel_inf(adv.GlobalTimeDerivative(0.0), P.tendency(c)) <= 1e-12
    adv.ForwardStepRK3(0.0, 20)
    assert rel_inf(adv.GetSolution(), P.rk3(c, 20)) <= 1e-11
    adv.Trash()


@pytest.mark.parametrize("N,nx,nEq", [(4, 5, 2), (6, 3, 1)])
def test_br1_inflow_parity(oracle, gpu_ctx, N, nx, nEq):
    import self_gb300 as sg
    nod, mesh, c, u, v, dt, P = _inflow_problem(oracle, N, nx, nEq, 5e-3)
    adv = sg.Advection(gpu_ctx, nod, mesh, u, v, dt, nTracers=nEq, kappa=5e-3)
    adv.SetSolution(c)
    errs = per_var_rel(adv.GlobalTimeDerivative(0.3), P.tendency(c, t=0.3), nEq, (N + 1) ** 2)
    assert max(errs) <= 1e-12, errs
    adv.ForwardStepRK3(0.0, 10)
    errs = per_var_rel(adv.GetSolution(), P.rk3(c, 10), nEq, (N + 1) ** 2)
    assert max(errs) <= 1e-11, errs
    adv.Trash()


def test_br1_exact_mode_is_bitwise_oracle(oracle, gpu_ctx):
    import self_gb300 as sg
    nod, mesh, c, u, v, dt, P = _periodic(oracle, 5, 6, 0.03, 1e-2, (1.0, 0.5), seed=4)
    adv = sg.Advection(gpu_ctx, nod, mesh, u, v, dt, kappa=1e-2, precision=sg._native.PREC_FP64_EXACT)
    adv.SetSolution(c)
    assert np.array_equal(adv.GlobalTimeDerivative(0.0), P.tendency(c))
    adv.ForwardStepRK3(0.0, 10)
    assert np.array_equal(adv.GetSolution(), P.rk3(c, 10))
    adv.Trash()


def test_br1_rejected_outside_fp64_advection(gpu_ctx):
    import self_gb300 as sg
    nod, mesh = sg.NodalStorage_2D(3), sg.QuadMesh(3, 3, 3, periodic=(True, True))
    u = np.ones(mesh.x.size)
    with pytest.raises(sg._native.SelfError):
        sg.Advection(gpu_ctx, nod, mesh, u, u, 1e-3, kappa=1e-2, precision=sg._native.PREC_FP32)
