"""GPU alternate shallow-water forms (ShallowWaterClass.f90) against the CPU oracle.

LINEAR formulation (SELF_MODEL_SW_LINEAR, state u, v, eta) and SKEW_SYMMETRIC (SELF_MODEL_SW_SKEW, state u, v,
eta, zeta).  Tolerances as for the conservative form: one tendency 1e-12 per variable, 20 RK3 steps 1e-11; the
bit-faithful FP64 mode equals the oracle bit for bit.
"""
import numpy as np
import pytest

from helpers import per_var_rel
from test_sw_forms_cpu import _linear_problem, _skew_problem

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("N,nx,warp,drag,relax", [(3, 4, 0.05, 0.0, False), (7, 12, 0.05, 0.0, False),
                                                  (5, 6, 0.0, 1e-5, True), (9, 3, 0.05, 1e-5, False)])
def test_linear_sw_parity(oracle, gpu_ctx, N, nx, warp, drag, relax):
    import self_gb300 as sg
    nod, mesh, lin, h, fcor, dt, P, rl, ts = _linear_problem(oracle, N, nx, warp, drag, relax)
    sw = sg.ShallowWater(gpu_ctx, nod, mesh, h, fcor, dt, linear_drag=drag, relax=rl, timescale=ts,
                         formulation="linear")
    sw.SetSolution(lin)
    errs = per_var_rel(sw.GlobalTimeDerivative(0.0), P.tendency(lin), 3, (N + 1) ** 2)
    assert max(errs) <= 1e-12, errs
    sw.ForwardStepRK3(0.0, 20)
    errs = per_var_rel(sw.GetSolution(), P.rk3(lin, 20), 3, (N + 1) ** 2)
    assert max(errs) <= 1e-11, errs
    sw.Trash()


@pytest.mark.parametrize("N,nx,warp,drag,relax", [(4, 5, 0.05, 0.0, False), (6, 4, 0.0, 1e-5, True)])
def test_linear_sw_exact_mode_is_bitwise_oracle(oracle, gpu_ctx, N, nx, warp, drag, relax):
    import self_gb300 as sg
    nod, mesh, lin, h, fcor, dt, P, rl, ts = _linear_problem(oracle, N, nx, warp, drag, relax)
    sw = sg.ShallowWater(gpu_ctx, nod, mesh, h, fcor, dt, linear_drag=drag, relax=rl, timescale=ts,
                         formulation="linear", precision=sg._native.PREC_FP64_EXACT)
    sw.SetSolution(lin)
    assert np.array_equal(sw.GlobalTimeDerivative(0.0), P.tendency(lin))
    sw.ForwardStepRK3(0.0, 10)
    assert np.array_equal(sw.GetSolution(), P.rk3(lin, 10))
    sw.Trash()


def test_linear_sw_lake_at_rest_on_gpu(oracle, gpu_ctx):
    import self_gb300 as sg
    nod, mesh, lin, h, fcor, dt, P, _, _ = _linear_problem(oracle)
    sw = sg.ShallowWater(gpu_ctx, nod, mesh, h, fcor, dt, formulation="linear")
    sw.SetSolution(np.zeros_like(lin))
    assert np.abs(sw.GlobalTimeDerivative(0.0)).max() == 0.0
    sw.Trash()


@pytest.mark.parametrize("N,nx,warp,drag,relax", [(3, 4, 0.05, 0.0, False), (7, 10, 0.05, 0.0, False),
                                                  (5, 6, 0.0, 1e-5, True), (9, 3, 0.05, 1e-5, False)])
def test_skew_sw_parity(oracle, gpu_ctx, N, nx, warp, drag, relax):
    import self_gb300 as sg
    nod, mesh, q, h, fcor, dt, P, rl, ts = _skew_problem(oracle, N, nx, warp, drag, relax)
    sw = sg.ShallowWater(gpu_ctx, nod, mesh, h, fcor, dt, linear_drag=drag, relax=rl, timescale=ts,
                         formulation="skew_symmetric")
    sw.SetSolution(q)
    errs = per_var_rel(sw.GlobalTimeDerivative(0.0), P.tendency(q), 4, (N + 1) ** 2)
    assert max(errs) <= 1e-12, errs
    sw.ForwardStepRK3(0.0, 20)
    errs = per_var_rel(sw.GetSolution(), P.rk3(q, 20), 4, (N + 1) ** 2)
    assert max(errs) <= 1e-11, errs
    sw.Trash()


@pytest.mark.parametrize("N,nx,warp,drag,relax", [(4, 5, 0.05, 0.0, False), (6, 4, 0.0, 1e-5, True)])
def test_skew_sw_exact_mode_is_bitwise_oracle(oracle, gpu_ctx, N, nx, warp, drag, relax):
    import self_gb300 as sg
    nod, mesh, q, h, fcor, dt, P, rl, ts = _skew_problem(oracle, N, nx, warp, drag, relax)
    sw = sg.ShallowWater(gpu_ctx, nod, mesh, h, fcor, dt, linear_drag=drag, relax=rl, timescale=ts,
                         formulation="skew_symmetric", precision=sg._native.PREC_FP64_EXACT)
    sw.SetSolution(q)
    assert np.array_equal(sw.GlobalTimeDerivative(0.0), P.tendency(q))
    sw.ForwardStepRK3(0.0, 10)
    assert np.array_equal(sw.GetSolution(), P.rk3(q, 10))
    sw.Trash()
