"""Hot path on meshes read from ISM-V2 files (unstructured connectivity, edges of both orientations, curved
boundary records): DG shallow-water tendency and RK3 (FP64 against the oracle, FP32 form against FP64) on
tests/golden/box.mesh, and the CGSEM PCG solve on tests/golden/square.mesh."""
import os

import numpy as np
import pytest

from helpers import per_var_rel, rel_inf

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))


def _box_sw(oracle, N):
    import self_gb300 as sg
    nod = sg.NodalStorage_2D(N)
    mesh = sg.read_ism_mesh(os.path.join(HERE, "golden", "box.mesh"), N, sg._native.GAUSS)
    x, y = mesh.x, mesh.y
    h = 10.0 - 2.0 * np.exp(-((x - 0.5) ** 2 + (y - 0.5) ** 2) / 0.02)
    H = h + 0.1 * np.exp(-((x - 0.3) ** 2 + (y - 0.6) ** 2) / 0.005)
    rng = np.random.default_rng(3)
    n2, ne = (N + 1) ** 2, mesh.nEl
    q = np.zeros((ne, 3, n2))
    q[:, 0] = rng.normal(0, 0.5, (ne, n2))
    q[:, 1] = rng.normal(0, 0.5, (ne, n2))
    q[:, 2] = H.reshape(ne, n2)
    fcor = 1.0 + 0.5 * y
    c = np.sqrt(9.81 * H.max())
    dt = 0.2 * float(np.sqrt(np.abs(mesh.J).min())) / ((2 * N + 1) * c)
    dhdx, dhdy = sg.bathymetry_gradient(nod, mesh, h)
    P = oracle.DGProblem(nod, mesh, 1, 3, dt, g=9.81, h=h, dhdx=dhdx, dhdy=dhdy, fcor=fcor)
    return nod, mesh, q.ravel(), h, fcor, dhdx, dhdy, dt, P


def test_sw_tendency_and_rk3_on_ism_mesh(oracle, gpu_ctx):
    import self_gb300 as sg
    N = 7
    nod, mesh, q, h, fcor, dhdx, dhdy, dt, P = _box_sw(oracle, N)
    sw = sg.ShallowWater(gpu_ctx, nod, mesh, h, fcor, dt, dhdx=dhdx, dhdy=dhdy)
    sw.SetSolution(q)
    errs = per_var_rel(sw.GlobalTimeDerivative(0.0), P.tendency(q), 3, (N + 1) ** 2)
    assert max(errs) <= 1e-12, errs
    sw.ForwardStepRK3(0.0, 10)
    ref = P.rk3(q, 10)
    errs = per_var_rel(sw.GetSolution(), ref, 3, (N + 1) ** 2)
    assert max(errs) <= 1e-11, errs
    # FP32 form (fused stage, N = 7, walls only) close to FP64 in the perturbation
    s32 = sg.ShallowWater(gpu_ctx, nod, mesh, h, fcor, dt, dhdx=dhdx, dhdy=dhdy, precision=sg._native.PREC_FP32)
    s32.SetSolution(q)
    s32.ForwardStepRK3(0.0, 10)
    got = s32.GetSolution().reshape(mesh.nEl, 3, -1)
    r = ref.reshape(mesh.nEl, 3, -1)
    hh = h.reshape(mesh.nEl, -1)
    assert rel_inf(got[:, 0], r[:, 0]) < 1e-4 and rel_inf(got[:, 1], r[:, 1]) < 1e-4
    assert rel_inf(got[:, 2] - hh, r[:, 2] - hh) < 1e-4


def test_pcg_on_ism_mesh_with_curved_boundary_records(oracle, gpu_ctx):
    import self_gb300 as sg
    from self_gb300 import workloads as W
    N = 6
    nod = sg.NodalStorage_2D(N, sg._native.GAUSS_LOBATTO, sg._native.CG)
    mesh = sg.read_ism_mesh(os.path.join(HERE, "golden", "square.mesh"), N, sg._native.GAUSS_LOBATTO)
    k, f, source = W.helmholtz(mesh, N)
    P = oracle.CGProblem(nod, mesh, k, lam=0.1)
    cg = sg.CGsemElliptic_2D(gpu_ctx, nod, mesh, k, lam=0.1)
    u = np.random.default_rng(4).normal(size=cg.nl)
    assert rel_inf(cg.MatrixAction(u), P.matrix_action(u)) <= 1e-12
    sol, rep = cg.Solve(source, method="pcg", tolerance=1e-10)
    osol, ioerr, oit, _ = P.solve_pcg(source, maxIters=5000, tol=1e-10)
    assert rep["ioerr"] == 0 and ioerr == 0
    assert abs(rep["iterations"] - oit) <= max(2, 0.02 * oit)
    assert rel_inf(sol, osol) <= 1e-8
