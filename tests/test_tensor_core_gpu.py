"""FP32 CGSEM operator with its derivative contractions on the tensor cores (tcgen05 GEMMs over 32-element tiles,
compensated TF32 products), N = 7.

* Operator: the FP32 MatrixAction with the tensor-core contractions agrees with the FP64 MatrixAction to 2e-5 of
  max |Au| (the FP32 operator's own rounding; the CUDA-core FP32 form is held to the same bar), on a mesh with a
  partial last tile, for the Helmholtz operator and the advection-diffusion operator (6 factors).
* Solve: FP32-inner PCG under FP64 refinement with tensor_cores reaches ||r||/||r0|| < 1e-10, its solution is within
  1e-8 of the FP64 PCG solution, and its inner iteration count is within 10 % of the CUDA-core FP32 form.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _cg(gpu_ctx, nx, op=0):
    import self_gb300 as sg
    from self_gb300 import _native as nat
    from self_gb300 import workloads as W
    N = 7
    nod = sg.NodalStorage_2D(N, nat.GAUSS_LOBATTO, nat.CG)
    mesh = sg.QuadMesh(nx, nx, N, nat.GAUSS_LOBATTO, warp=0.03, boundary_flag=nat.DIRICHLET)
    k, f, source = W.helmholtz(mesh, N)
    if op == 1:
        return sg.CGsemElliptic_2D(gpu_ctx, nod, mesh, np.full_like(k, 1e-2), lam=0.0, op=1, vel=(1.0, 0.5)), source
    return sg.CGsemElliptic_2D(gpu_ctx, nod, mesh, k, lam=0.1), source


@pytest.mark.parametrize("nx,op", [(6, 0), (9, 0), (6, 1)])
def test_tensor_core_operator_matches_fp64(gpu_ctx, nx, op):
    cg, _ = _cg(gpu_ctx, nx, op)
    rng = np.random.default_rng(17)
    u = cg.UnMask(cg.Mask(rng.normal(size=cg.nl)))
    ref = cg.MatrixAction(u)
    scale = np.abs(ref).max()
    tc = cg.MatrixAction32(u, tensor_cores=True)
    cc = cg.MatrixAction32(u, tensor_cores=False)
    assert np.abs(cc - ref).max() <= 2e-5 * scale
    assert np.abs(tc - ref).max() <= 2e-5 * scale, np.abs(tc - ref).max() / scale
    assert not np.array_equal(tc, cc)  # a different kernel: the products round differently
    cg.Trash()


def test_tensor_core_fp32_refined_pcg(gpu_ctx):
    cg, source = _cg(gpu_ctx, 12)
    s64, r64 = cg.Solve(source, method="pcg", tolerance=1e-10)
    s32, r32 = cg.Solve(source, method="pcg", precision="fp32", tolerance=1e-10)
    stc, rtc = cg.Solve(source, method="pcg", precision="fp32", tolerance=1e-10, tensor_cores=True)
    assert rtc["ioerr"] == 0 and rtc["rel_residual"] < 1e-10
    assert np.abs(stc - s64).max() <= 1e-8 * np.abs(s64).max()
    assert abs(rtc["iterations"] - r32["iterations"]) <= 0.1 * r32["iterations"]
    cg.Trash()
