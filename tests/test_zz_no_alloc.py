"""self_dot_noalloc: the dot product for callers that cannot allocate device memory where they need it (their
device arrays live in their own OpenACC / CUDA Fortran data regions that forbid allocation in the time loop).
It must give the same inner product as the existing DotProduct entry point (self_cg2d_dot) on the same masked
vectors, on two calls in a row that share its static scratch array; sum many tiles with a partial last tile as
an FP64 dot does; and reject lengths beyond its scratch limit.  Collected last on purpose."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

LIMIT = 4096 * 16384  # elements covered by the static array of partial sums


def _fn():
    from self_gb300 import _native as nat
    f = nat.lib().self_dot_noalloc
    f.argtypes = [C.c_void_p, C.c_void_p, C.c_longlong, C.c_void_p, C.c_void_p]
    f.restype = C.c_int
    return f


def test_dot_noalloc_matches_dotproduct_two_calls(gpu_ctx):
    torch = pytest.importorskip("torch")
    import self_gb300 as sg
    from self_gb300 import _native as nat
    from self_gb300 import workloads as W
    N, nx = 5, 6
    nod = sg.NodalStorage_2D(N, nat.GAUSS_LOBATTO, nat.CG)
    mesh = sg.QuadMesh(nx, nx, N, nat.GAUSS_LOBATTO, boundary_flag=nat.DIRICHLET)
    k, f, source = W.helmholtz(mesh, N)
    cg = sg.CGsemElliptic_2D(gpu_ctx, nod, mesh, k, lam=0.1)
    dot = _fn()
    rng = np.random.default_rng(2024)
    res = torch.zeros(1, dtype=torch.float64, device="cuda")
    for call in range(2):
        u, v = rng.normal(size=cg.nl), rng.normal(size=cg.nl)
        expected = cg.DotProduct(u, v)  # existing entry point: masks both vectors, then sums
        um, vm = cg.Mask(u), cg.Mask(v)
        xd = torch.from_numpy(um).to("cuda")
        yd = torch.from_numpy(vm).to("cuda")
        torch.cuda.synchronize()
        rc = dot(xd.data_ptr(), yd.data_ptr(), um.size, res.data_ptr(), None)
        assert rc == 0, nat.last_error()
        torch.cuda.synchronize()
        got = res.item()
        assert abs(got - expected) <= 1e-12 * np.sum(np.abs(um * vm)), (call, got, expected)


def test_dot_noalloc_many_tiles_partial_tail(gpu_ctx):
    """n spans several 16384-element tiles plus a partial one, so the partials of many blocks are indexed and
    summed; two calls in a row with different data and lengths reuse the scratch."""
    torch = pytest.importorskip("torch")
    from self_gb300 import _native as nat
    dot = _fn()
    rng = np.random.default_rng(7)
    res = torch.zeros(1, dtype=torch.float64, device="cuda")
    for n in (3 * 16384 + 17, 37 * 16384 + 1):
        x, y = rng.normal(size=n), rng.normal(size=n)
        xd, yd = torch.from_numpy(x).to("cuda"), torch.from_numpy(y).to("cuda")
        torch.cuda.synchronize()
        rc = dot(xd.data_ptr(), yd.data_ptr(), n, res.data_ptr(), None)
        assert rc == 0, nat.last_error()
        torch.cuda.synchronize()
        expected = float(np.dot(x, y))
        assert abs(res.item() - expected) <= 1e-12 * float(np.sum(np.abs(x * y))), (n, res.item(), expected)


def test_dot_noalloc_rejects_length_beyond_scratch(gpu_ctx):
    torch = pytest.importorskip("torch")
    from self_gb300 import _native as nat
    dot = _fn()
    x = torch.zeros(16, dtype=torch.float64, device="cuda")
    res = torch.zeros(1, dtype=torch.float64, device="cuda")
    rc = dot(x.data_ptr(), x.data_ptr(), LIMIT + 1, res.data_ptr(), None)
    assert rc == -1  # SELF_ERR_INVALID
    assert "exceeds" in nat.last_error()
    # a valid length right after the rejected one still works
    rc = dot(x.data_ptr(), x.data_ptr(), 16, res.data_ptr(), None)
    torch.cuda.synchronize()
    assert rc == 0 and res.item() == 0.0
