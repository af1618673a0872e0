"""ctypes binding of libselfgpu.so (the C ABI declared in include/self_gpu.h).

The library is built in-tree by self_gb300/build.py.  There is no CPU fallback: if the shared library
is missing or a call fails, an exception is raised.
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libselfgpu.so")

OK = 0
NO_NORMAL_FLOW = -100
INFLOW_ONE = -103
INFLOW_TWO = -104
DIRICHLET = -200
GAUSS = 1
GAUSS_LOBATTO = -1
DG = 2000
CG = 2001
MODEL_SW_CONSERVATIVE = 1
MODEL_ADVECTION = 2
MODEL_SW_LINEAR = 3
MODEL_SW_SKEW = 4
PREC_FP64 = 0
PREC_FP32 = 1
PREC_FP64_EXACT = 2

dp = C.POINTER(C.c_double)
fp = C.POINTER(C.c_float)
ip = C.POINTER(C.c_int)

_lib = None


class SelfError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(f"libselfgpu status {status}: {msg}")
        self.status = status


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"{LIB_PATH} is missing: build it with "
                              "`python -c 'import __graft_entry__ as g; g.build()'` (no CPU fallback exists)")
        L = C.CDLL(LIB_PATH)
        L.self_status_string.restype = C.c_char_p
        L.self_ctx_kernel_launches.restype = C.c_longlong
        _lib = L
    return _lib


def last_error(ctx=None):
    buf = C.create_string_buffer(1024)
    lib().self_last_error(ctx, buf, 1024)
    return buf.value.decode(errors="replace")


def check(status, ctx=None):
    if status != OK:
        raise SelfError(status, last_error(ctx) or lib().self_status_string(status).decode())
    return status


def d(a):
    if a is None:
        return None
    assert a.dtype == np.float64 and a.flags["C_CONTIGUOUS"], "float64 C-contiguous array required"
    return a.ctypes.data_as(dp)


def f32(a):
    if a is None:
        return None
    assert a.dtype == np.float32 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(fp)


def i(a):
    if a is None:
        return None
    assert a.dtype == np.int32 and a.flags["C_CONTIGUOUS"], "int32 C-contiguous array required"
    return a.ctypes.data_as(ip)


class DG2DDesc(C.Structure):
    _fields_ = [("N", C.c_int), ("nEl", C.c_int), ("nEdges", C.c_int), ("nEq", C.c_int), ("model", C.c_int),
                ("precision", C.c_int),
                ("dmatS", dp), ("dmatP", dp), ("qweight", dp), ("lagW", dp), ("lagE", dp), ("lagS", dp),
                ("lagN", dp), ("edges", ip), ("dxds", dp), ("dxdp", dp), ("dyds", dp), ("dydp", dp), ("J", dp),
                ("nhx", dp), ("nhy", dp), ("nlen", dp), ("h", dp), ("dhdx", dp), ("dhdy", dp), ("fcor", dp),
                ("relax", dp), ("rfac", dp), ("u", dp), ("v", dp),
                ("g", C.c_double), ("linear_drag", C.c_double), ("dt", C.c_double), ("kappa", C.c_double)]
