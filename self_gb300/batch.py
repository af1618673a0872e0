"""Batched uneven CGSEM solves (self_cgbatch_*): many Helmholtz problems of different sizes and degrees in one
set of launches, with the project autotuner for the element-operator tiles."""
import ctypes as C

import numpy as np

from . import _native as nat
from .cgsem import CG2DDesc, SolveOpts, SolveReport


class CGBatch:
    def __init__(self, ctx, problems):
        """problems: list of dicts with keys nodal, mesh, k, source, lam."""
        self.ctx = ctx
        n = len(problems)
        descs = (CG2DDesc * n)()
        self._keep = []
        for p, pr in enumerate(problems):
            nod, mesh = pr["nodal"], pr["mesh"]
            k = np.ascontiguousarray(pr["k"], dtype=np.float64)
            s = descs[p]
            s.N, s.nEl, s.nEdges, s.nNodes = nod.N, mesh.nEl, mesh.nEdges, mesh.nNodes
            s.dmat, s.qweight = nat.d(nod.dmatS), nat.d(nod.w)
            s.edges, s.nodeType = nat.i(mesh.edges), nat.i(mesh.nodeType)
            s.n2e_ptr, s.n2e_elem, s.n2e_local = nat.i(mesh.n2e_ptr), nat.i(mesh.n2e_elem), nat.i(mesh.n2e_local)
            s.dxds, s.dxdp, s.dyds, s.dydp, s.J = (nat.d(getattr(mesh, f)) for f in ("dxds", "dxdp", "dyds", "dydp", "J"))
            s.fluxCoeff = nat.d(k)
            s.lam, s.op, s.vx, s.vy = pr.get("lam", 0.1), 0, 0.0, 0.0
            self._keep.append((nod, mesh, k))
        p = C.c_void_p()
        nat.check(nat.lib().self_cgbatch_create(ctx.ptr, n, descs, C.byref(p)), ctx.ptr)
        self.ptr = p
        ctx.adopt(self)
        self.n = n
        self.sizes = []
        for i, pr in enumerate(problems):
            src = np.ascontiguousarray(pr["source"], dtype=np.float64)
            nat.check(nat.lib().self_cgbatch_set_source(self.ptr, i, nat.d(src)), ctx.ptr)
            nl = C.c_longlong()
            nat.check(nat.lib().self_cgbatch_problem_size(self.ptr, i, C.byref(nl)), ctx.ptr)
            self.sizes.append(nl.value)
        self._keep = None

    def autotune(self, cache_path=None):
        nat.check(nat.lib().self_cgbatch_autotune(self.ptr, cache_path.encode() if cache_path else None), self.ctx.ptr)
        out = {}
        for N in range(2, 10):
            for b in range(4):
                e = C.c_int()
                nat.check(nat.lib().self_cgbatch_tuning(self.ptr, N, b, C.byref(e)), self.ctx.ptr)
                out[(N, b)] = e.value
        return out

    def Solve(self, precision="fp32", tolerance=1e-10, inner_tolerance=1e-4, maxIters=50000, max_outer=30):
        o = SolveOpts()
        o.method, o.precision, o.maxIters, o.m = 1, nat.PREC_FP32 if precision == "fp32" else nat.PREC_FP64, maxIters, 0
        o.tolerance, o.inner_tolerance, o.max_outer = tolerance, inner_tolerance, max_outer
        reps = (SolveReport * self.n)()
        nat.check(nat.lib().self_cgbatch_solve(self.ptr, C.byref(o), reps), self.ctx.ptr)
        return [r.as_dict() for r in reps]

    def GetSolution(self, p):
        out = np.zeros(self.sizes[p])
        nat.check(nat.lib().self_cgbatch_get_solution(self.ptr, p, nat.d(out)), self.ctx.ptr)
        return out

    def Trash(self):
        if getattr(self, "ptr", None):
            nat.lib().self_cgbatch_destroy(self.ptr)
            self.ptr = None

    def __del__(self):
        try:
            self.Trash()
        except Exception:
            pass
