"""Continuous-batching serving loop for elliptic solves and short shallow-water ensemble runs on one GPU.

Requests arrive over time (seeded Poisson stream).  The loop admits a request as soon as its device footprint
fits the HBM budget, then keeps it on the GPU until it finishes:

* Helmholtz solves join a single CGBatch slot pool (self_cgbatch_add): every loop tick advances all active
  solves together -- FP64 outer residual updates for those whose inner solve ended, then one CUDA graph of
  FP32 inner PCG iterations covering every active problem (one launch per phase for all of them, whatever their
  mesh size and degree).  Finished solves leave their slot (self_cgbatch_remove) and free their memory.
* Shallow-water ensemble members (FP32 form) each get their own handle on one of a few extra streams and advance
  in chunks of RK3 steps enqueued asynchronously, so their kernels overlap with the batched solves on the device.

Every result depends only on its own request: the batched solver's per-problem arithmetic and reduction order do
not depend on which other problems share the pool, and each ensemble member runs on its own handle, so a result
computed in the mix is bit-identical to the same request served alone (tests/test_serving_gpu.py checks this).
"""
import ctypes as C
import time

import numpy as np

from . import _native as nat
from .batch import CGBatch
from .cgsem import CG2DDesc, SolveOpts, SolveReport
from .dgsem import Context, ShallowWater


def poisson_arrivals(n, rate, seed):
    rng = np.random.default_rng(seed)
    return np.cumsum(rng.exponential(1.0 / rate, n))


class Request:
    def __init__(self, rid, kind, arrival, payload):
        self.rid, self.kind, self.arrival, self.payload = rid, kind, arrival, payload
        self.admitted = self.finished = None
        self.result = None
        self.report = None


class Server:
    def __init__(self, ctx, hbm_budget=150e9, sw_streams=4, sw_chunk=10, tolerance=1e-10, inner_tolerance=1e-4,
                 precision="fp32", graph_chunk=None):
        self.ctx = ctx
        self.budget = hbm_budget
        self.sw_chunk = sw_chunk
        self.pool = CGBatch(ctx, [])
        self.opts = SolveOpts()
        self.opts.method, self.opts.precision = 1, nat.PREC_FP32 if precision == "fp32" else nat.PREC_FP64
        self.opts.maxIters, self.opts.m, self.opts.tolerance = 100000, 0, tolerance
        self.opts.inner_tolerance, self.opts.max_outer = inner_tolerance, 30
        self.sw_ctx = [Context(0) for _ in range(sw_streams)]
        self.active_cg = {}  # slot -> request
        self.active_sw = []  # (request, handle, ctx, steps_done)
        self.used = 0
        self.keep_results = True

    # -------------------------------------------------------------------------------- admission
    def _cg_footprint(self, pr):
        d = CG2DDesc()
        d.N, d.nEl = pr["nodal"].N, pr["mesh"].nEl
        b = C.c_longlong()
        nat.check(nat.lib().self_cgbatch_footprint(C.byref(d), C.byref(b)))
        return b.value

    def _sw_footprint(self, pr):
        n2 = (pr["nodal"].N + 1) ** 2
        return pr["mesh"].nEl * n2 * 4 * 40  # FP32 state, register, metrics, aux, traces and staging

    def footprint(self, req):
        return self._cg_footprint(req.payload) if req.kind == "helmholtz" else self._sw_footprint(req.payload)

    def _admit(self, req, now):
        pr = req.payload
        if req.kind == "helmholtz":
            nod, mesh = pr["nodal"], pr["mesh"]
            d = CG2DDesc()
            k = np.ascontiguousarray(pr["k"], dtype=np.float64)
            d.N, d.nEl, d.nEdges, d.nNodes = nod.N, mesh.nEl, mesh.nEdges, mesh.nNodes
            d.dmat, d.qweight = nat.d(nod.dmatS), nat.d(nod.w)
            d.edges, d.nodeType = nat.i(mesh.edges), nat.i(mesh.nodeType)
            d.n2e_ptr, d.n2e_elem, d.n2e_local = nat.i(mesh.n2e_ptr), nat.i(mesh.n2e_elem), nat.i(mesh.n2e_local)
            d.dxds, d.dxdp, d.dyds, d.dydp, d.J = (nat.d(getattr(mesh, f)) for f in ("dxds", "dxdp", "dyds", "dydp", "J"))
            d.fluxCoeff = nat.d(k)
            d.lam, d.op = pr.get("lam", 0.1), 0
            slot = C.c_int()
            src = np.ascontiguousarray(pr["source"], dtype=np.float64)
            nat.check(nat.lib().self_cgbatch_add(self.pool.ptr, C.byref(d), nat.d(src), C.byref(slot)), self.ctx.ptr)
            self.pool.sizes_by_slot = getattr(self.pool, "sizes_by_slot", {})
            nl = C.c_longlong()
            nat.check(nat.lib().self_cgbatch_problem_size(self.pool.ptr, slot.value, C.byref(nl)))
            self.pool.sizes_by_slot[slot.value] = nl.value
            self.active_cg[slot.value] = req
        else:
            cx = self.sw_ctx[len(self.active_sw) % len(self.sw_ctx)]
            sw = ShallowWater(cx, pr["nodal"], pr["mesh"], pr["h"], pr["fcor"], pr["dt"], dhdx=pr["dhdx"],
                              dhdy=pr["dhdy"], precision=nat.PREC_FP32)
            sw.SetSolution(pr["q"])
            self.active_sw.append([req, sw, cx, 0])
        req.admitted = now
        self.used += self.footprint(req)

    # -------------------------------------------------------------------------------- loop
    def run(self, requests, t_offset=None):
        """Serve `requests` (sorted by arrival time, seconds from the start).  Returns the list of requests with
        admitted/finished times filled in."""
        pending = list(requests)
        queue = []
        t0 = time.perf_counter() if t_offset is None else t_offset
        lib = nat.lib()
        done = 0
        total = len(pending)
        while done < total:
            now = time.perf_counter() - t0
            while pending and pending[0].arrival <= now:
                queue.append(pending.pop(0))
            while queue and self.used + self.footprint(queue[0]) <= self.budget:
                self._admit(queue.pop(0), now)
            # shallow-water members: enqueue the next chunk on idle streams
            for ent in self.active_sw:
                req, sw, cx, steps = ent
                if steps < req.payload["steps"] and lib.self_ctx_query(cx.ptr) == 1:
                    k = min(self.sw_chunk, req.payload["steps"] - steps)
                    sw.ForwardStepRK3_async(0.0, k)
                    ent[3] = steps + k
            # batched solves: one tick for every active problem
            if self.active_cg:
                nfin = C.c_int()
                nat.check(lib.self_cgbatch_step(self.pool.ptr, C.byref(self.opts), C.byref(nfin)), self.ctx.ptr)
                for slot in list(self.active_cg):
                    rep, fin = SolveReport(), C.c_int()
                    nat.check(lib.self_cgbatch_report(self.pool.ptr, slot, C.byref(rep), C.byref(fin)))
                    if fin.value:
                        req = self.active_cg.pop(slot)
                        req.report = rep.as_dict()
                        if self.keep_results:
                            out = np.zeros(self.pool.sizes_by_slot[slot])
                            nat.check(lib.self_cgbatch_get_solution(self.pool.ptr, slot, nat.d(out)))
                            req.result = out
                        nat.check(lib.self_cgbatch_remove(self.pool.ptr, slot))
                        req.finished = time.perf_counter() - t0
                        self.used -= self.footprint(req)
                        done += 1
            # finished shallow-water members
            still = []
            for ent in self.active_sw:
                req, sw, cx, steps = ent
                if steps >= req.payload["steps"] and lib.self_ctx_query(cx.ptr) == 1:
                    if self.keep_results:
                        req.result = sw.GetSolution()
                    sw.Trash()
                    req.finished = time.perf_counter() - t0
                    self.used -= self.footprint(req)
                    done += 1
                else:
                    still.append(ent)
            self.active_sw = still
            if not self.active_cg and not self.active_sw and not queue and pending:
                time.sleep(max(0.0, min(1e-3, pending[0].arrival - (time.perf_counter() - t0))))
        return requests

    def close(self):
        self.pool.Trash()
        for c in self.sw_ctx:
            c.close()


def latency_stats(reqs):
    lat = np.array([r.finished - r.arrival for r in reqs])
    span = max(r.finished for r in reqs) - min(r.arrival for r in reqs)
    return {"p50_ms": 1e3 * float(np.percentile(lat, 50)), "p99_ms": 1e3 * float(np.percentile(lat, 99)),
            "mean_ms": 1e3 * float(lat.mean()), "throughput_req_s": len(reqs) / span, "requests": len(reqs)}


def make_requests(mod, n, rate=2000.0, seed=5, frac_helmholtz=0.7, sw_nx=64, sw_N=5, sw_steps=100,
                  helmholtz_nmax=64):
    """The serving mix: Poisson arrivals; 70 % Helmholtz solves from the batched distribution, 30 % shallow-water
    ensemble members (64x64 quads, N = 5, 100 steps, initial heights perturbed by the member's seed)."""
    from . import workloads as W
    arr = poisson_arrivals(n, rate, seed)
    rng = np.random.default_rng(seed + 1)
    kinds = rng.uniform(size=n) < frac_helmholtz
    reqs = []
    sw_mesh = None
    for i in range(n):
        if kinds[i]:
            r = np.random.default_rng(seed * 100000 + i)
            nx, N = int(r.integers(8, helmholtz_nmax + 1)), int(r.integers(3, 10))
            reqs.append(Request(i, "helmholtz", float(arr[i]), W.batched_problem(mod, nx, N, seed * 100000 + i)))
        else:
            if sw_mesh is None:
                nod = mod.NodalStorage_2D(sw_N)
                mesh = mod.QuadMesh(sw_nx, sw_nx, sw_N, warp=W.SW_WARP, scale=(W.SW_L, W.SW_L))
                sw_mesh = (nod, mesh)
            nod, mesh = sw_mesh
            q, h, fcor, dt = W.shallow_water(mesh, sw_N, sw_nx, seed=seed * 100000 + i)
            dhdx, dhdy = mod.bathymetry_gradient(nod, mesh, h)
            reqs.append(Request(i, "sw", float(arr[i]), {"nodal": nod, "mesh": mesh, "q": q, "h": h, "fcor": fcor,
                                                          "dt": dt, "dhdx": dhdx, "dhdy": dhdy, "steps": sw_steps}))
    return reqs
