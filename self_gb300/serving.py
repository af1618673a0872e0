"""Continuous-batching serving of elliptic solves and short shallow-water ensemble runs on one GPU.

The request loop is the library's (self_serve_*, a worker thread in C++ that owns every CUDA call): requests are
admitted in arrival order while their device footprint fits the HBM budget and stay on the GPU until they finish.
Helmholtz solves share one batched slot pool whose ticks (outer FP64 residual step, outer decision and inner PCG
iterations) run on the device with one synchronisation per tick; shallow-water members run on their own handles on
a few extra streams, in chunks of RK3 steps enqueued asynchronously, so their kernels overlap the solves.  A result
depends only on its own request, so it is bit-identical alone and in the mix (tests/test_serving_gpu.py).

This module is the Python driver: it builds the requests' descriptors, submits each request at its arrival time
and reads back the outcome.
"""
import ctypes as C
import time

import numpy as np

from . import _native as nat
from .cgsem import CG2DDesc, SolveReport, cg2d_desc
from .dgsem import dg2d_desc

QUEUED, RUNNING, DONE, CANCELLED, FAILED = 0, 1, 2, 3, 4


class ServeOpts(C.Structure):
    _fields_ = [("hbm_budget_bytes", C.c_double), ("precision", C.c_int), ("tolerance", C.c_double),
                ("inner_tolerance", C.c_double), ("max_outer", C.c_int), ("maxIters", C.c_int),
                ("sw_streams", C.c_int), ("sw_chunk", C.c_int), ("max_active", C.c_int)]


class ServeInfo(C.Structure):
    _fields_ = [("state", C.c_int), ("kind", C.c_int), ("status", C.c_int), ("steps_done", C.c_int),
                ("submit_s", C.c_double), ("admit_s", C.c_double), ("done_s", C.c_double), ("report", SolveReport)]


class ServeStats(C.Structure):
    _fields_ = [("submitted", C.c_longlong), ("admitted", C.c_longlong), ("finished", C.c_longlong),
                ("cancelled", C.c_longlong), ("failed", C.c_longlong), ("queued", C.c_longlong),
                ("running", C.c_longlong), ("bytes_in_use", C.c_longlong), ("p50_ms", C.c_double),
                ("p99_ms", C.c_double), ("mean_ms", C.c_double), ("throughput_per_s", C.c_double),
                ("elapsed_s", C.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


def poisson_arrivals(n, rate, seed):
    rng = np.random.default_rng(seed)
    return np.cumsum(rng.exponential(1.0 / rate, n))


class Request:
    def __init__(self, rid, kind, arrival, payload):
        self.rid, self.kind, self.arrival, self.payload = rid, kind, arrival, payload
        self.admitted = self.finished = None
        self.result = None
        self.report = None
        self.state = None


class Server:
    """Drives one self_serve loop per run().  precision "fp32": FP32-inner solves under FP64 refinement and FP32
    shallow-water members; "fp64": the plain FP64 path for both.  max_active = 1 serves one request at a time."""

    def __init__(self, ctx, hbm_budget=150e9, sw_streams=4, sw_chunk=10, tolerance=1e-10, inner_tolerance=1e-4,
                 precision="fp32", max_active=0):
        self.ctx = ctx
        self.budget = hbm_budget
        self.sw_streams, self.sw_chunk = sw_streams, sw_chunk
        self.tolerance, self.inner_tolerance = tolerance, inner_tolerance
        self.precision = nat.PREC_FP32 if precision == "fp32" else nat.PREC_FP64
        self.max_active = max_active
        self.keep_results = True
        self.stats = None

    def footprint(self, req):
        """Device bytes the loop charges a request at admission (the same estimate as the library's)."""
        pr = req.payload
        if req.kind == "helmholtz":
            d = CG2DDesc()
            d.N, d.nEl = pr["nodal"].N, pr["mesh"].nEl
            b = C.c_longlong()
            nat.check(nat.lib().self_cgbatch_footprint(C.byref(d), C.byref(b)))
            return b.value
        nn = (pr["nodal"].N + 1) ** 2
        return pr["mesh"].nEl * (nn * 3 * 4 * 40 // 3) * (1 if self.precision == nat.PREC_FP32 else 2) + 4096

    def _desc(self, req):
        pr = req.payload
        if req.kind == "helmholtz":
            d, keep = cg2d_desc(pr["nodal"], pr["mesh"], pr["k"], pr.get("lam", 0.1))
            src = np.ascontiguousarray(pr["source"], dtype=np.float64)
            return d, (keep, src), src
        d, keep = dg2d_desc(pr["nodal"], pr["mesh"], nat.MODEL_SW_CONSERVATIVE, 3, pr["dt"], self.precision,
                            h=pr["h"], dhdx=pr["dhdx"], dhdy=pr["dhdy"], fcor=pr["fcor"])
        q = np.ascontiguousarray(pr["q"], dtype=np.float64)
        return d, (keep, q), q

    def run(self, requests):
        """Serve `requests` (sorted by arrival time, seconds from the start): each is submitted at its arrival time
        and the call returns when all are finished.  admitted / finished are on the arrival clock."""
        L = nat.lib()
        o = ServeOpts(self.budget, self.precision, self.tolerance, self.inner_tolerance, 30, 100000, self.sw_streams,
                      self.sw_chunk, self.max_active)
        sp = C.c_void_p()
        nat.check(L.self_serve_create(self.ctx.ptr, C.byref(o), C.byref(sp)), self.ctx.ptr)
        tickets = []
        try:
            descs = [self._desc(r) for r in requests]  # kept alive until the loop is destroyed
            t0 = time.perf_counter()
            for r, (d, k, data) in zip(requests, descs):
                wait = r.arrival - (time.perf_counter() - t0)
                if wait > 0:
                    time.sleep(wait)
                t = C.c_longlong()
                if r.kind == "helmholtz":
                    nat.check(L.self_serve_submit_solve(sp, C.byref(d), nat.d(data), C.byref(t)))
                else:
                    nat.check(L.self_serve_submit_sw(sp, C.byref(d), nat.d(data), int(r.payload["steps"]), C.byref(t)))
                tickets.append(t.value)
            nat.check(L.self_serve_wait(sp, C.c_double(3600.0)))
            for r, t, (d, k, data) in zip(requests, tickets, descs):
                info = ServeInfo()
                nat.check(L.self_serve_poll(sp, C.c_longlong(t), C.byref(info)))
                r.state = info.state
                if info.state != DONE:
                    raise nat.SelfError(info.status, f"request {r.rid} ended in state {info.state}")
                shift = r.arrival - info.submit_s
                r.admitted, r.finished = info.admit_s + shift, info.done_s + shift
                if r.kind == "helmholtz":
                    r.report = {k2: getattr(info.report, k2) for k2, _ in SolveReport._fields_}
                if self.keep_results:
                    n = data.size if r.kind == "sw" else r.payload["mesh"].nEl * (r.payload["nodal"].N + 1) ** 2
                    out = np.zeros(n)
                    nat.check(L.self_serve_result(sp, C.c_longlong(t), nat.d(out), C.c_size_t(n)))
                    r.result = out
            st = ServeStats()
            nat.check(L.self_serve_stats(sp, C.byref(st)))
            self.stats = st.as_dict()
        finally:
            L.self_serve_destroy(sp)
        return requests

    def close(self):
        pass


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
