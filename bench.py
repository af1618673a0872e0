#!/usr/bin/env python3
"""Benchmark of the DGSEM 2-D shallow-water step (LSRK3) on one GB300 per rank.

Workload (the configuration the DG metric is quoted on): conservative shallow water on [0, 2e6 m]^2,
128 x 128 curvilinear quads (x,y += 0.05 L sin(2 pi x/L) sin(2 pi y/L)), N = 7 Legendre-Gauss nodes,
3 variables = 3,145,728 DOF, beta-plane, seamount bathymetry, 16 seeded Gaussian bumps, mirror walls.
A step is one LSRK3 step: 3 stages, each an edge-flux kernel and a volume + RK-update kernel in the plain FP64
drop-in (the headline), or one fused kernel (edge fluxes + volume + RK update + traces) in the FP32 form.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gpu|reference] [--precision fp64|fp32]
                  [--no-cpu] [--no-elliptic] [--batched-n P] [--serve-n R]

value      DOF-updates/s of the device-resident FP64 drop-in step (inputs in HBM, L2 flushed between timed
           steps), whole job (sum over ranks; ranks are independent replicas).
e2e        the same metric through the C ABI with host (pinned) FP64 buffers: every step uploads the state
           (self_dg2d_set_state), advances one step (self_dg2d_rk3) and downloads it (self_dg2d_get_state).
roofline   one RK stage of the FP64 drop-in (edge-flux + volume kernels, both bound by the FP64 pipe): algorithmic
           FP64 flops per stage / the stage's average duration over the timed region, against the FP64 FMA rate
           measured on this GPU in the same run; the HBM fraction of the same stage beside it.
fp32_form  the FP32 perturbation form on the same workload: DOF-updates/s, its HBM roofline (algorithmic bytes of
           the three fused stages of a step / step time), a cold single launch, e2e, and its height error
           against FP64 after 1000 steps.
cpu_baseline  the CPU oracle (C++ restatement of the reference's Fortran, OpenMP) on a bounded sample.
elliptic   CGSEM Helmholtz 256x256 N=7: FP64 PCG vs FP32-inner PCG under FP64 refinement (solves/s to 1e-10),
           GMRES(30) on advection-diffusion; oracle and GPU solves of a 64x64 N=7 problem timed to 1e-10.
batched    512 uneven Helmholtz problems solved together vs one FP64 solve per launch.
serving    seeded Poisson stream of Helmholtz solves and shallow-water ensemble members: continuous batching
           latency (p50/p99) and throughput vs plain FP64 one request at a time.
--impl reference  times the oracle alone on the host cores, the problem built by the oracle's own set-up
           routines (the reference itself is Fortran with no compiler on this image; the oracle is its
           restatement).
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N_POLY, NX = 7, 128
WORKLOAD = ("DGSEM 2D conservative shallow water, 128x128 curvilinear quads, N=7 Legendre-Gauss, 3 vars = "
            "3,145,728 DOF, one LSRK3 step")
L2_FLUSH_BYTES = 512 << 20  # > 129 MB L2


def _peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class Clocks:
    """nvidia-smi sampling during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                                          "-lms", "200", "-i", str(self.device)], stdout=open(self.path, "w"),
                                         stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for nm, val in zip(names, parts[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(nm)
        os.unlink(self.path)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def build_problem(mod, N=N_POLY, nx=NX):
    """Mesh, bathymetry and initial state of the workload (host set-up, not timed)."""
    from self_gb300 import workloads as W
    nod = mod.NodalStorage_2D(N)
    mesh = mod.QuadMesh(nx, nx, N, warp=W.SW_WARP, scale=(W.SW_L, W.SW_L))
    q, h, fcor, dt = W.shallow_water(mesh, N, nx, seed=2)
    dhdx, dhdy = mod.bathymetry_gradient(nod, mesh, h)
    return nod, mesh, q, h, fcor, dhdx, dhdy, dt


def bytes_per_fused_stage(nEl, n, mode):
    """Algorithmic HBM bytes of one fused FP32 stage (edge fluxes inside): q r/w, G written (and read in stages 2-3,
    mode 2), 5 metric fields, 4 aux fields, 3 lake-at-rest tendency fields, per-side edge data (nx, ny, |n|, hP,
    hS per side node), the element's own and its 4 neighbours' traces read and the element's new traces written."""
    nn = n * n
    g_rw = 2 if mode == 2 else 1
    return 4 * (2 * 3 * nn + g_rw * 3 * nn + 5 * nn + 4 * nn + 3 * nn + 4 * 5 * n + 3 * 4 * 3 * n) * nEl


def bytes_per_fused_step(nEl, n):
    """One LSRK3 step of the FP32 form: stage 1 (no G read) + stages 2 and 3."""
    return bytes_per_fused_stage(nEl, n, 1) + 2 * bytes_per_fused_stage(nEl, n, 2)


# algorithmic FP64 flops of one element-stage at N=7 (both kernels of a stage): volume kernel = traces 1,536, volume
# fluxes 2,176, contractions 6,144, lift 1,536, 1/J 384, sources 512, RK update 768; edge kernel = Riemann 960
FLOPS_VOLUME_PER_EL_N7 = 1536 + 2176 + 6144 + 1536 + 384 + 512 + 768
FLOPS_EDGE_PER_EL_N7 = 960
FLOPS_PER_EL_STAGE_N7 = FLOPS_VOLUME_PER_EL_N7 + FLOPS_EDGE_PER_EL_N7
# algorithmic HBM bytes of one FP64 element-stage at N=7: 8 B x (4 nEq n^2 [q r/w, G r/w] + 5 n^2 metrics + 3 n^2
# aux + 3 2n edge geometry + 2 4 nEq n traces write + read)
BYTES_FP64_PER_EL_STAGE_N7 = 8 * (4 * 3 * 64 + 5 * 64 + 3 * 64 + 3 * 2 * 8 + 2 * 4 * 3 * 8)
# DRAM bytes (read + write) per launch measured by ncu --set full on this workload (one launch each)
NCU_TRAFFIC_BYTES = {"sw32_fused": 80.76e6 + 3.96e6, "dg_volume": 130.06e6 + 24.99e6}


def cpu_baseline(oracle, nod, mesh, q, h, fcor, dhdx, dhdy, dt, budget_s=12.0, max_steps=5000):
    import multiprocessing
    cores = os.cpu_count() or multiprocessing.cpu_count()
    oracle.set_threads(cores)
    P = oracle.DGProblem(nod, mesh, 1, 3, dt, h=h, dhdx=dhdx, dhdy=dhdy, fcor=fcor)
    qq = q.copy()
    qq = P.rk3(qq, 1)  # warm-up
    steps, t0 = 0, time.perf_counter()
    while steps < max_steps and time.perf_counter() - t0 < budget_s:
        qq = P.rk3(qq, 1)
        steps += 1
    el = time.perf_counter() - t0
    dof = q.size
    return {"value": dof * steps / el, "unit": "DOF-updates/s", "cores": cores, "kind": "port",
            "sample": f"{steps} LSRK3 steps of the full 128x128 N=7 shallow-water workload ({el:.1f} s)"}


def dist_init():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    if ws > 1:
        import torch.distributed as dist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group("gloo")
        return dist, int(os.environ.get("RANK", "0")), ws, int(os.environ.get("LOCAL_RANK", "0"))
    return None, 0, 1, 0


def allmax(dist, x):
    if dist is None:
        return x
    import torch
    t = torch.tensor([float(x)], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def build_problem_oracle(O, N=N_POLY, nx=NX):
    """The same workload built by the oracle's own set-up routines (NodalStorage_2D, QuadMesh + MappedGeometry_2D,
    CalculateBathymetryGradient restated): the reference arm loads no product code."""
    from self_gb300 import workloads as W  # seeded numpy input generator (no native code)
    nod = O.Nodal(N, O.GAUSS, O.DG)
    mesh = O.Mesh(nx, nx, N, O.GAUSS, warp=W.SW_WARP, scale=(W.SW_L, W.SW_L))
    q, h, fcor, dt = W.shallow_water(mesh, N, nx, seed=2)
    dhdx, dhdy = O.DGProblem(nod, mesh, 1, 3, dt, h=h).bathymetry_gradient()
    return nod, mesh, q, h, fcor, dhdx, dhdy, dt


def run_reference(args):
    dist, rank, ws, local = dist_init()
    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return
    from oracle import oracle as O
    O.build()
    cores = os.cpu_count()
    O.set_threads(cores)
    nod, mesh, q, h, fcor, dhdx, dhdy, dt = build_problem_oracle(O)
    P = O.DGProblem(nod, mesh, 1, 3, dt, h=h, dhdx=dhdx, dhdy=dhdy, fcor=fcor)
    qq = q.copy()
    for _ in range(args.warmup):
        qq = P.rk3(qq, 1)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        qq = P.rk3(qq, 1)
    el = time.perf_counter() - t0
    val = q.size * args.steps / el
    line = {"metric": "DG DOF-updates/s", "value": val, "unit": "DOF-updates/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * el / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "impl": "reference",
            "config": {"workload": WORKLOAD, "precision_form": "FP64 (the reference's arithmetic)",
                       "parallelism": f"host threads x{cores}"},
            "cpu_baseline": {"value": val, "unit": "DOF-updates/s", "cores": cores, "kind": "port",
                             "sample": f"{args.steps} full LSRK3 steps after {args.warmup} warm-up steps, problem "
                                       "built by the oracle's set-up routines"},
            "e2e": {"value": val, "unit": "DOF-updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


def _time_steps(nat, L, ctx, sw, steps):
    """Device time of `steps` single RK3 steps, each bracketed by CUDA events, L2 flushed in between."""
    import ctypes as C
    ms = C.c_double()
    total = 0.0
    for _ in range(steps):
        nat.check(L.self_ctx_flush_l2(ctx.ptr, C.c_size_t(L2_FLUSH_BYTES)), ctx.ptr)
        nat.check(L.self_ctx_timer_start(ctx.ptr), ctx.ptr)
        sw.ForwardStepRK3_async(0.0, 1)
        nat.check(L.self_ctx_timer_stop(ctx.ptr, C.byref(ms)), ctx.ptr)
        total += ms.value
    return total


def _kernel_ms(nat, L, ctx, sw):
    import ctypes as C
    kms = (C.c_double * 2)()
    nat.check(L.self_dg2d_time_kernels(sw.ptr, 20, C.c_size_t(L2_FLUSH_BYTES), kms), ctx.ptr)
    return kms[0], kms[1]


def _e2e(nat, L, ctx, sw, dof, steps, dist):
    """Through the C ABI with pinned host buffers: upload state, one RK3 step, download state, per step."""
    import ctypes as C
    nbytes = dof * 8
    hp = C.c_void_p()
    nat.check(L.self_host_alloc(C.c_size_t(nbytes), C.byref(hp)))
    hq = np.ctypeslib.as_array((C.c_double * dof).from_address(hp.value))
    hq[:] = sw.GetSolution()
    if dist:
        dist.barrier()
    ms = C.c_double()
    t = 0.0
    for _ in range(steps):
        nat.check(L.self_ctx_timer_start(ctx.ptr), ctx.ptr)
        nat.check(L.self_dg2d_set_state(sw.ptr, hq.ctypes.data_as(nat.dp)), ctx.ptr)
        nat.check(L.self_dg2d_rk3(sw.ptr, C.c_double(0.0), 1), ctx.ptr)
        nat.check(L.self_dg2d_get_state(sw.ptr, hq.ctypes.data_as(nat.dp)), ctx.ptr)
        nat.check(L.self_ctx_timer_stop(ctx.ptr, C.byref(ms)), ctx.ptr)
        t += ms.value
    # the same three calls timed one by one (not part of the reported value)
    parts = {"set_state_ms": 0.0, "rk3_ms": 0.0, "get_state_ms": 0.0}
    calls = (("set_state_ms", lambda: L.self_dg2d_set_state(sw.ptr, hq.ctypes.data_as(nat.dp))),
             ("rk3_ms", lambda: L.self_dg2d_rk3(sw.ptr, C.c_double(0.0), 1)),
             ("get_state_ms", lambda: L.self_dg2d_get_state(sw.ptr, hq.ctypes.data_as(nat.dp))))
    for _ in range(steps):
        for key, fn in calls:
            nat.check(L.self_ctx_timer_start(ctx.ptr), ctx.ptr)
            nat.check(fn(), ctx.ptr)
            nat.check(L.self_ctx_timer_stop(ctx.ptr, C.byref(ms)), ctx.ptr)
            parts[key] += ms.value / steps
    L.self_host_free(hp)
    return t, nbytes, parts


# ------------------------------------------------------------------------------------------ elliptic legs
def elliptic_leg(sg, ctx, nx=256, N=7, gmres_iters=20000):
    """256x256 N=7 variable-coefficient Helmholtz (k = 1 + 0.5 sin 4pi x cos 4pi y, lambda = 0.1, Dirichlet 0,
    Jacobi): plain FP64 PCG vs FP32-inner PCG under FP64 refinement, both to ||r||/||r0|| < 1e-10; GMRES(30) and
    Jacobi-preconditioned flexible GMRES(30) on the advection-diffusion operator (v = (1, 0.5), kappa = 1e-3) to
    1e-10, FP64 and FP32-inner under FP64 refinement."""
    from self_gb300 import workloads as W
    from self_gb300 import _native as nat
    nod = sg.NodalStorage_2D(N, nat.GAUSS_LOBATTO, nat.CG)
    mesh = sg.QuadMesh(nx, nx, N, nat.GAUSS_LOBATTO, boundary_flag=nat.DIRICHLET)
    k, f, source = W.helmholtz(mesh, N, seed=3)
    cg = sg.CGsemElliptic_2D(ctx, nod, mesh, k, lam=0.1)
    out = {"workload": f"CGSEM Helmholtz {nx}x{nx} N={N} GLL, {mesh.nEl * (N + 1) ** 2} local nodes"}
    for prec in ("fp64", "fp32"):
        cg.Solve(source, method="pcg", precision=prec, tolerance=1e-10, maxIters=200)  # warm-up (graphs, buffers)
        ctx.synchronize()
        t0 = time.perf_counter()
        sol, rep = cg.Solve(source, method="pcg", precision=prec, tolerance=1e-10, maxIters=50000)
        el = time.perf_counter() - t0
        out["pcg_" + prec] = {"seconds": el, "solves_per_s": 1.0 / el, "iterations": rep["iterations"],
                              "ms_per_iteration": 1e3 * el / max(1, rep["iterations"]),
                              "outer": rep["outer_iterations"], "rel_residual": rep["rel_residual"],
                              "ioerr": rep["ioerr"]}
        if prec == "fp64":
            s64 = sol
        else:
            out["pcg_fp32"]["max_rel_diff_vs_fp64"] = float(np.abs(sol - s64).max() / np.abs(s64).max())
    out["speedup_fp32_ir_vs_fp64"] = out["pcg_fp64"]["seconds"] / out["pcg_fp32"]["seconds"]
    out["pcg_fp32"]["layout"] = "compact (one value per unknown; pcg_apply_compact_f32 + pcg_update_compact)"

    def fp32_variant(**kw):
        cg.Solve(source, method="pcg", precision="fp32", tolerance=1e-10, maxIters=200, **kw)
        ctx.synchronize()
        t0 = time.perf_counter()
        sol, rep = cg.Solve(source, method="pcg", precision="fp32", tolerance=1e-10, maxIters=50000, **kw)
        el = time.perf_counter() - t0
        return {"seconds": el, "solves_per_s": 1.0 / el, "iterations": rep["iterations"],
                "ms_per_iteration": 1e3 * el / max(1, rep["iterations"]), "outer": rep["outer_iterations"],
                "rel_residual": rep["rel_residual"], "ioerr": rep["ioerr"],
                "max_rel_diff_vs_fp64": float(np.abs(sol - s64).max() / np.abs(s64).max())}

    # the same FP32-inner solve on the element-local masked L-vectors (3 launches per iteration: apply, direct-
    # stiffness sum, update), and with the operator's derivative contractions on the tensor cores (tcgen05,
    # compensated TF32; element-local layout)
    out["pcg_fp32_element_local"] = fp32_variant(inner_layout="local")
    out["pcg_fp32_element_local"]["kernel"] = "pcg_apply_fused_f32 + cg_dss_mask_pairs + pcg_update_fused_vec"
    out["pcg_fp32_tensor_cores"] = fp32_variant(tensor_cores=True)
    out["pcg_fp32_tensor_cores"]["kernel"] = "pcg_apply_tc (tcgen05.mma kind::tf32, 3 products per contraction)"
    # the reference's own %Solve: PCG with the linear-FEM preconditioner (pcIterates = 20, pcTolerance = 1e-4 as in
    # its paraboloid example); the first call builds the preconditioner mesh (host) and captures the graphs
    t0 = time.perf_counter()
    cg.Solve(source, method="pcg_linear", tolerance=1e-10, maxIters=4, pc_iterations=20)
    ctx.synchronize()
    setup = time.perf_counter() - t0
    for prec in ("fp64", "fp32"):
        cg.Solve(source, method="pcg_linear", precision=prec, tolerance=1e-10, maxIters=4, pc_iterations=20)
        ctx.synchronize()
        t0 = time.perf_counter()
        sol, rep = cg.Solve(source, method="pcg_linear", precision=prec, tolerance=1e-10, maxIters=20000,
                            pc_iterations=20, pc_tolerance=1e-4)
        el = time.perf_counter() - t0
        out["pcg_linear_" + prec] = {"seconds": el, "solves_per_s": 1.0 / el, "iterations": rep["iterations"],
                                     "ms_per_iteration": 1e3 * el / max(1, rep["iterations"]),
                                     "inner_iterations_max": 20, "outer": rep["outer_iterations"],
                                     "rel_residual": rep["rel_residual"], "ioerr": rep["ioerr"],
                                     "max_rel_diff_vs_pcg_fp64": float(np.abs(sol - s64).max() / np.abs(s64).max())}
    out["pcg_linear_fp64"]["preconditioner_setup_seconds"] = setup
    cg.Trash()
    ad = sg.CGsemElliptic_2D(ctx, nod, mesh, np.full_like(k, 1e-3), lam=0.0, op=1, vel=(1.0, 0.5))
    ref = None
    for method, prec in (("gmres", "fp64"), ("gmres", "fp32"), ("pgmres", "fp64"), ("pgmres", "fp32")):
        key = ("gmres30_" if method == "gmres" else "pgmres30_jacobi_") + prec
        ad.Solve(source, method=method, precision=prec, m=30, tolerance=1e-10, maxIters=60)  # warm-up
        ctx.synchronize()
        t0 = time.perf_counter()
        sol, rep = ad.Solve(source, method=method, precision=prec, m=30, tolerance=1e-10, maxIters=gmres_iters)
        el = time.perf_counter() - t0
        out[key] = {"seconds": el, "solves_per_s": 1.0 / el, "arnoldi_steps": rep["iterations"],
                    "ms_per_step": 1e3 * el / max(1, rep["iterations"]), "refinement_steps": rep["outer_iterations"],
                    "rel_residual": rep["rel_residual"], "ioerr": rep["ioerr"],
                    "operator": "-kappa Lap u + v.grad u, kappa 1e-3, v (1, 0.5)"}
        if ref is None:
            ref = sol
        else:
            out[key]["max_rel_diff_vs_gmres30_fp64"] = float(np.abs(sol - ref).max() / np.abs(ref).max())
    out["speedup_gmres_fp32_ir_vs_fp64"] = out["gmres30_fp64"]["seconds"] / out["gmres30_fp32"]["seconds"]
    ad.Trash()
    return out, (nod, mesh, k, source)


def elliptic_cpu(oracle, nod, mesh, k, source, iters_gpu, budget_s=10.0):
    """Oracle PCG-Jacobi (restated CGsemElliptic_2D%Solve) on the same problem for a bounded number of
    iterations; solves/s extrapolated with the GPU's iteration count."""
    P = oracle.CGProblem(nod, mesh, k, lam=0.1)
    oracle.set_threads(os.cpu_count())
    n_it = 5
    while True:
        t0 = time.perf_counter()
        P.solve_pcg(source, maxIters=n_it, tol=1e-30, precond=1)
        el = time.perf_counter() - t0
        if el > budget_s / 3 or n_it >= 400:
            break
        n_it *= 2
    per_it = el / n_it
    return {"value": 1.0 / (per_it * iters_gpu), "unit": "solves/s", "cores": os.cpu_count(), "kind": "port",
            "sample": f"{n_it} PCG iterations of the 256x256 N=7 Helmholtz solve ({el:.1f} s), scaled to "
                      f"{iters_gpu} iterations"}


def elliptic_small_measured(sg, ctx, oracle, nx=64, N=7):
    """Whole solves timed on both sides (no extrapolation): the Helmholtz problem of the elliptic leg on a
    64x64 N=7 mesh, PCG-Jacobi to ||r||/||r0|| < 1e-10 by the oracle (OpenMP, all host cores; problem built by the
    oracle's own set-up) and by the GPU (FP64 drop-in and FP32-inner + FP64 refinement)."""
    from self_gb300 import _native as nat
    from self_gb300 import workloads as W
    onod = oracle.Nodal(N, oracle.GAUSS_LOBATTO, oracle.CG)
    omesh = oracle.Mesh(nx, nx, N, oracle.GAUSS_LOBATTO, boundary_flag=oracle.DIRICHLET)
    k, f, source = W.helmholtz(omesh, N, seed=3)
    P = oracle.CGProblem(onod, omesh, k, lam=0.1)
    oracle.set_threads(os.cpu_count())
    t0 = time.perf_counter()
    osol, oerr, oit, _ = P.solve_pcg(source, maxIters=20000, tol=1e-10, precond=1)
    t_cpu = time.perf_counter() - t0
    nod = sg.NodalStorage_2D(N, nat.GAUSS_LOBATTO, nat.CG)
    mesh = sg.QuadMesh(nx, nx, N, nat.GAUSS_LOBATTO, boundary_flag=nat.DIRICHLET)
    cg = sg.CGsemElliptic_2D(ctx, nod, mesh, k, lam=0.1)
    res = {"workload": f"CGSEM Helmholtz {nx}x{nx} N={N} GLL, {mesh.nEl * (N + 1) ** 2} local nodes, PCG-Jacobi",
           "oracle": {"seconds": t_cpu, "solves_per_s": 1.0 / t_cpu, "iterations": oit, "ioerr": oerr,
                      "cores": os.cpu_count()}}
    for prec in ("fp64", "fp32"):
        cg.Solve(source, method="pcg", precision=prec, tolerance=1e-10, maxIters=100)
        ctx.synchronize()
        t0 = time.perf_counter()
        sol, rep = cg.Solve(source, method="pcg", precision=prec, tolerance=1e-10, maxIters=20000)
        el = time.perf_counter() - t0
        res["gpu_" + prec] = {"seconds": el, "solves_per_s": 1.0 / el, "iterations": rep["iterations"],
                              "rel_residual": rep["rel_residual"], "ioerr": rep["ioerr"],
                              "max_rel_diff_vs_oracle": float(np.abs(sol - osol).max() / np.abs(osol).max()),
                              "speedup_vs_oracle": t_cpu / el}
    cg.Trash()
    return res


def batched_leg(sg, ctx, nprob=512, fp64_sample=32):
    """512 uneven Helmholtz problems (n x n, n in [8, 64], N in {3..9}, own k and f): one batched FP32-inner /
    FP64-refined solve of all of them (autotuned tiles) vs plain FP64 one-solve-per-launch (sampled)."""
    from self_gb300 import workloads as W
    specs = W.batched_specs(nprob)
    t0 = time.perf_counter()
    probs = [W.batched_problem(sg, nx, N, seed) for nx, N, seed in specs]
    setup = time.perf_counter() - t0
    B = sg.CGBatch(ctx, probs)
    tune = B.autotune(os.path.join(ROOT, "self_gb300", "_build", "cgbatch_tuning_lines.json"))  # line-form FP32 tiles
    B.Solve(precision="fp32", tolerance=1e-10, maxIters=64)  # warm-up: graphs
    ctx.synchronize()
    t0 = time.perf_counter()
    reps = B.Solve(precision="fp32", tolerance=1e-10)
    el32 = time.perf_counter() - t0
    ok = sum(1 for r in reps if r["ioerr"] == 0 and r["rel_residual"] < 1e-10)
    t0 = time.perf_counter()
    reps64 = B.Solve(precision="fp64", tolerance=1e-10)
    el64b = time.perf_counter() - t0
    B.Trash()
    idx = np.linspace(0, nprob - 1, min(fp64_sample, nprob)).astype(int)
    t_single = 0.0
    for i in idx:
        pr = probs[i]
        cg = sg.CGsemElliptic_2D(ctx, pr["nodal"], pr["mesh"], pr["k"], lam=pr["lam"])
        t0 = time.perf_counter()
        cg.Solve(pr["source"], method="pcg", precision="fp64", tolerance=1e-10)
        t_single += time.perf_counter() - t0
        cg.Trash()
    single_rate = len(idx) / t_single
    nl = [pr["mesh"].nEl * (pr["nodal"].N + 1) ** 2 for pr in probs]
    nodes = sum(nl)
    # streamed bytes of the inner iterations: per node and FP32 iteration 44 B in the apply (w, v own and gathered,
    # v written, 4 factors, z written, src) + 32 B in the update (u, r read + write, v, z, 1/diag read, w written)
    node_its = sum(int(r["iterations"]) * n for r, n in zip(reps, nl))
    peak, peak_src = _peaks()
    gbs = node_its * 76.0 / el32 / 1e9
    return {"problems": nprob, "local_nodes": int(nodes), "host_setup_s": setup,
            "fp32_ir_batched": {"seconds": el32, "solves_per_s": nprob / el32, "converged": ok,
                                "max_rel_residual": max(r["rel_residual"] for r in reps),
                                "inner_node_iterations": node_its,
                                "streamed": {"bytes_per_node_iteration": 76, "achieved_gbs": gbs, "peak_gbs": peak,
                                             "frac": gbs / peak, "peak_source": peak_src,
                                             "note": "whole leg incl. outer FP64 residuals and scalar steps"}},
            "fp64_batched": {"seconds": el64b, "solves_per_s": nprob / el64b},
            "fp64_one_solve_per_launch": {"solves_per_s": single_rate, "sampled_problems": int(len(idx))},
            "speedup_vs_fp64_single": (nprob / el32) / single_rate,
            "autotuned_elements_per_tile": {f"N{N}_b{b}": e for (N, b), e in tune.items()}}


def serving_leg(sg, ctx, nreq=300, rate=2000.0, seed=5, sweep_n=150, base_n=120):
    """Poisson streams (seeded) mixing 70 % Helmholtz solves from the batched distribution and 30 % shallow-water
    ensemble members (64x64, N=5, 100 steps), served by the library's request loop (self_serve_*): continuous
    batching (FP32 inner + FP64 refinement, FP32 members) at the configured 2000 req/s and at 25 / 50 / 75 % of the
    capacity it measured there; the plain FP64 path one request at a time (the same loop with max_active = 1 and
    FP64 solves and members), run on the same 2000 req/s stream and at half its own capacity."""
    from self_gb300 import serving as S

    def serve(n, r, precision, max_active=0, seed_=seed):
        reqs = S.make_requests(sg, n, rate=r, seed=seed_)
        srv = S.Server(ctx, precision=precision, max_active=max_active)
        srv.keep_results = False
        srv.run(reqs)
        st = S.latency_stats(reqs)
        st["offered_req_s"] = r
        st["requests"] = n
        return st

    out = {"requests": nreq, "rate_req_s": rate, "loop": "self_serve (C++ worker thread, device-side tick decisions)"}
    mix = serve(nreq, rate, "fp32")
    out["continuous_batching"] = mix
    cap = mix["throughput_req_s"]
    fracs = (0.25, 0.5, 0.75)
    out["load_sweep"] = [serve(sweep_n, f * cap, "fp32", seed_=seed + 10 + i) for i, f in enumerate(fracs)]
    for row, f in zip(out["load_sweep"], fracs):
        row["fraction_of_capacity"] = f
    base = serve(base_n, rate, "fp64", max_active=1)
    out["fp64_one_at_a_time"] = base
    out["fp64_one_at_a_time_half_load"] = serve(base_n // 2, 0.5 * base["throughput_req_s"], "fp64", max_active=1,
                                                seed_=seed + 20)
    out["fp64_one_at_a_time_half_load"]["fraction_of_capacity"] = 0.5
    out["throughput_ratio"] = cap / base["throughput_req_s"]
    return out


def run_cg_profile(args):
    """Bounded CGSEM workload for profilers (no JSON line; the solves looped from the host so that every kernel
    launch is listed): the 256x256 N=7 Helmholtz problem of the elliptic leg, `--profile-cg K` PCG iterations (`--profile-method`: pcg = Jacobi, pcg_linear = the linear-FEM
    preconditioner with 20 inner iterations; `--profile-precision`) after a short warm-up solve; gmres = K FP64
    GMRES(30) Arnoldi steps on the advection-diffusion operator of the leg."""
    import self_gb300 as sg
    from self_gb300 import _native as nat
    from self_gb300 import workloads as W
    ctx = sg.Context(0)
    ctx.host_loop()  # every PCG launch visible to kernel profilers (no conditional graph nodes)
    N, nx = 7, 256
    nod = sg.NodalStorage_2D(N, nat.GAUSS_LOBATTO, nat.CG)
    mesh = sg.QuadMesh(nx, nx, N, nat.GAUSS_LOBATTO, boundary_flag=nat.DIRICHLET)
    k, f, source = W.helmholtz(mesh, N, seed=3)
    method, prec = args.profile_method, args.profile_precision
    if method == "gmres":  # the GMRES(30) operator of the elliptic leg, FP64, K Arnoldi steps
        ad = sg.CGsemElliptic_2D(ctx, nod, mesh, np.full_like(k, 1e-3), lam=0.0, op=1, vel=(1.0, 0.5))
        ad.Solve(source, method="gmres", m=30, tolerance=1e-10, maxIters=30)
        ctx.synchronize()
        t0 = time.perf_counter()
        _, rep = ad.Solve(source, method="gmres", m=30, tolerance=1e-30, maxIters=args.profile_cg)
        el = time.perf_counter() - t0
        print(f"profile-cg: {rep['iterations']} FP64 gmres Arnoldi steps in {el:.4f} s", flush=True)
        ad.Trash()
        ctx.close()
        return
    cg = sg.CGsemElliptic_2D(ctx, nod, mesh, k, lam=0.1)
    warm = 32 if method == "pcg" else 4
    cg.Solve(source, method=method, precision=prec, tolerance=1e-10, maxIters=warm, pc_iterations=20,
             tensor_cores=args.profile_tc, inner_layout=args.profile_layout)
    ctx.synchronize()
    t0 = time.perf_counter()
    _, rep = cg.Solve(source, method=method, precision=prec, tolerance=1e-30, maxIters=args.profile_cg, max_outer=1,
                      pc_iterations=20, pc_tolerance=0.0, tensor_cores=args.profile_tc,
                      inner_layout=args.profile_layout)
    el = time.perf_counter() - t0
    print(f"profile-cg: {rep['iterations']} {prec.upper()} {method} iterations in {el:.4f} s", flush=True)
    cg.Trash()
    ctx.close()


def run_gpu(args):
    dist, rank, ws, local = dist_init()
    import ctypes as C

    import self_gb300 as sg
    from self_gb300 import _native as nat

    head = nat.PREC_FP32 if args.precision == "fp32" else nat.PREC_FP64
    other = nat.PREC_FP64 if head == nat.PREC_FP32 else nat.PREC_FP32
    nod, mesh, q, h, fcor, dhdx, dhdy, dt = build_problem(sg)
    ctx = sg.Context(local)
    L = nat.lib()
    n = N_POLY + 1
    dof = q.size
    forms = {}
    for prec in (nat.PREC_FP64, nat.PREC_FP32):
        sw = sg.ShallowWater(ctx, nod, mesh, h, fcor, dt, dhdx=dhdx, dhdy=dhdy, precision=prec)
        sw.SetSolution(q)
        forms[prec] = sw

    # accuracy of the FP32 form against FP64 on this workload (device-resident runs from the same state)
    acc_steps = args.accuracy_steps
    res = {}
    for prec, sw in forms.items():
        sw.ForwardStepRK3(0.0, acc_steps)
        res[prec] = sw.GetSolution().reshape(mesh.nEl, 3, -1)
        sw.SetSolution(q)
    H64, H32 = res[nat.PREC_FP64][:, 2], res[nat.PREC_FP32][:, 2]
    h_err = float(np.abs(H32 - H64).max() / np.abs(H64).max())
    eta_err = float(np.abs(H32 - H64).max() / np.abs(H64 - h.reshape(mesh.nEl, -1)).max())

    out = {}
    launches = 0
    ck = None
    for prec in (head, other):
        sw = forms[prec]
        for _ in range(args.warmup):
            sw.ForwardStepRK3(0.0, 1)
        ctx.synchronize()
        if dist:
            dist.barrier()
        if prec == head:
            clocks = Clocks(local)
            clocks.start()
            l0 = ctx.kernel_launches()
        total = _time_steps(nat, L, ctx, sw, args.steps)
        if prec == head:
            launches = ctx.kernel_launches() - l0
            ck = clocks.stop()
        total = allmax(dist, total)
        e_ms, v_ms = _kernel_ms(nat, L, ctx, sw)
        out[prec] = {"ms": total / args.steps, "value": ws * dof * args.steps / (total * 1e-3),
                     "edge_ms": e_ms, "volume_ms": v_ms}

    hbm_peak, hbm_src = _peaks()
    f64peak = C.c_double()
    nat.check(L.self_probe_fma_peak(ctx.ptr, 1, C.byref(f64peak)), ctx.ptr)
    nEl = mesh.nEl

    def roof_fp64():
        """FP64 drop-in: one RK stage (dg_edge_flux + dg_volume, both bound by the FP64 pipe).  Average stage
        duration over the timed region = timed step / 3; the HBM fraction of the same stage beside it."""
        o = out[nat.PREC_FP64]
        stage_ms = o["ms"] / 3.0
        fl = FLOPS_PER_EL_STAGE_N7 * nEl
        ach = fl / (stage_ms * 1e-3) / 1e12
        hb = BYTES_FP64_PER_EL_STAGE_N7 * nEl
        hbm_ach = hb / (stage_ms * 1e-3) / 1e9
        vol_fl = FLOPS_VOLUME_PER_EL_N7 * nEl
        return {"bound": "fp64", "achieved": ach, "peak": f64peak.value, "unit": "TFLOP/s",
                "frac": ach / f64peak.value, "traffic": NCU_TRAFFIC_BYTES["dg_volume"],
                "traffic_kernel": "dg_volume", "traffic_unit": "B per launch",
                "traffic_source": "ncu --set full capture of one dg_volume launch on this workload",
                "kernel": "one RK stage: dg_edge_flux (LLF edge fluxes) + dg_volume (volume + RK update + traces)",
                "flops_per_element_stage": FLOPS_PER_EL_STAGE_N7, "flops_per_launch": fl,
                "launch_ms": stage_ms, "launch_ms_source": "timed step / 3 stages (CUDA events, L2 flushed per step)",
                "peak_source": "FP64 FMA rate measured on this GPU in this run (self_probe_fma_peak), of measured",
                "hbm": {"achieved": hbm_ach, "peak": hbm_peak, "unit": "GB/s", "frac": hbm_ach / hbm_peak,
                        "bytes_per_stage": hb, "peak_source": hbm_src},
                "kernels_alone": {"dg_volume_ms": o["volume_ms"], "dg_edge_flux_ms": o["edge_ms"],
                                  "dg_volume_fp64_frac": vol_fl / (o["volume_ms"] * 1e-3) / 1e12 / f64peak.value,
                                  "note": "each kernel timed alone after a 512 MiB L2 flush"}}

    def roof_fp32():
        """FP32 form: algorithmic bytes of the step's three fused stages (stage 1 reads no G) / timed step time."""
        o = out[nat.PREC_FP32]
        fused = o["edge_ms"] == 0.0
        step_b = bytes_per_fused_step(nEl, n)
        ach = step_b / (o["ms"] * 1e-3) / 1e9
        cold_b = bytes_per_fused_stage(nEl, n, 2)
        cold = cold_b / (o["volume_ms"] * 1e-3) / 1e9
        return {"bound": "hbm", "achieved": ach, "peak": hbm_peak, "unit": "GB/s", "frac": ach / hbm_peak,
                "traffic": NCU_TRAFFIC_BYTES["sw32_fused"] if fused else None, "traffic_unit": "B per launch",
                "traffic_source": "ncu --set full capture of one cold sw32_fused launch on this workload",
                "kernel": ("sw32_fused (TMA-staged edge fluxes + volume + RK update + traces), 3 launches per step"
                           if fused else "edge32 + volume32"),
                "bytes_per_step": step_b, "bytes_per_stage": {"stage1": bytes_per_fused_stage(nEl, n, 1),
                                                              "stages2_3": cold_b},
                "launch_ms": o["ms"] / 3.0, "launch_ms_source": "timed step / 3 launches",
                "peak_source": hbm_src,
                "cold_launch": {"launch_ms": o["volume_ms"], "achieved": cold, "frac": cold / hbm_peak,
                                "note": "one stage-2 launch alone after a 512 MiB L2 flush (no reuse between stages)"}}

    e2e_steps = max(3, min(args.steps, 50))
    t_e2e, nbytes, e2e_parts = _e2e(nat, L, ctx, forms[head], dof, e2e_steps, dist)
    t_e2e = allmax(dist, t_e2e)
    t_e2e_o, _, e2e_parts_o = _e2e(nat, L, ctx, forms[other], dof, e2e_steps, dist)
    t_e2e_o = allmax(dist, t_e2e_o)

    cpu = None
    if rank == 0 and not args.no_cpu:
        from oracle import oracle as O
        O.build()
        cpu = cpu_baseline(O, nod, mesh, q, h, fcor, dhdx, dhdy, dt)

    for sw in forms.values():
        sw.Trash()
    forms = {}
    elliptic = batched = serving = None
    if args.elliptic:
        elliptic, eprob = elliptic_leg(sg, ctx)
        if rank == 0 and not args.no_cpu:
            from oracle import oracle as O
            elliptic["cpu_baseline_pcg_fp64"] = elliptic_cpu(O, *eprob, elliptic["pcg_fp64"]["iterations"])
            elliptic["measured_64x64"] = elliptic_small_measured(sg, ctx, O)
    if args.batched_n > 0:
        batched = batched_leg(sg, ctx, nprob=args.batched_n)
    if args.serve_n > 0:
        serving = serving_leg(sg, ctx, nreq=args.serve_n)

    if rank == 0:
        r64, r32 = roof_fp64(), roof_fp32()
        o32 = out[nat.PREC_FP32]
        e2e_head = {"value": ws * dof * e2e_steps / (t_e2e * 1e-3), "unit": "DOF-updates/s",
                    "h2d_bytes_per_step": nbytes, "d2h_bytes_per_step": nbytes, "steps": e2e_steps,
                    "calls": "self_dg2d_set_state + self_dg2d_rk3 + self_dg2d_get_state (pinned FP64 host state)",
                    "per_call": e2e_parts}
        e2e_other = {"value": ws * dof * e2e_steps / (t_e2e_o * 1e-3), "unit": "DOF-updates/s",
                     "h2d_bytes_per_step": nbytes, "d2h_bytes_per_step": nbytes, "steps": e2e_steps,
                     "per_call": e2e_parts_o}
        form_names = {nat.PREC_FP64: "plain FP64 drop-in", nat.PREC_FP32: "FP32 perturbation form about the lake at rest"}
        fp32_obj = {"value": o32["value"], "ms_per_step": o32["ms"], "volume_ms": o32["volume_ms"],
                    "edge_ms": o32["edge_ms"], "roofline": r32,
                    "e2e": e2e_other if head == nat.PREC_FP64 else e2e_head,
                    "accuracy": {"steps": acc_steps, "height_rel_err_fp32_vs_fp64": h_err,
                                 "height_err_rel_to_max_eta": eta_err, "tolerance": 1e-6}}
        line = {
            "metric": "DG DOF-updates/s", "value": out[head]["value"], "unit": "DOF-updates/s", "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": out[head]["ms"], "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32" if head == nat.PREC_FP32 else "f64",
            "data": "synthetic (seeded; shapes of the shallow-water configuration)",
            "config": {"workload": WORKLOAD, "precision_form": form_names[head],
                       "l2": "flushed (512 MiB write) between timed steps", "parallelism": f"replicas x{ws}"},
            "gpu_launches": int(launches),
            "roofline": r64 if head == nat.PREC_FP64 else r32,
            "e2e": e2e_head,
            "cpu_baseline": cpu,
            "clocks": ck,
            "fp32_form": fp32_obj,
            "fp64_plain": {"value": out[nat.PREC_FP64]["value"], "ms_per_step": out[nat.PREC_FP64]["ms"],
                           "roofline": r64} if head == nat.PREC_FP32 else None,
            "elliptic": elliptic,
            "batched": batched,
            "serving": serving,
        }
        print(json.dumps(line), flush=True)
    ctx.close()
    if dist:
        dist.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gpu", choices=["gpu", "reference"])
    ap.add_argument("--precision", default="fp64", choices=["fp64", "fp32"], help="form of the headline value")
    ap.add_argument("--accuracy-steps", type=int, default=1000, help="FP32-vs-FP64 height check length")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--no-elliptic", dest="elliptic", action="store_false", help="skip the CGSEM solve leg")
    ap.add_argument("--batched-n", type=int, default=512, help="problems of the batched leg (0 skips it)")
    ap.add_argument("--serve-n", type=int, default=300, help="requests of the serving leg (0 skips it)")
    ap.add_argument("--profile-cg", type=int, default=0,
                    help="run only K PCG iterations of the elliptic workload (for profilers) and exit")
    ap.add_argument("--profile-method", default="pcg", choices=["pcg", "pcg_linear", "gmres"])
    ap.add_argument("--profile-precision", default="fp32", choices=["fp32", "fp64"])
    ap.add_argument("--profile-tc", action="store_true", help="FP32 profile run with the tensor-core operator")
    ap.add_argument("--profile-layout", default="compact", choices=["compact", "local"],
                    help="FP32 inner vectors of the profile run: compact (one value per unknown) or element-local")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    if args.profile_cg > 0:
        run_cg_profile(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
