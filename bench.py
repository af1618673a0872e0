#!/usr/bin/env python3
"""Benchmark of the DGSEM 2-D shallow-water step (LSRK3) on one GB300 per rank.

Workload (the configuration the DG metric is quoted on): conservative shallow water on [0, 2e6 m]^2,
128 x 128 curvilinear quads (x,y += 0.05 L sin(2 pi x/L) sin(2 pi y/L)), N = 7 Legendre-Gauss nodes,
3 variables = 3,145,728 DOF, beta-plane, seamount bathymetry, 16 seeded Gaussian bumps, mirror walls.
A step is one LSRK3 step (3 stages x {edge-flux kernel, volume+update kernel}).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gpu|reference] [--precision fp64|fp32]

value      DOF-updates/s of the device-resident step (inputs in HBM, L2 flushed between timed steps),
           whole job (sum over ranks; ranks are independent replicas).
e2e        the same metric through the C ABI with host (pinned) buffers: every step uploads the state,
           advances one step and downloads the state, copies inside the timed region.
roofline   dominant kernel (volume + RK update): algorithmic bytes per launch / CUDA-event launch time.
cpu_baseline  the CPU oracle (C++ restatement of the reference's Fortran, OpenMP) on a bounded sample.
--impl reference  times the oracle alone on the host cores (the reference itself is Fortran with no compiler
           on this image; the oracle is its restatement).
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


def bytes_per_volume_launch(nEl, n, prec_bytes):
    """Algorithmic HBM bytes of one volume + RK-update launch: q r/w, G r/w, 5 metric fields, 3 aux fields
    (dhdx, dhdy, f), boundary fluxes read and new traces written (4 sides x n x 3 vars each)."""
    nn = n * n
    per_el = prec_bytes * (4 * 3 * nn + 5 * nn + 3 * nn + 2 * 4 * n * 3)
    return per_el * nEl


def cpu_baseline(oracle, nod, mesh, q, h, fcor, dhdx, dhdy, dt, budget_s=15.0, max_steps=20):
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


def run_reference(args):
    dist, rank, ws, local = dist_init()
    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return
    from oracle import oracle as O
    import self_gb300 as sg
    O.build()
    nod, mesh, q, h, fcor, dhdx, dhdy, dt = build_problem(sg)
    cores = os.cpu_count()
    O.set_threads(cores)
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
            "config": {"workload": "DGSEM 2D conservative shallow water 128x128 curvilinear, N=7 LG, 3,145,728 DOF, "
                                   "LSRK3", "parallelism": "host threads"},
            "cpu_baseline": {"value": val, "unit": "DOF-updates/s", "cores": cores, "kind": "port",
                             "sample": f"{args.steps} full LSRK3 steps after {args.warmup} warm-up steps"},
            "e2e": {"value": val, "unit": "DOF-updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


def run_gpu(args):
    dist, rank, ws, local = dist_init()
    import ctypes as C

    import self_gb300 as sg
    from self_gb300 import _native as nat

    prec = nat.PREC_FP32 if args.precision == "fp32" else nat.PREC_FP64
    nod, mesh, q, h, fcor, dhdx, dhdy, dt = build_problem(sg)
    ctx = sg.Context(local)
    sw = sg.ShallowWater(ctx, nod, mesh, h, fcor, dt, dhdx=dhdx, dhdy=dhdy, precision=prec)
    sw.SetSolution(q)
    L = nat.lib()
    n = N_POLY + 1
    dof = q.size

    for _ in range(args.warmup):
        sw.ForwardStepRK3(0.0, 1)
    ctx.synchronize()
    if dist:
        dist.barrier()
    clocks = Clocks(local)
    clocks.start()
    launches0 = ctx.kernel_launches()
    total_ms = 0.0
    ms = C.c_double()
    for _ in range(args.steps):
        nat.check(L.self_ctx_flush_l2(ctx.ptr, C.c_size_t(L2_FLUSH_BYTES)), ctx.ptr)
        nat.check(L.self_ctx_timer_start(ctx.ptr), ctx.ptr)
        sw.ForwardStepRK3_async(0.0, 1)
        nat.check(L.self_ctx_timer_stop(ctx.ptr, C.byref(ms)), ctx.ptr)
        total_ms += ms.value
    launches = ctx.kernel_launches() - launches0
    ck = clocks.stop()
    total_ms = allmax(dist, total_ms)
    ms_step = total_ms / args.steps
    value = ws * dof * args.steps / (total_ms * 1e-3)

    # dominant kernel: volume + RK update, CUDA events around single launches (L2 flushed before each)
    kms = (C.c_double * 2)()
    nat.check(L.self_dg2d_time_kernels(sw.ptr, 20, C.c_size_t(L2_FLUSH_BYTES), kms), ctx.ptr)
    pb = 8 if prec == nat.PREC_FP64 else 4
    vbytes = bytes_per_volume_launch(mesh.nEl, n, pb)
    achieved = vbytes / (kms[1] * 1e-3) / 1e9
    peak, peak_kind = _peaks()

    # end to end through the C ABI with pinned host buffers
    nbytes = dof * 8
    hp = C.c_void_p()
    nat.check(L.self_host_alloc(C.c_size_t(nbytes), C.byref(hp)))
    hq = np.ctypeslib.as_array((C.c_double * dof).from_address(hp.value))
    hq[:] = sw.GetSolution()
    e2e_steps = max(3, min(args.steps, 50))
    if dist:
        dist.barrier()
    t_e2e = 0.0
    for _ in range(e2e_steps):
        nat.check(L.self_ctx_timer_start(ctx.ptr), ctx.ptr)
        nat.check(L.self_dg2d_set_state(sw.ptr, hq.ctypes.data_as(nat.dp)), ctx.ptr)
        nat.check(L.self_dg2d_rk3(sw.ptr, C.c_double(0.0), 1), ctx.ptr)
        nat.check(L.self_dg2d_get_state(sw.ptr, hq.ctypes.data_as(nat.dp)), ctx.ptr)
        nat.check(L.self_ctx_timer_stop(ctx.ptr, C.byref(ms)), ctx.ptr)
        t_e2e += ms.value
    t_e2e = allmax(dist, t_e2e)
    e2e_value = ws * dof * e2e_steps / (t_e2e * 1e-3)
    L.self_host_free(hp)

    cpu = None
    if rank == 0 and not args.no_cpu:
        from oracle import oracle as O
        O.build()
        cpu = cpu_baseline(O, nod, mesh, q, h, fcor, dhdx, dhdy, dt)

    if rank == 0:
        line = {
            "metric": "DG DOF-updates/s", "value": value, "unit": "DOF-updates/s", "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64" if prec == nat.PREC_FP64 else "f32",
            "data": "synthetic (seeded; shapes of the shallow-water configuration)",
            "config": {"workload": "DGSEM 2D conservative shallow water, 128x128 curvilinear quads, N=7 Legendre-Gauss,"
                                   " 3 vars = 3,145,728 DOF, one LSRK3 step",
                       "precision_form": "plain FP64 drop-in" if prec == nat.PREC_FP64 else "FP32 perturbation form",
                       "l2": "flushed (512 MiB write) between timed steps", "parallelism": f"replicas x{ws}"},
            "gpu_launches": int(launches),
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                         "traffic": None, "kernel": "dg_volume (volume + RK update + traces)",
                         "launch_ms": kms[1], "bytes_per_launch": vbytes, "peak_source": peak_kind,
                         "edge_kernel_ms": kms[0]},
            "e2e": {"value": e2e_value, "unit": "DOF-updates/s", "h2d_bytes_per_step": nbytes,
                    "d2h_bytes_per_step": nbytes, "steps": e2e_steps},
            "cpu_baseline": cpu,
            "clocks": ck,
        }
        print(json.dumps(line), flush=True)
    sw.Trash()
    ctx.close()
    if dist:
        dist.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gpu", choices=["gpu", "reference"])
    ap.add_argument("--precision", default="fp64", choices=["fp64", "fp32"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
