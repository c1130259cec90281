"""Benchmark of the RHS hot path: Mpts*RKstages/s on the 512^3 Taylor-Green
vortex (ASTR main-solver ordering: compact 6th-order derivatives, 10th-order
compact filter, RK3, FP64).

One JSON line on rank 0.  A "step" is one RK3 time step (three stages) over
the whole 512^3 periodic box; value = unique points (512^3) * 3 stages *
steps / device time.  Inputs are resident in HBM (about 50 GB, far larger
than the 129 MB L2, so no flush is needed between steps).  e2e is the same
metric through the C ABI with host buffers: every step uploads the full
state from page-locked host memory, runs one RK3 step, and downloads q and
the statistics.

--impl reference times the CPU restatement of the reference (oracle/, a
C++ port of the Fortran routines; the Fortran itself cannot be built on
this image) on all host cores, on bounded 128^3 samples of the same case.

Multi-GPU: the path does not shard (single-rank numerics), so N GPUs run N
independent replicas ("scaling": "weak").
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

METRIC = "Mpts*RKstages/s (TGV 512^3, FP64)"
UNIT = "Mpts*stages/s"

# Algorithmic work of the FP64 form per interior point per launch, from the
# reference's arithmetic with diagonal metrics (Thomas: 3 flops forward +
# 2 backward per row; a divide or square root counts as one flop).
#   filter: RHS 17 + Thomas 5 per value, 5 variables
#   convgrad: fluxes 14, 5 derivatives (RHS 5 + Thomas 5) + accumulate 5,
#             4 gradients (10 + 1 metric multiply); the last direction adds
#             the viscous stress and heat flux (48)
#   visc: fluxes 8, 4 derivatives (40), accumulate 4; the last direction
#         adds the RK3 update (40) and primitive recovery (14)
FLOPS_PER_PT = {"filter": 110.0, "convgrad": 113.0, "convgrad_last": 161.0,
                "visc": 52.0, "visc_last": 106.0}
# Algorithmic DRAM bytes per interior point per launch (FP64 words * 8):
#   filter: q 5 in, 5 out; convgrad x: q, u, v, w, p, T, dxi, J in; qrhs 5 +
#   4 gradients out; y adds qrhs in; z adds 8 gradients in and sigma 6 +
#   heat flux 3 out; visc x/y: 3 sigma + 1 heat flux + dxi + J + 4 qrhs in,
#   4 out; visc z: 4 + dxi + J + qrhs 5 + qsave 5 + q 5 in, q 5 + 6
#   primitives out.
BYTES_PER_PT = {"filter": 80.0, "convgrad": (168.0 + 208.0 + 344.0) / 3.0,
                "visc": (112.0 + 112.0 + 256.0) / 3.0}


def env_int(name, default):
    try:
        return int(os.environ.get(name, default))
    except ValueError:
        return default


class ClockSampler:
    """nvidia-smi clocks and throttle reasons during the timed region."""
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index=0):
        self.gpu = gpu_index
        self.proc = None
        self.path = os.path.join(ROOT, "gpurun_out", f"clocks_bench_{os.getpid()}.csv")

    def start(self):
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=self.fh, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.fh.close()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            p = [x.strip() for x in line.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                mx.append(float(p[2]))
            except ValueError:
                continue
            for n, v in zip(names, p[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def dist_setup():
    world = env_int("WORLD_SIZE", 1)
    rank = env_int("RANK", 0)
    if world > 1:
        import torch
        import torch.distributed as dist
        local = env_int("LOCAL_RANK", 0)
        torch.cuda.set_device(local)
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group("nccl")
        return rank, world, dist
    return rank, world, None


def barrier(dist):
    if dist is not None:
        dist.barrier()


def max_over_ranks(dist, v):
    if dist is None:
        return v
    import torch
    t = torch.tensor([v], dtype=torch.float64, device="cuda")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def cpu_port_throughput(n, steps, threads=None):
    """The oracle (C++ port of the reference routines) on the host cores:
    Mpts*stages/s over `steps` RK3 steps of the n^3 TGV (main ordering)."""
    from oracle import pyoracle as po
    if threads:
        po.set_threads(threads)
    o = po.tgv_main(n)
    o.rk3_steps(1)  # warm-up
    t0 = time.perf_counter()
    o.rk3_steps(steps)
    dt = time.perf_counter() - t0
    return n ** 3 * 3 * steps / dt / 1e6, po.get_threads(), dt


def run_reference(args, rank, world, dist):
    if rank != 0:
        return 0
    n = 128
    from oracle import pyoracle as po
    threads = os.cpu_count()
    po.set_threads(threads)
    o = po.tgv_main(n)
    for _ in range(args.warmup):
        o.rk3_steps(1)
    t0 = time.perf_counter()
    o.rk3_steps(args.steps)
    dt = time.perf_counter() - t0
    v = n ** 3 * 3 * args.steps / dt / 1e6
    line = {
        "impl": "reference", "metric": METRIC, "value": round(v, 3), "unit": UNIT,
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(1e3 * dt / args.steps, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": "Taylor-Green vortex 512^3, main-solver RK3 stage order",
                   "sample": f"TGV {n}^3, one RK3 step per timed step"},
        "cpu_baseline": {"value": round(v, 3), "unit": UNIT, "cores": po.get_threads(),
                         "kind": "port",
                         "sample": f"C++ restatement of the reference routines, TGV {n}^3, "
                                   f"{args.steps} RK3 steps, 1 process, {po.get_threads()} OpenMP threads"},
        "e2e": {"value": round(v, 3), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def run_gpu(args, rank, world, dist):
    from astr_gb300 import capi, cases
    from astr_gb300.solver import GpuSolver

    n = args.n
    L = 2.0 * np.pi
    t0 = time.perf_counter()
    x, y, z = cases.gridcube(n, n, n, L, L, L)
    (d11, d22, d33), J = cases.rect_metrics(x, y, z, diag_only=True)
    st = cases.tgv_state(n, n, n, mach=0.1, x=x, y=y, z=z)
    t_setup = time.perf_counter() - t0

    g = GpuSolver(n, n, n, order=capi.ORDER_MAIN, precision=capi.FP64, mach=0.1,
                  reynolds=1600.0, deltat=1e-3)
    g.set_metrics_diag(d11, d22, d33, J)
    del d11, d22, d33
    g.upload_state(st["q"], st["rho"], st["vel"], st["prs"], st["tmp"])
    hist0 = g.time_integration_rk(1)  # includes kernel warm-up
    if args.warmup > 1:
        g.timed_steps(args.warmup - 1)

    clocks = ClockSampler(env_int("LOCAL_RANK", 0))
    clocks.start()
    barrier(dist)
    g.set_profiling(True)
    ms = g.timed_steps(args.steps)
    kt = g.kernel_times()
    g.set_profiling(False)
    barrier(dist)
    clk = clocks.stop()
    ms = max_over_ranks(dist, ms)
    pts = float(n) ** 3
    value = world * pts * 3 * args.steps / (ms / 1e3) / 1e6

    # roofline of the dominant kernel class
    I = n + 1
    pts_int = float(I) ** 3
    tf_peak = ctypes_peak()
    classes = {}
    for k in ("filter", "convgrad", "visc"):
        tms, cnt = kt[k]
        if cnt == 0:
            continue
        if k == "filter":
            flops = FLOPS_PER_PT["filter"] * pts_int * cnt
        elif k == "convgrad":
            per_stage = 2 * FLOPS_PER_PT["convgrad"] + FLOPS_PER_PT["convgrad_last"]
            flops = per_stage / 3.0 * pts_int * cnt
        else:
            per_stage = 2 * FLOPS_PER_PT["visc"] + FLOPS_PER_PT["visc_last"]
            flops = per_stage / 3.0 * pts_int * cnt
        nbytes = BYTES_PER_PT[k] * pts_int * cnt
        classes[k] = {"ms": tms, "launches": cnt, "avg_ms": tms / cnt,
                      "tflops": flops / (tms / 1e3) / 1e12, "gbs": nbytes / (tms / 1e3) / 1e9,
                      "flops_per_launch": flops / cnt, "bytes_per_launch": nbytes / cnt}
    dom = max(classes, key=lambda k: classes[k]["ms"])
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        pass
    hbm_peak = float(peaks.get("hbm_gbs", 6800.0))
    traffic = None
    try:
        prof = json.load(open(os.path.join(ROOT, "profiles", "ncu_traffic.json")))
        traffic = prof.get(dom, {}).get("bytes_per_launch_512")
    except Exception:
        pass
    dc = classes[dom]
    roofline = {
        "bound": "fp64",
        "kernel": dom,
        "achieved": round(dc["tflops"], 4),
        "peak": round(tf_peak, 4),
        "unit": "TFLOP/s",
        "frac": round(dc["tflops"] / tf_peak, 4),
        "peak_source": "FP64 FMA loop measured live in this run (astr_gpu_measure_fp64_peak)",
        "traffic": traffic,
        "hbm_achieved_gbs": round(dc["gbs"], 1),
        "hbm_frac_of_measured": round(dc["gbs"] / hbm_peak, 4),
        "classes": {k: {kk: (round(vv, 4) if isinstance(vv, float) else vv) for kk, vv in v.items()}
                    for k, v in classes.items()},
    }

    # end to end through the C ABI with page-locked host buffers
    pinned = {}
    for k in ("q", "rho", "vel", "prs", "tmp"):
        pa = capi.PinnedArray(st[k].shape)
        pa.array[...] = st[k]
        pinned[k] = pa
    qout = capi.PinnedArray(st["q"].shape)
    del st
    e2e_steps = max(1, min(args.steps, 3))
    barrier(dist)
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        g.upload_state(*(pinned[k].array for k in ("q", "rho", "vel", "prs", "tmp")))
        g.time_integration_rk(1)
        g._c(g.L.astr_gpu_download_state(g.h, capi.dptr(qout.array), None, None, None, None))
    t_e2e = time.perf_counter() - t0
    t_e2e = max_over_ranks(dist, t_e2e)
    h2d = sum(pinned[k].nbytes for k in pinned)
    d2h = qout.nbytes + 16
    e2e_value = world * pts * 3 * e2e_steps / t_e2e / 1e6
    for pa in list(pinned.values()) + [qout]:
        pa.free()
    launches_per_step = None
    g0 = g.launches
    g.timed_steps(1)
    launches_per_step = g.launches - g0
    g.close()

    cpu = None
    if rank == 0 and not args.no_cpu:
        v, cores, dt = cpu_port_throughput(128, 4, threads=os.cpu_count())
        cpu = {"value": round(v, 3), "unit": UNIT, "cores": cores, "kind": "port",
               "sample": f"C++ restatement of the reference routines (oracle/), TGV 128^3 "
                         f"main-solver ordering, 4 RK3 steps in {dt:.1f} s, {cores} OpenMP threads"}
    if rank == 0:
        line = {
            "metric": METRIC, "value": round(value, 3), "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": round(ms / args.steps, 3), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": f"Taylor-Green vortex {n}^3 ({n + 1}^3 stored nodes), Re 1600, "
                                   "Mach 0.1, 643c compact scheme + compact filter alpha 0.49, "
                                   "RK3 dt 1e-3, main-solver stage order",
                       "form": "plain FP64", "parallelism": f"replicas x{world}",
                       "l2": "inputs resident in HBM (~50 GB) >> 129 MB L2, no flush",
                       "setup_s": round(t_setup, 1)},
            "gpu_launches": launches_per_step * args.steps,
            "roofline": roofline,
            "e2e": {"value": round(e2e_value, 3), "unit": UNIT, "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h, "steps": e2e_steps},
            "cpu_baseline": cpu,
            "clocks": clk,
            "stats_first_step": {"kenergy": float(hist0[0, 0]), "enstrophy": float(hist0[0, 1])},
        }
        print(json.dumps(line), flush=True)
    return 0


def ctypes_peak():
    import ctypes
    from astr_gb300 import capi
    L = capi.load()
    v = ctypes.c_double()
    rc = L.astr_gpu_measure_fp64_peak(ctypes.byref(v))
    return v.value if rc == 0 else float("nan")


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--n", type=int, default=512)
    ap.add_argument("--no-cpu", action="store_true")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    rank, world, dist = dist_setup()
    if args.impl == "reference":
        return run_reference(args, rank, world, dist)
    return run_gpu(args, rank, world, dist)


if __name__ == "__main__":
    sys.exit(main())
