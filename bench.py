"""Benchmark of the RHS hot path: Mpts*RKstages/s on the 512^3 Taylor-Green
vortex (ASTR main-solver ordering: compact 6th-order derivatives, 10th-order
compact filter, RK3), FP32-storage form against the plain FP64 form, at the
measured error of the FP32-storage form.

One JSON line on rank 0.  A "step" is one RK3 time step (three stages) over
the whole 512^3 periodic box; value = unique points (512^3) * 3 stages *
steps / device time of the FP32-storage form (fields stored and swept in
FP32, RK3 base and master conserved state in FP64).  The plain FP64 form
runs the same steps from the same initial state; "forms" carries both
throughputs and "error_vs_fp64" the relative L2 / Linf difference of the
two final states.  Inputs are resident in HBM (about 37 GB / 50 GB, far
larger than the 129 MB L2, so no flush is needed between steps).  e2e is
the headline form through the C ABI with host buffers: every step uploads
the FP64 state q from page-locked host memory (the primitives are derived
from it on the device), runs one RK3 step, and downloads q and the
statistics.

The line also carries "serve": the first --serve-cases (100) requests of a
seeded Poisson stream of independent cases served through the batch kernels
and through per-case streams (time-to-solution p50/p99, cases/s);
--no-serve leaves it out, and --case serve runs that stream through the
arms of --serve-arms (default: batch kernels, per-case streams, sequential
FP64) instead.

--impl reference times the CPU restatement of the reference (oracle/, a
C++ port of the Fortran routines; the Fortran itself cannot be built on
this image) on all host cores, on bounded 128^3 samples of the same case.

--history N instead runs both forms N steps with the kinetic-energy and
enstrophy history sampled every step and prints their largest relative
difference and the final-state error (the 200-step scale comparison).

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
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

METRIC = "Mpts*RKstages/s (TGV 512^3, FP32 storage / FP64 accumulate, at stated error vs FP64)"
UNIT = "Mpts*stages/s"

# Algorithmic work per interior point per launch, from the reference's
# arithmetic with diagonal metrics (Thomas: 3 flops forward + 2 backward per
# row; a divide or square root counts as one flop).
#   filter: RHS 17 + Thomas 5 per value, 5 variables
#   convgrad: fluxes 14, 5 derivatives (RHS 5 + Thomas 5) + accumulate 5,
#             4 gradients (10 + 1 metric multiply)
#   point (k_sigma): viscous stress and heat flux at every point (48)
#   visc: fluxes 8, 4 derivatives (40), accumulate 4; the last direction
#         adds the RK3 update (40) and primitive recovery (14)
FLOPS_PER_PT = {"filter": 110.0, "convgrad": 113.0, "pointwise": 48.0,
                "visc": 52.0, "visc_last": 106.0}


def bytes_per_pt(kind, d, stage1, f32, tiled=False):
    """Algorithmic DRAM bytes per interior point of one launch: every array
    element the kernel must read or write once.  w = storage word (8 or 4);
    m = FP64 word of the RK3 base, the FP32 form's master state and 1/J.
      filter: q 5 in, 5 out (FP32 form: + master 5 in, 5 out)
      convgrad x: q 5, u v w p T, dxi, J in; qrhs 5 + 4 gradients out;
        stage 1 adds the RK3 base: qsave 5 out (FP32 form: + master 5 and an
        FP64 J in); y and z add qrhs 5 in; stage 1 z adds rho and 6
        gradients in for the statistics
      pointwise (k_sigma): 12 gradients, T, u v w in; stress 6 + heat flux
        3 out
      visc x, y: stress 3 + heat flux 1, dxi, J, qrhs 4 in; qrhs 4 out
      visc z: stress/heat 4, dxi, J, qrhs 5, q 5 in, qsave 5 and 1/J (FP64)
        in; q 5 + primitives 6 out (FP32 form: + FP64 J, master 5 in, 5 out)
    """
    w = 4.0 if f32 else 8.0
    m = 8.0
    if tiled:
        return tiled_bytes_per_pt(kind, d, f32)
    if kind == "filter":
        return 10 * w + (10 * m if f32 else 0.0)
    if kind == "convgrad":
        b = [21 * w, 26 * w, 26 * w][d]
        if stage1 and d == 0:
            b += 5 * m + (6 * m if f32 else 0.0)
        if stage1 and d == 2:
            b += 7 * w
        return b
    if kind == "pointwise":
        return 25 * w
    if kind == "visc":
        if d < 2:
            return 14 * w
        # the FP64 form's J is the array the fluxes read; the FP32 form reads
        # an FP64 copy of J beside its FP32 one
        return (4 + 1 + 1 + 5 + 5 + 5 + 6) * w + 6 * m + (11 * m if f32 else 0.0)
    raise ValueError(kind)


def tiled_bytes_per_pt(kind, d, f32):
    """The same count for the tile-staged sweeps, which leave the RK3 base,
    the stress and the RK3 update to point kernels.
      filter: as above
      convgrad x: q 5, u v w p T, dxi, J in; qrhs 5 + 4 gradients out; y, z
        add qrhs 5 in
      visc (every direction): stress 3 + heat flux 1, dxi, J, qrhs 4 in;
        qrhs 4 out
      pointwise, per step: 3 stress launches (12 gradients, T, u v w in;
        stress 6 + heat flux 3 out), 3 RK3 updates (qrhs 5, qsave 5 (FP64),
        q or the FP64 master 5, J and 1/J (FP64) in; q 5 (+ master 5) and the
        primitives 6 out) and 1 RK3 base (q or master 5, J in; qsave 5 out),
        averaged over the 7 launches"""
    w = 4.0 if f32 else 8.0
    m = 8.0
    if kind == "filter":
        return 10 * w + (10 * m if f32 else 0.0)
    if kind == "convgrad":
        return 21 * w if d == 0 else 26 * w
    if kind == "visc":
        return 14 * w
    if kind == "pointwise":
        sig = 25 * w
        if f32:
            rk = 5 * w + 5 * m + 5 * m + 2 * m + 5 * w + 5 * m + 6 * w
        else:
            rk = 5 * w + 5 * m + 5 * w + 2 * m + 5 * w + 6 * w
        base = 5 * m + m + 5 * m
        return (3 * sig + 3 * rk + base) / 7.0
    raise ValueError(kind)


# Algorithmic bytes per unique point and RK3 stage of the pass model
# (P1) of the scope table: s = stream word (4 or 8), S = 8 (FP64 master and
# RK3 base).  Per launch of a class: filter 10 s (three directions of 30 s);
# convective + gradient sweeps (A + B + C) / 3 = (14 + 19 + 32) s / 3;
# viscous sweeps (D + E + F) / 3 = ((12 + 12 + 17.33) s + 6.67 S) / 3.
def p1_bytes_per_launch(kind, f32):
    s = 4.0 if f32 else 8.0
    S = 8.0
    if kind == "filter":
        return 10.0 * s
    if kind == "convgrad":
        return (14.0 + 19.0 + 32.0) * s / 3.0
    if kind == "visc":
        return ((12.0 + 12.0 + 17.0 + 1.0 / 3.0) * s + (6.0 + 2.0 / 3.0) * S) / 3.0
    return None


def class_work(kind, f32, launches, pts, tiled=False):
    """Algorithmic bytes and flops of `launches` launches of one kernel class
    over whole RK3 steps (per step: 3 stages x 3 directions, or 3 stages x 1
    point launch)."""
    if tiled:
        nb = tiled_bytes_per_pt(kind, 0, f32) if kind != "convgrad" else \
            (tiled_bytes_per_pt(kind, 0, f32) + 2 * tiled_bytes_per_pt(kind, 1, f32)) / 3.0
        fl = {"filter": FLOPS_PER_PT["filter"], "convgrad": FLOPS_PER_PT["convgrad"],
              "visc": FLOPS_PER_PT["visc"] + 0.0,
              "pointwise": (3 * FLOPS_PER_PT["pointwise"] + 3 * (FLOPS_PER_PT["visc_last"] -
                                                                  FLOPS_PER_PT["visc"]) + 5) / 7.0}[kind]
        return nb * pts * launches, fl * pts * launches
    dirs = (0,) if kind == "pointwise" else (0, 1, 2)
    per_step_b = sum(bytes_per_pt(kind, d, s == 0, f32) for s in range(3) for d in dirs)
    if kind == "visc":
        per_step_f = 3 * (2 * FLOPS_PER_PT["visc"] + FLOPS_PER_PT["visc_last"])
    else:
        per_step_f = 3 * len(dirs) * FLOPS_PER_PT[kind]
    n = 3 * len(dirs)
    return per_step_b / n * pts * launches, per_step_f / n * pts * launches


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
        self.path = os.path.join(tempfile.gettempdir(), f"astr_clocks_{os.getpid()}_{id(self)}.csv")

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


def dist_setup(backend=None):
    """One process per GPU (torchrun environment): the replicas only meet in
    barriers and in the max-over-ranks of the timings (no data-path
    collective).  backend defaults to NCCL; gloo serves CPU-only runs."""
    world = env_int("WORLD_SIZE", 1)
    rank = env_int("RANK", 0)
    if world > 1:
        import torch
        import torch.distributed as dist
        backend = backend or os.environ.get("ASTR_DIST_BACKEND", "nccl")
        if backend == "nccl":
            torch.cuda.set_device(env_int("LOCAL_RANK", 0))
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group(backend)
        return rank, world, dist
    return rank, world, None


def barrier(dist):
    if dist is not None:
        dist.barrier()


def max_over_ranks(dist, v):
    if dist is None:
        return v
    import torch
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([v], dtype=torch.float64, device=dev)
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


def mem_available_gb():
    try:
        for line in open("/proc/meminfo"):
            if line.startswith("MemAvailable:"):
                return float(line.split()[1]) / 1024 ** 2
    except Exception:
        pass
    return 0.0


def run_reference(args, rank, world, dist):
    """The oracle (C++ restatement of the reference routines) on all host
    cores.  At the headline size (512^3) when the host has the memory for it
    (about 66 GB), with at most 2 timed steps after 1 warm-up step (each
    step is some 30-70 s of CPU work); otherwise 128^3 steps, whose per-point
    rate stands in for 512^3 (stated in config.sample)."""
    if rank != 0:
        return 0
    from oracle import pyoracle as po
    threads = os.cpu_count()
    po.set_threads(threads)
    need = 1.24 * ((512 + 11) / (128 + 11)) ** 3  # GB, scaled from a 128^3 measurement
    big = mem_available_gb() >= 1.5 * need and not os.environ.get("ASTR_REF_SMALL")
    n = 512 if big else 128
    steps = min(args.steps, 2) if big else args.steps
    warmup = 1 if big else args.warmup
    o = po.tgv_main(n)
    for _ in range(warmup):
        o.rk3_steps(1)
    t0 = time.perf_counter()
    o.rk3_steps(steps)
    dt = time.perf_counter() - t0
    v = n ** 3 * 3 * steps / dt / 1e6
    sample = (f"C++ restatement of the reference routines, TGV {n}^3 (main-solver order), "
              f"{steps} timed RK3 steps after {warmup} warm-up, 1 process, "
              f"{po.get_threads()} OpenMP threads")
    if not big:
        sample += "; the 512^3 workload did not fit the host memory, its per-point rate stands in"
    line = {
        "impl": "reference", "metric": METRIC, "value": round(v, 3), "unit": UNIT,
        "n_gpus": world, "steps": steps, "warmup": warmup,
        "ms_per_step": round(1e3 * dt / steps, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": "Taylor-Green vortex 512^3, main-solver RK3 stage order",
                   "sample": f"TGV {n}^3, one RK3 step per timed step",
                   "same_size": big},
        "cpu_baseline": {"value": round(v, 3), "unit": UNIT, "cores": po.get_threads(),
                         "kind": "port", "sample": sample},
        "e2e": {"value": round(v, 3), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


CFL = 0.5


def tgv_inputs(n):
    """Grid metrics and initial state of the n^3 TGV, and the time step at
    CFL 0.5 (cflcal's measure) on that grid."""
    from astr_gb300 import cases
    L = 2.0 * np.pi
    x, y, z = cases.gridcube(n, n, n, L, L, L)
    (d11, d22, d33), J = cases.rect_metrics(x, y, z, diag_only=True)
    st = cases.tgv_state(n, n, n, mach=0.1, x=x, y=y, z=z)
    st["deltat"] = cases.cfl_deltat(st, (d11, d22, d33), 0.1, CFL)
    return (d11, d22, d33, J), st


def make_solver(n, precision, metrics, st):
    from astr_gb300 import capi
    from astr_gb300.solver import GpuSolver
    g = GpuSolver(n, n, n, order=capi.ORDER_MAIN, precision=precision, mach=0.1,
                  reynolds=1600.0, deltat=st["deltat"])
    g.set_metrics_diag(*metrics)
    g.upload_state(st["q"], st["rho"], st["vel"], st["prs"], st["tmp"])
    return g


def interior_q(g, n):
    """Interior conserved variables (n+1)^3 x 5 from the device."""
    s = g.download_state()
    h = 5
    return np.ascontiguousarray(s["q"][h:h + n + 1, h:h + n + 1, h:h + n + 1, :])


def state_error(q, ref):
    """Relative L2 and Linf of q against ref: density and energy field by
    field, momentum as one vector field (the TGV's w starts at zero), and the
    whole state with each variable scaled by its reference RMS."""
    def l2(a, b):
        return float(np.linalg.norm((a - b).ravel()) / np.linalg.norm(b.ravel()))

    def linf(a, b):
        return float(np.max(np.abs(a - b)) / np.max(np.abs(b)))

    groups = {"rho": slice(0, 1), "momentum": slice(1, 4), "energy": slice(4, 5)}
    out = {"rel_l2": {}, "rel_linf": {}}
    for k, sl in groups.items():
        out["rel_l2"][k] = l2(q[..., sl], ref[..., sl])
        out["rel_linf"][k] = linf(q[..., sl], ref[..., sl])
    return out


def form_roofline(kt, f32, pts_int, fp64_peak, hbm_peak, hbm_source, tiled=False, pts_unique=None):
    classes = {}
    for k in ("filter", "convgrad", "pointwise", "visc"):
        tms, cnt = kt[k]
        if cnt == 0:
            continue
        nbytes, flops = class_work(k, f32, cnt, pts_int, tiled)
        classes[k] = {"ms": tms, "launches": cnt, "avg_ms": tms / cnt,
                      "gbs": nbytes / (tms / 1e3) / 1e9, "tflops": flops / (tms / 1e3) / 1e12,
                      "bytes_per_launch": nbytes / cnt, "flops_per_launch": flops / cnt}
    dom = max(classes, key=lambda k: classes[k]["ms"])
    dc = classes[dom]
    traffic = None
    try:
        prof = json.load(open(os.path.join(ROOT, "profiles", "ncu_traffic.json")))
        bpt = prof.get("fp32" if f32 else "fp64", {}).get(dom, {}).get("bytes_per_pt")
        traffic = None if bpt is None else round(bpt * pts_int)
    except Exception:
        pass
    rnd = lambda v: round(v, 4) if isinstance(v, float) else v  # noqa: E731
    if f32:
        roof = {"bound": "hbm", "kernel": dom, "achieved": round(dc["gbs"], 1),
                "peak": hbm_peak, "unit": "GB/s", "frac": round(dc["gbs"] / hbm_peak, 4),
                "peak_source": hbm_source}
    else:
        roof = {"bound": "fp64", "kernel": dom, "achieved": round(dc["tflops"], 4),
                "peak": round(fp64_peak, 4), "unit": "TFLOP/s",
                "frac": round(dc["tflops"] / fp64_peak, 4),
                "peak_source": "FP64 FMA loop measured live in this run",
                "hbm_achieved_gbs": round(dc["gbs"], 1),
                "hbm_frac": round(dc["gbs"] / hbm_peak, 4), "hbm_peak_source": hbm_source}
    roof["traffic"] = traffic
    roof["bytes_model"] = ("per-kernel: every array element the launch reads or writes once "
                           "(stored nodes)")
    # the same kernel against the scope table's pass-model bytes (P1, unique
    # points): the fraction a fully fused pass structure would score
    p1 = p1_bytes_per_launch(dom, f32)
    if p1 is not None and pts_unique:
        a1 = p1 * pts_unique / (dc["avg_ms"] / 1e3) / 1e9
        roof["p1"] = {"bytes_per_point_launch": round(p1, 2), "achieved": round(a1, 1),
                      "unit": "GB/s", "frac": round(a1 / hbm_peak, 4),
                      "note": "pass-model (P1) bytes per unique point and launch of this class "
                              "over its average CUDA-event launch time, against the same peak"}
    roof["classes"] = {k: {kk: rnd(vv) for kk, vv in v.items()} for k, v in classes.items()}
    return roof


def time_form(g, args, dist):
    """Warm-up, then K timed steps with per-class kernel times; returns
    (device ms for K steps, kernel times, clock record, first-step stats)."""
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
    return max_over_ranks(dist, ms), kt, clk, hist0


def run_gpu(args, rank, world, dist):
    from astr_gb300 import capi

    n = args.n
    t0 = time.perf_counter()
    metrics, st = tgv_inputs(n)
    deltat = st["deltat"]
    t_setup = time.perf_counter() - t0
    pts = float(n) ** 3
    pts_int = float(n + 1) ** 3
    steps_total = args.warmup + args.steps
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        pass
    if "hbm_gbs" in peaks:
        hbm_peak = float(peaks["hbm_gbs"])
        hbm_source = "hbm_gbs of measured (MEASURED_PEAKS.json, burst copy)"
    else:
        hbm_peak = 6800.0
        hbm_source = "6800 GB/s of fallback (no MEASURED_PEAKS.json on this machine)"
    fp64_peak = ctypes_peak()

    forms = {}
    finals = {}
    clocks = {}
    runs = [("fp64", capi.FP64), ("fp32_storage", capi.FP32_STORAGE)]
    if args.form != "both":
        # one form only (for profiling); no error against FP64
        runs = [r for r in runs if r[0] == args.form]
    # end to end through the C ABI with page-locked host buffers, per form:
    # every step uploads the state q (the primitives are recomputed from it
    # on the device, astr_gpu_upload_q), runs one RK3 step, and downloads q
    pinned_q = capi.PinnedArray(st["q"].shape)
    pinned_q.array[...] = st["q"]
    qout = capi.PinnedArray(st["q"].shape)
    e2e_steps = max(10, args.steps)
    launches_per_step = 0
    v2env = os.environ.get("ASTR_V2", "1")
    for name, prec in runs:
        g = make_solver(n, prec, metrics, st)
        f32 = prec == capi.FP32_STORAGE
        tiled = (f32 and v2env != "0") or v2env == "2"
        ms, kt, clk, hist0 = time_form(g, args, dist)
        forms[name] = {
            "value": round(world * pts * 3 * args.steps / (ms / 1e3) / 1e6, 3),
            "ms_per_step": round(ms / args.steps, 3),
            "roofline": form_roofline(kt, f32, pts_int, fp64_peak, hbm_peak, hbm_source, tiled, pts),
            "sweeps": "tiled" if tiled else "register-window",
            "footprint_gb": round(capi.load().astr_gpu_footprint(g.dims, g.params) / 1e9, 2),
            "stats_first_step": {"kenergy": float(hist0[0, 0]), "enstrophy": float(hist0[0, 1])},
        }
        clocks[name] = clk
        finals[name] = interior_q(g, n) if rank == 0 else None
        # one untimed round trip (first-use costs of the transfer path)
        g.upload_q(pinned_q.array)
        g.time_integration_rk(1)
        g._c(g.L.astr_gpu_download_state(g.h, capi.dptr(qout.array), None, None, None, None))
        barrier(dist)
        t0 = time.perf_counter()
        for _ in range(e2e_steps):
            g.upload_q(pinned_q.array)
            g.time_integration_rk(1)
            g._c(g.L.astr_gpu_download_state(g.h, capi.dptr(qout.array), None, None, None, None))
        t_e2e = max_over_ranks(dist, time.perf_counter() - t0)
        forms[name]["e2e"] = {"value": round(world * pts * 3 * e2e_steps / t_e2e / 1e6, 3),
                              "unit": UNIT, "h2d_bytes_per_step": pinned_q.nbytes,
                              "d2h_bytes_per_step": qout.nbytes + 16, "steps": e2e_steps}
        if name == runs[-1][0]:
            g0 = g.launches
            g.timed_steps(1)
            launches_per_step = g.launches - g0
        g.close()
    pinned_q.free()
    qout.free()
    err = None
    if rank == 0 and len(runs) == 2:
        err = state_error(finals["fp32_storage"], finals["fp64"])
        err["steps"] = steps_total
        err["reference"] = "plain FP64 GPU form, same initial state and steps"
    finals.clear()

    # kinetic-energy / enstrophy histories of both forms over the scale
    # test's 200 steps from the same initial state (untimed)
    history = None
    if rank == 0 and len(runs) == 2 and args.history_steps > 0:
        hist = {}
        for name, prec in runs:
            g = make_solver(n, prec, metrics, st)
            hist[name] = g.time_integration_rk(args.history_steps)
            if name == "fp64":
                q64_end = interior_q(g, n)
            else:
                q32_end = interior_q(g, n)
            g.close()
        h64, h32 = hist["fp64"], hist["fp32_storage"]
        rel = np.abs(h32 - h64) / np.abs(h64)
        history = {"steps": args.history_steps,
                   "kenergy_max_rel_diff": float(rel[:, 0].max()),
                   "enstrophy_max_rel_diff": float(rel[:, 1].max()),
                   "kenergy_fp64_first_last": [float(h64[0, 0]), float(h64[-1, 0])],
                   "enstrophy_fp64_first_last": [float(h64[0, 1]), float(h64[-1, 1])],
                   "final_state_error": state_error(q32_end, q64_end),
                   "reference": "plain FP64 GPU form, same initial state, statistics every step"}
        del q64_end, q32_end
    e2e_line = forms[runs[-1][0]]["e2e"]

    cpu = None
    if rank == 0 and not args.no_cpu:
        v, cores, dt = cpu_port_throughput(128, 4, threads=os.cpu_count())
        cpu = {"value": round(v, 3), "unit": UNIT, "cores": cores, "kind": "port",
               "sample": f"C++ restatement of the reference routines (oracle/), FP64, TGV 128^3 "
                         f"main-solver ordering, 4 RK3 steps in {dt:.1f} s, {cores} OpenMP threads"}
    if rank == 0:
        f32 = forms[runs[-1][0]]
        line = {
            "metric": METRIC, "value": f32["value"], "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": f32["ms_per_step"], "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32 storage, f64 accumulate",
            "data": "synthetic",
            "config": {"workload": f"Taylor-Green vortex {n}^3 ({n + 1}^3 stored nodes), Re 1600, "
                                   "Mach 0.1, 643c compact scheme + compact filter alpha 0.49, "
                                   f"RK3 at CFL {CFL} (dt {deltat:.4e}), main-solver stage order",
                       "form": "FP32 storage / FP64 accumulate (headline); plain FP64 beside it",
                       "parallelism": f"replicas x{world}",
                       "l2": "inputs resident in HBM (37-50 GB) >> 129 MB L2, no flush",
                       "setup_s": round(t_setup, 1)},
            "forms": forms,
            "fp32_over_fp64": (round(f32["value"] / forms["fp64"]["value"], 3)
                               if len(forms) == 2 else None),
            "error_vs_fp64": err,
            "history_vs_fp64": history,
            "gpu_launches": launches_per_step * args.steps,
            "roofline": f32["roofline"],
            "e2e": e2e_line,
            "cpu_baseline": cpu,
            "clocks": clocks[runs[-1][0]],
            "clocks_fp64": clocks.get("fp64"),
        }
    # serving (the batch kernels) on the same GPU, after the TGV runs
    if args.serve_in_line and args.serve_cases > 0:
        srv = serve_summary(args, rank, world, dist, ("batched", "streams"))
        if rank == 0:
            line["serve"] = srv
    if rank == 0:
        print(json.dumps(line), flush=True)
    return 0


def run_history(args, rank, world, dist):
    """Both forms N steps with per-step statistics; the largest relative
    difference of the kinetic-energy / enstrophy histories and the final
    state error."""
    from astr_gb300 import capi
    if rank != 0:
        return 0
    n = args.n
    metrics, st = tgv_inputs(n)
    hist, finals, ms = {}, {}, {}
    for name, prec in (("fp64", capi.FP64), ("fp32_storage", capi.FP32_STORAGE)):
        g = make_solver(n, prec, metrics, st)
        t0 = time.perf_counter()
        hist[name] = g.time_integration_rk(args.history)
        ms[name] = 1e3 * (time.perf_counter() - t0) / args.history
        finals[name] = interior_q(g, n)
        g.close()
    h64, h32 = hist["fp64"], hist["fp32_storage"]
    rel = np.abs(h32 - h64) / np.abs(h64)
    err = state_error(finals["fp32_storage"], finals["fp64"])
    line = {
        "workload": f"Taylor-Green vortex {n}^3, Re 1600, Mach 0.1, main-solver order, "
                    f"CFL {CFL} (dt {st['deltat']:.4e})",
        "steps": args.history,
        "kenergy_max_rel_diff": float(rel[:, 0].max()),
        "enstrophy_max_rel_diff": float(rel[:, 1].max()),
        "kenergy_first_last_fp64": [float(h64[0, 0]), float(h64[-1, 0])],
        "enstrophy_first_last_fp64": [float(h64[0, 1]), float(h64[-1, 1])],
        "final_state_error": err,
        "wall_ms_per_step_with_stats": {k: round(v, 2) for k, v in ms.items()},
    }
    print(json.dumps(line), flush=True)
    if args.history_out:
        os.makedirs(os.path.dirname(os.path.abspath(args.history_out)), exist_ok=True)
        np.savetxt(args.history_out, np.column_stack([np.arange(1, args.history + 1), h64, h32]),
                   header="step ke_fp64 enstrophy_fp64 ke_fp32s enstrophy_fp32s")
    return 0


def run_vortex(args, rank, world, dist):
    """2-D isentropic vortex transport (periodic [-5,5]^2, beta 5, freestream
    (1,1), inviscid, CFL 0.5): both forms for args.vortex_steps steps, each
    scored by relative L2 / Linf error against the analytic translated
    vortex and the FP32-storage form against the FP64 form."""
    from astr_gb300 import capi, cases
    from astr_gb300.solver import GpuSolver
    if rank != 0:
        return 0
    n = args.vortex_n
    gamma = 1.4
    mach = 1.0 / np.sqrt(gamma)
    st = cases.vortex_state(n)
    x, y, z = cases.vortex_grid(n)
    (d11, d22, d33), J = cases.rect_metrics(x, y, z, diag_only=True)
    dt = cases.cfl_deltat(st, (d11, d22, d33), mach, CFL)
    steps = args.vortex_steps
    t_end = steps * dt
    ex = cases.vortex_state(n, t=t_end)
    h = 5
    sl = (slice(h, h + n + 1), slice(h, h + n + 1), h)

    def errs(s, ref):
        out = {}
        for name, a, b in (("rho", s["rho"][sl], ref["rho"][sl]),
                           ("u", s["vel"][sl + (0,)], ref["vel"][sl + (0,)]),
                           ("v", s["vel"][sl + (1,)], ref["vel"][sl + (1,)]),
                           ("p", s["prs"][sl], ref["prs"][sl])):
            d = a - b
            out[name] = {"rel_l2": float(np.linalg.norm(d) / np.linalg.norm(b)),
                         "rel_linf": float(np.abs(d).max() / np.abs(b).max())}
        return out

    forms, finals = {}, {}
    for name, prec in (("fp64", capi.FP64), ("fp32_storage", capi.FP32_STORAGE)):
        g = GpuSolver(n, n, 0, precision=prec, diffterm=False, mach=mach, reynolds=1e4, deltat=dt)
        g.set_metrics_diag(d11, d22, d33, J)
        g.upload_state(st["q"], st["rho"], st["vel"], st["prs"], st["tmp"])
        g.timed_steps(args.warmup)
        # plain launches, CUDA-event timed; then the same steps as CUDA graph
        # launches (astr_gpu_step_async), wall-clock timed: 263K points make
        # the 36 launches of a step latency-bound
        g.upload_state(st["q"], st["rho"], st["vel"], st["prs"], st["tmp"])
        ms = g.timed_steps(steps)
        g.upload_state(st["q"], st["rho"], st["vel"], st["prs"], st["tmp"])
        g.step_async(1)
        g.synchronize()
        g.upload_state(st["q"], st["rho"], st["vel"], st["prs"], st["tmp"])
        t0 = time.perf_counter()
        g.step_async(steps)
        g.synchronize()
        ms_graph = 1e3 * (time.perf_counter() - t0)
        s = g.download_state()
        g.close()
        pts2 = float(n) ** 2 * 3 * steps
        forms[name] = {"value": round(pts2 / (ms_graph / 1e3) / 1e6, 3),
                       "ms_per_step": round(ms_graph / steps, 4),
                       "plain_launch_value": round(pts2 / (ms / 1e3) / 1e6, 3),
                       "error_vs_analytic": errs(s, ex)}
        finals[name] = s
    forms["fp32_storage"]["error_vs_fp64"] = errs(finals["fp32_storage"], finals["fp64"])
    line = {
        "case": "vortex2d",
        "workload": f"isentropic vortex beta 5, periodic [-5,5]^2, {n}^2, freestream (1,1), "
                    f"inviscid, filter alpha 0.49, CFL {CFL} (dt {dt:.4e}), {steps} RK3 steps "
                    f"(t = {t_end:.4f})",
        "unit": UNIT, "forms": forms,
        "fp32_over_fp64": round(forms["fp32_storage"]["value"] / forms["fp64"]["value"], 3),
        "note": "analytic solution: the initial vortex translated by (t, t), nearest periodic "
                "image; value: wall time of the graph-launched stepping loop (no statistics), "
                "plain_launch_value: CUDA-event time of ordinary launches; state resident in HBM",
    }
    print(json.dumps(line), flush=True)
    return 0


def run_channel(args, rank, world, dist):
    """Compressible channel (Mach 0.5, Re 3000 on the half height, Re_tau
    about 185), 256 x 192 x 128 intervals, tanh-stretched y, noslip
    isothermal walls, body force from the mass-flux controller, laminar
    profile + 5 % seeded perturbation, CFL 0.5: both forms for
    args.channel_steps steps; the FP32-storage form against the FP64 one."""
    from astr_gb300 import capi, cases
    from astr_gb300.solver import GpuSolver
    if rank != 0:
        return 0
    im, jm, km = args.channel_dims
    mach, re = 0.5, 3000.0
    x, y, z = cases.channel_grid(im, jm, km)
    st = cases.channel_state(im, jm, km, y, mach=mach)
    dxi, J = cases.rect_metrics(x, y, z, npdc=(3, 4, 3))
    diag = tuple(np.asfortranarray(dxi[..., d, d]) for d in range(3))
    dt = cases.cfl_deltat(st, diag, mach, CFL)
    xh = cases.grid_halo(x, y, z)
    steps = args.channel_steps
    h = 5
    sl = (slice(h, h + im + 1), slice(h, h + jm + 1), slice(h, h + km + 1))
    pts = float(im) * float(jm + 1) * float(km)  # unique nodes: walls counted, periodic once
    forms, finals = {}, {}
    for name, prec in (("fp64", capi.FP64), ("fp32_storage", capi.FP32_STORAGE)):
        g = GpuSolver(im, jm, km, precision=prec, npdc=(3, 4, 3), mach=mach, reynolds=re,
                      deltat=dt, channel=True, twall=1.0)
        # rectilinear kernels: gridgeom's off-diagonal rounding residue
        # (about 1e-12 of the diagonal) is dropped
        g.set_metrics_diag(*diag, J)
        g.set_grid(xh)
        g.upload_state(st["q"], st["rho"], st["vel"], st["prs"], st["tmp"])
        ms = g.timed_steps(steps)
        s = g.download_state()
        cs = g.channel_state()
        g.close()
        forms[name] = {"value": round(pts * 3 * steps / (ms / 1e3) / 1e6, 3),
                       "ms_per_step": round(ms / steps, 4),
                       "force": float(cs[0]), "massflux": float(cs[1]),
                       "massflux_target": float(cs[2]), "wall_friction": float(cs[3])}
        finals[name] = s["q"][sl]
    a, b = finals["fp32_storage"], finals["fp64"]
    err = {}
    for nm, sel in (("rho", slice(0, 1)), ("momentum", slice(1, 4)), ("energy", slice(4, 5))):
        d = a[..., sel] - b[..., sel]
        err[nm] = {"rel_l2": float(np.linalg.norm(d) / np.linalg.norm(b[..., sel])),
                   "rel_linf": float(np.abs(d).max() / np.abs(b[..., sel]).max())}
    forms["fp32_storage"]["error_vs_fp64"] = err
    line = {
        "case": "channel",
        "workload": f"channel {im}x{jm}x{km}, Mach {mach}, Re {re:g}, y tanh stretch 2.0, "
                    f"isothermal walls Tw = 1, CFL {CFL} (dt {dt:.4e}), {steps} RK3 steps",
        "unit": UNIT, "points": pts, "forms": forms,
        "fp32_over_fp64": round(forms["fp32_storage"]["value"] / forms["fp64"]["value"], 3),
        "note": "device time of the stepping loop incl. walls, bulk sums and the controller; "
                "state resident in HBM",
    }
    print(json.dumps(line), flush=True)
    return 0


SERVE_WORKLOAD = ("seeded Poisson stream (seed 20261203): TGV 3-D / vortex 2-D 50/50, edge "
                  "log-U 32-192 / 64-1024, Re log-U 100-3000, Mach U(0.05,0.3), steps "
                  "U{50..500}, CFL 0.5")


def serve_arm(reqs, backend, budget, slots, dist, total):
    """Serve `reqs` through `backend`; the summary with the makespan taken
    over ranks and cases/s over all `total` requests."""
    from astr_gb300 import serve
    srv = serve.Server(backend, budget, max_active=slots)
    barrier(dist)
    recs = serve.serve(reqs, srv)
    srv.close()
    out = serve.summarize(reqs, recs)
    out["makespan_s"] = round(max_over_ranks(dist, out["makespan_s"]), 3)
    out["cases_per_s"] = round(total / out["makespan_s"], 3)
    out.update({"peak_active": srv.peak_active, "peak_hbm_gb": round(srv.peak_used / 1e9, 2),
                "gpu_launches": srv.launches + getattr(backend, "batch_launches", 0)})
    if hasattr(backend, "calls"):
        out["batched_calls"] = backend.calls
    return out


def serve_summary(args, rank, world, dist, arms):
    """Serving: a Poisson stream of independent cases (3-D TGV / 2-D vortex,
    50/50; edge log-uniform 32-192 / 64-1024; Re log-uniform 100-3000; Mach
    uniform 0.05-0.3; steps uniform 50-500) at args.serve_rate per second,
    the first args.serve_cases requests of the stream, through each arm:
    "batched": FP32-storage cases stepped together by the batch kernels
    (persistent kernels over (case, block) work lists; cases join and leave
    between calls of a few steps; cases the batch kernels do not take run on
    their own graphs), "hybrid": the same with the cases of more than
    args.serve_hybrid_points points on their own graphs, "streams": every
    case on its own stream and graphs, "sequential_fp64": one case at a time
    in plain FP64."""
    import torch  # noqa: F401  (CUDA context for the memory query)
    from astr_gb300 import capi, serve
    allreqs = serve.make_requests(args.serve_cases, rate=args.serve_rate, seed=20261203)
    # N GPUs: N independent servers, each taking every N-th request
    reqs = serve.partition(allreqs, rank, world)
    free, total = torch.cuda.mem_get_info()
    budget = int(0.8 * free)
    out = {}
    for arm in arms:
        if arm in ("batched", "hybrid"):
            mp = args.serve_hybrid_points if arm == "hybrid" else None
            be = serve.BatchBackend(capi.FP32_STORAGE, chunk=args.serve_chunk,
                                    groups=args.serve_groups, max_points=mp)
            out[arm] = serve_arm(reqs, be, budget, args.serve_slots, dist, len(allreqs))
            out[arm]["chunk_steps"] = args.serve_chunk
            out[arm]["batches"] = args.serve_groups
            if mp is not None:
                out[arm]["batched_up_to_points"] = mp
            be.close()
        elif arm == "streams":
            out[arm] = serve_arm(reqs, serve.GpuBackend(capi.FP32_STORAGE), budget,
                                 args.serve_slots, dist, len(allreqs))
        else:
            barrier(dist)
            seq = serve.summarize(reqs, serve.serve_sequential(reqs, serve.GpuBackend(capi.FP64)))
            seq["makespan_s"] = round(max_over_ranks(dist, seq["makespan_s"]), 3)
            seq["cases_per_s"] = round(len(allreqs) / seq["makespan_s"], 3)
            out[arm] = seq
    work = sum(serve.request_points(q) * 3 * q.steps for q in allreqs)
    out.update({
        "workload": f"first {len(allreqs)} requests at {args.serve_rate:g}/s of the "
                    + SERVE_WORKLOAD,
        "offered_mpts_stages": round(work / 1e6, 1),
        "hbm_budget_gb": round(budget / 1e9, 1), "slots": args.serve_slots, "n_gpus": world,
        "latency_note": "p50/p99 of rank 0's share when n_gpus > 1",
        "note": "time to solution = finish - arrival (wall clock, host-driven loop incl. case "
                "set-up, upload and download); the offered load exceeds one GPU, so latency "
                "includes queueing",
    })
    return out


def run_serve(args, rank, world, dist):
    out = serve_summary(args, rank, world, dist, tuple(args.serve_arms.split(",")))
    if rank == 0:
        print(json.dumps(dict(case="serve", **out)), flush=True)
    return 0


def run_mp(args, rank, world, dist):
    """Compact MP convective scheme (conschm 543c: Steger-Warming split,
    compact upwind interface fluxes, Roe characteristic projection, MP5
    limiting, Ducros sensor; FP64) on the periodic 3-D shock box (TGV at
    Mach 0.3 with a pressure jump, Re 1600, viscous, no filter, CFL 0.5),
    beside the same case with the central scheme; the oracle on the host
    cores on a bounded sample; the Sod tube against the exact Riemann
    solution."""
    from astr_gb300 import capi, cases
    from astr_gb300.solver import GpuSolver
    if rank != 0:
        return 0
    n, mach = args.mp_n, 0.3
    L = 2.0 * np.pi
    x, y, z = cases.gridcube(n, n, n, L, L, L)
    (d11, d22, d33), J = cases.rect_metrics(x, y, z, diag_only=True)
    st = cases.shock_box_state(n, mach=mach, jump=0.5)
    dt = cases.cfl_deltat(st, (d11, d22, d33), mach, CFL)
    pts = float(n) ** 3
    forms = {}
    for scheme in ("543c", "643c"):
        g = GpuSolver(n, n, n, mach=mach, reynolds=1600.0, deltat=dt, lfilter=False,
                      conschm=scheme)
        g.set_metrics_diag(d11, d22, d33, J)
        g.upload_state(st["q"], st["rho"], st["vel"], st["prs"], st["tmp"])
        g.time_integration_rk(1)
        g.timed_steps(args.warmup - 1)
        clocks = ClockSampler(env_int("LOCAL_RANK", 0))
        clocks.start()
        l0 = g.launches
        ms = g.timed_steps(args.steps)
        launches = (g.launches - l0) // args.steps
        clk = clocks.stop()
        g.set_profiling(True)
        g.timed_steps(1)
        kt = {k: round(v[0], 3) for k, v in g.kernel_times().items() if v[1]}
        g.set_profiling(False)
        q = g.download_state()["q"]
        g.close()
        forms[scheme] = {"value": round(pts * 3 * args.steps / (ms / 1e3) / 1e6, 3),
                         "ms_per_step": round(ms / args.steps, 3),
                         "kernel_ms_one_step": kt, "launches_per_step": launches,
                         "finite": bool(np.isfinite(q).all()), "clocks": clk}
    # oracle (C++ restatement, all host cores) on a 64^3 sample of the case
    from oracle import pyoracle as po
    po.set_threads(os.cpu_count())
    ns = 64
    sts = cases.shock_box_state(ns, mach=mach, jump=0.5)
    xs, ys, zs = cases.gridcube(ns, ns, ns, L, L, L)
    ds, _ = cases.rect_metrics(xs, ys, zs, diag_only=True)
    o = po.from_state(sts, (ns, ns, ns), lx=L, ly=L, lz=L, mach=mach, reynolds=1600.0,
                      lfilter=False, conschm="543c",
                      deltat=cases.cfl_deltat(sts, ds, mach, CFL))
    o.rk3_steps(1)
    t0 = time.perf_counter()
    o.rk3_steps(2)
    tc = time.perf_counter() - t0
    cpu = ns ** 3 * 3 * 2 / tc / 1e6
    # Sod tube, 400 points, t = 1.5, against the exact Riemann solution
    im, jm, sdt = 400, 8, 0.004
    ss = cases.shock_tube_state("sod", im, jm)
    xg, yg, zg = cases.grid1d(im, jm)
    dxi, Jg = cases.rect_metrics(xg, yg, zg, npdc=(4, 3, 3))
    g = GpuSolver(im, jm, 0, npdc=(4, 3, 3), mach=3.0, deltat=sdt, lfilter=False,
                  diffterm=False, conschm="543c")
    g.set_metrics(dxi, Jg)
    g.upload_state(ss["q"], ss["rho"], ss["vel"], ss["prs"], ss["tmp"])
    g.time_integration_rk(int(round(1.5 / sdt)))
    rho = g.download_state()["rho"][5:5 + im + 1, 5, 5]
    g.close()
    re_, _, _ = cases.riemann_exact((1.0, 0.0, 1.0), (0.125, 0.0, 0.1), xg, 1.5)
    line = {
        "case": "mp",
        "workload": f"periodic shock box {n}^3: TGV at Mach {mach}, pressure x1.5 in z < pi, "
                    f"Re 1600, viscous, no filter, CFL {CFL} (dt {dt:.4e}); conschm 543c "
                    "(lchardecomp, bfacmpld 0.3, shkcrt 0.01) against 643c on the same case",
        "unit": UNIT, "dtype": "f64", "forms": forms,
        "mp_over_central_time": round(forms["543c"]["ms_per_step"] / forms["643c"]["ms_per_step"], 3),
        "cpu_baseline": {"value": round(cpu, 3), "unit": UNIT, "cores": po.get_threads(),
                         "kind": "port",
                         "sample": f"oracle, the same case at {ns}^3, conschm 543c, 2 RK3 steps in "
                                   f"{tc:.2f} s"},
        "sod_400_t1.5": {"rho_l1_vs_exact": round(float(np.mean(np.abs(rho - re_))), 6)},
        "note": "device time of the stepping loop (CUDA events), state resident in HBM; "
                "kernel_ms_one_step from a separate profiled step",
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
    ap.add_argument("--form", default="both", choices=["both", "fp64", "fp32_storage"])
    ap.add_argument("--case", default="tgv", choices=["tgv", "vortex2d", "channel", "serve", "mp"])
    ap.add_argument("--mp-n", type=int, default=256)
    ap.add_argument("--serve-cases", type=int, default=100)
    ap.add_argument("--serve-rate", type=float, default=50.0)
    ap.add_argument("--serve-slots", type=int, default=32)
    ap.add_argument("--serve-chunk", type=int, default=20)
    ap.add_argument("--serve-arms", default="batched,streams,sequential_fp64")
    ap.add_argument("--serve-groups", type=int, default=1)
    ap.add_argument("--serve-hybrid-points", type=float, default=2e5)
    ap.add_argument("--no-serve", dest="serve_in_line", action="store_false",
                    help="leave the serving key out of the TGV line")
    ap.add_argument("--channel-dims", type=int, nargs=3, default=[256, 192, 128])
    ap.add_argument("--channel-steps", type=int, default=500)
    ap.add_argument("--vortex-n", type=int, default=512)
    ap.add_argument("--vortex-steps", type=int, default=1000)
    ap.add_argument("--history", type=int, default=0)
    ap.add_argument("--history-steps", type=int, default=200)
    ap.add_argument("--history-out", default="")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    rank, world, dist = dist_setup()
    if args.impl == "reference":
        return run_reference(args, rank, world, dist)
    if args.case == "vortex2d":
        return run_vortex(args, rank, world, dist)
    if args.case == "channel":
        return run_channel(args, rank, world, dist)
    if args.case == "serve":
        return run_serve(args, rank, world, dist)
    if args.case == "mp":
        return run_mp(args, rank, world, dist)
    if args.history:
        return run_history(args, rank, world, dist)
    return run_gpu(args, rank, world, dist)


if __name__ == "__main__":
    sys.exit(main())
