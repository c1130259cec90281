"""Build the sm_103a shared library of the RHS hot path (in-tree).

Compiles the per-direction sweep translation units and the host/ABI unit in
parallel with nvcc and links ``astr_gb300/_build/libastr_gb300.so``.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libastr_gb300.so")
SOURCES = ["astr_gpu.cu", "sweep_x_f64.cu", "sweep_y_f64.cu", "sweep_z_f64.cu",
           "sweep_x_f32.cu", "sweep_y_f32.cu", "sweep_z_f32.cu", "stats_noalloc.cu", "mp.cu",
           "sweep2_x_f64.cu", "sweep2_y_f64.cu", "sweep2_z_f64.cu", "sweep2_x_f32.cu",
           "sweep2_y_f32.cu", "sweep2_z_f32.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
         "--expt-relaxed-constexpr"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _stale(obj: str, deps) -> bool:
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False, force: bool = False, out_dir: str = BUILD, defines=()) -> str:
    """Compile (what is stale) and link; `out_dir` and `defines` (-D flags,
    e.g. launch-shape constants) build a variant beside the default one."""
    os.makedirs(out_dir, exist_ok=True)
    lib = os.path.join(out_dir, "libastr_gb300.so")
    headers = [os.path.join(CSRC, h) for h in os.listdir(CSRC) if h.endswith((".cuh", ".h"))]
    headers.append(os.path.join(HERE, "..", "include", "astr_gpu.h"))
    objs, jobs = [], []
    for src in SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(out_dir, src.replace(".cu", ".o"))
        objs.append(o)
        if force or _stale(o, [s] + headers):
            cmd = [nvcc()] + ARCH + FLAGS + [f"-D{d}" for d in defines] + ["-c", s, "-o", o + ".tmp"]
            if verbose:
                cmd.insert(1, "-Xptxas=-v")
            jobs.append((cmd, o))

    def run(job):
        cmd, o = job
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
        os.replace(o + ".tmp", o)
        return r.stdout + r.stderr

    if jobs:
        with cf.ThreadPoolExecutor(max_workers=len(jobs)) as ex:
            for out in ex.map(run, jobs):
                if verbose and out:
                    sys.stderr.write(out)
    if jobs or not os.path.exists(lib):
        cmd = [nvcc()] + ARCH + ["-shared", "-o", lib + ".tmp"] + objs + ["-lcudart"]
        subprocess.check_call(cmd)
        os.replace(lib + ".tmp", lib)
    return lib


if __name__ == "__main__":
    t = build(verbose="-v" in sys.argv, force="-f" in sys.argv)
    print(t)
