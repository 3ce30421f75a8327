"""Build the bwa-cuda shared library (libbwacuda.so) for sm_103a.

Compiles every ``csrc/*.cu`` translation unit in parallel with nvcc and links
them into ``bwa-mem4_gb300/libbwacuda.so`` (static CUDA runtime, no torch
dependency).  Usage: ``python bwa-mem4_gb300/build.py [--force] [-j N]``.
"""
from __future__ import annotations

import argparse
import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libbwacuda.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
              "--expt-relaxed-constexpr", "-Xptxas", "-warn-spills"]


def nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found: the CUDA extension cannot be built")
    return cand


def _sources():
    return sorted(glob.glob(os.path.join(CSRC, "*.cu")))


def _headers():
    return sorted(glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(os.path.join(CSRC, "*.cuh")) +
                  glob.glob(os.path.join(HERE, "..", "include", "*.h")))


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


SYNTH_SRC = os.path.join(CSRC, "synth.c")
SYNTH_LIB = os.path.join(HERE, "libbwasynth.so")


def build_synth(force: bool = False) -> str:
    """Host-only workload generator (gcc, OpenMP); portable C, no arch flags."""
    if force or _stale(SYNTH_LIB, [SYNTH_SRC]):
        cc = shutil.which("gcc") or shutil.which("cc")
        cmd = [cc, "-O2", "-std=c11", "-fPIC", "-shared", "-fopenmp", "-o", SYNTH_LIB, SYNTH_SRC]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            sys.stderr.write(r.stdout + r.stderr)
            raise RuntimeError("building libbwasynth.so failed")
    return SYNTH_LIB


def build(force: bool = False, jobs: int = 0, verbose: bool = False) -> str:
    os.makedirs(OUT_DIR, exist_ok=True)
    build_synth(force)
    srcs = _sources()
    hdrs = _headers()
    objs = []
    todo = []
    for s in srcs:
        o = os.path.join(OUT_DIR, os.path.basename(s)[:-3] + ".o")
        objs.append(o)
        if force or _stale(o, [s] + hdrs):
            todo.append((s, o))
    exe = nvcc()

    def compile_one(so):
        s, o = so
        cmd = [exe] + ARCH + NVCC_FLAGS + ["-c", s, "-o", o]
        r = subprocess.run(cmd, capture_output=True, text=True)
        return s, r

    if todo:
        n = jobs or min(len(todo), os.cpu_count() or 4)
        with cf.ThreadPoolExecutor(max_workers=n) as ex:
            for s, r in ex.map(compile_one, todo):
                if verbose or r.returncode != 0:
                    sys.stderr.write(r.stdout + r.stderr)
                if r.returncode != 0:
                    raise RuntimeError(f"nvcc failed on {os.path.basename(s)}")
    if force or todo or _stale(LIB, objs):
        cmd = [exe] + ARCH + ["-shared", "-o", LIB] + objs + ["-lpthread"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            sys.stderr.write(r.stdout + r.stderr)
            raise RuntimeError("linking libbwacuda.so failed")
    return LIB


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--force", action="store_true")
    ap.add_argument("-j", type=int, default=0)
    ap.add_argument("-v", action="store_true")
    a = ap.parse_args()
    print(build(force=a.force, jobs=a.j, verbose=a.v))
