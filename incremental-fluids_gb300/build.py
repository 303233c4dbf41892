"""Build libifluids.so (the CUDA solver behind include/ifluids.h) in-tree.

Every translation unit is compiled by nvcc for sm_103a only, in parallel, and
linked into ``incremental-fluids_gb300/ifluids/libifluids.so``.  The whole
library is compiled with ``--fmad=false``: the FP64 drop-in path must not
contract multiply-adds, so that advection, assembly and the MIC(0) sweeps are
bit-identical to the reference's arithmetic; FP32-form kernels use explicit
fma() where they want one.

    python incremental-fluids_gb300/build.py [--force]
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(PKG, "csrc")
OUT_DIR = os.path.join(PKG, "ifluids")
BUILD_DIR = os.path.join(PKG, "_build")
LIB = os.path.join(OUT_DIR, "libifluids.so")

SOURCES = ["k_fields.cu", "k_pcg.cu", "k_flip.cu", "k_gs.cu", "solver.cu", "batch.cu", "noalloc.cu", "server.cpp", "capi.cpp"]
HEADERS = ["ifl_internal.h", "ifl_device.cuh", "solver.h"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "--fmad=false", "-std=c++17", "-Xcompiler", "-fPIC,-O2,-ffp-contract=off",
         "-I" + os.path.join(PKG, "..", "include")]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.isabs(cand) and os.path.exists(cand) or not os.path.isabs(cand)):
            return cand
    return "nvcc"


def _stale(target: str, deps) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(BUILD_DIR, exist_ok=True)
    nvcc = _nvcc()
    hdrs = [os.path.join(CSRC, h) for h in HEADERS] + [os.path.join(PKG, "..", "include", "ifluids.h")]
    jobs = []
    objs = []
    for src in SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD_DIR, src + ".o")
        objs.append(o)
        if force or _stale(o, [s] + hdrs):
            cmd = [nvcc] + ARCH + FLAGS + ["-c", s, "-o", o]
            if src.endswith(".cpp"):
                cmd = [nvcc] + FLAGS + ["-x", "c++", "-c", s, "-o", o]
            jobs.append(cmd)

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        return cmd, r

    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        for cmd, r in ex.map(run, jobs):
            if verbose or r.returncode != 0:
                sys.stderr.write(" ".join(cmd) + "\n" + r.stdout + r.stderr)
            if r.returncode != 0:
                raise RuntimeError(f"nvcc failed for {cmd[-3]}")
    if force or jobs or _stale(LIB, objs):
        cmd = [nvcc] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            sys.stderr.write(" ".join(cmd) + "\n" + r.stdout + r.stderr)
            raise RuntimeError("link failed")
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
