"""Compile libcacg.so in-tree for sm_103a with nvcc (no cmake, no torch).

Translation units are compiled in parallel.  Everything that must match the
reference's FP64 operation order is compiled with ``-fmad=false``; the fast
FP64 and mixed-precision kernels get contraction.  Host code is built with
``-ffp-contract=off`` so that, on any host ISA, the spline tables and element
shape functions computed on the CPU are the reference's own values.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
from typing import List

PKG = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libcacg.so")
ROOT = os.path.dirname(PKG)

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler",
          "-ffp-contract=off", "-I", os.path.join(ROOT, "include"), "-I", SRC]

# (source, extra flags)
UNITS = [
    ("host.cpp", ["-x", "cu", "-fmad=false"]),
    ("k_comm.cu", ["-fmad=false"]),
    ("k_neigh.cu", ["-fmad=false"]),
    ("k_nve.cu", ["-fmad=false"]),
    ("k_force_exact.cu", ["-fmad=false"]),
    ("k_force_fma.cu", ["-fmad=true"]),
    ("k_mixed.cu", ["-fmad=true"]),
    ("k_thermo.cu", ["-fmad=true"]),
    ("k_noalloc.cu", ["-fmad=true"]),
    ("k_gemm.cu", ["-fmad=true"]),
    ("mlp.cu", ["-fmad=true"]),
    ("k_surrogate.cu", ["-fmad=true"]),
    ("k_analysis.cu", ["-fmad=false"]),
]


def nvcc() -> str:
    p = shutil.which("nvcc")
    if p:
        return p
    cand = "/usr/local/cuda/bin/nvcc"
    if os.path.exists(cand):
        return cand
    raise RuntimeError("nvcc not found")


def _stale(obj: str, deps: List[str]) -> bool:
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(d) > t for d in deps)


def build_library(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    headers = [os.path.join(SRC, f) for f in os.listdir(SRC) if f.endswith((".h", ".cuh"))]
    headers.append(os.path.join(ROOT, "include", "cacg.h"))
    jobs = []
    objs = []
    for src, extra in UNITS:
        path = os.path.join(SRC, src)
        if not os.path.exists(path):
            continue
        obj = os.path.join(BUILD, src + ".o")
        objs.append(obj)
        if force or _stale(obj, [path] + headers):
            cmd = [nvcc()] + ARCH + COMMON + extra + ["-c", path, "-o", obj]
            jobs.append(cmd)

    def run(cmd):
        p = subprocess.run(cmd, capture_output=True, text=True)
        if p.returncode != 0:
            raise RuntimeError("nvcc failed:\n" + " ".join(cmd) + "\n" + p.stdout + p.stderr)
        if verbose and (p.stdout or p.stderr):
            print(p.stdout + p.stderr)
        return p

    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(8, len(jobs))) as ex:
            list(ex.map(run, jobs))
    if force or jobs or not os.path.exists(LIB):
        link = [nvcc()] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart"]
        run(link)
    return LIB
