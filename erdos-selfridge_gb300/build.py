#!/usr/bin/env python3
"""Build libes_gb300.so (sm_103a) in-tree with nvcc: the scan kernels (one translation unit per
table layout), the host C ABI and the learned-planner MLP kernels, compiled in parallel, linked
against the CUDA runtime.

    python erdos-selfridge_gb300/build.py [--force]

The output lands next to this file; it is git-ignored and rebuilt on each machine (the CPU
build container and the Arm GPU host compile the same sources).
"""
from __future__ import annotations

import argparse
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "libes_gb300.so")
OBJDIR = os.path.join(HERE, "_build")
SOURCES = ["es_scan_wm.cu", "es_scan_wmc.cu", "es_scan_pair.cu", "es_scan_sc.cu", "es_scan_sm.cu", "es_scan_sp.cu", "es_scan.cu", "es_abi.cu",
           "es_mlp.cu", "es_mitm.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.sep not in cand or os.path.exists(cand)):
            return cand
    return "nvcc"


def _stale(out: str, deps: list[str]) -> bool:
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(OBJDIR, exist_ok=True)
    headers = [os.path.join(CSRC, h) for h in os.listdir(CSRC) if h.endswith((".h", ".cuh"))]
    headers.append(os.path.join(ROOT, "include", "es_gb300.h"))
    srcs = [os.path.join(CSRC, s) for s in SOURCES if os.path.exists(os.path.join(CSRC, s))]
    objs = [os.path.join(OBJDIR, os.path.basename(s) + ".o") for s in srcs]
    flags = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xptxas", "-v"]

    def compile_one(src_obj):
        src, obj = src_obj
        if not force and not _stale(obj, [src] + headers):
            return src, "", 0
        cmd = [nvcc()] + flags + ["-c", src, "-o", obj]
        p = subprocess.run(cmd, capture_output=True, text=True)
        return src, p.stdout + p.stderr, p.returncode

    with ThreadPoolExecutor(max_workers=len(srcs)) as ex:
        results = list(ex.map(compile_one, zip(srcs, objs)))
    for src, log, rc in results:
        if rc != 0:
            raise RuntimeError(f"nvcc failed for {os.path.basename(src)}:\n{log}")
        if verbose and log:
            print(log, file=sys.stderr)
    if force or _stale(OUT, objs):
        cmd = [nvcc()] + ARCH + ["-shared", "-o", OUT] + objs + ["-lcudart"]
        p = subprocess.run(cmd, capture_output=True, text=True)
        if p.returncode != 0:
            raise RuntimeError(f"link failed:\n{p.stdout}{p.stderr}")
    return OUT


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--force", action="store_true")
    ap.add_argument("-v", "--verbose", action="store_true")
    a = ap.parse_args()
    print(build(a.force, a.verbose))
