"""Build the native parts in-tree, for sm_103a, without cmake.

Outputs (git-ignored, rebuilt on every machine):
    gpuexplore_gb300/_lib/libgpx.so     the C-ABI library (CUDA kernels + host driver)
    gpuexplore_gb300/_lib/gpuexplore    the command-line tool (links libgpx.so)
    oracle/_build/gpx_oracle            the CPU oracle (test infrastructure only)

Translation units compile in parallel; a rebuild is skipped when the outputs are
newer than every source.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from typing import List

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "gpuexplore_gb300")
CSRC = os.path.join(PKG, "csrc")
LIBDIR = os.path.join(PKG, "_lib")
INCLUDE = os.path.join(ROOT, "include")
ORACLE_DIR = os.path.join(ROOT, "oracle")
ORACLE_BUILD = os.path.join(ORACLE_DIR, "_build")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-I" + INCLUDE, "-I" + CSRC]

LIB = os.path.join(LIBDIR, "libgpx.so")
CLI = os.path.join(LIBDIR, "gpuexplore")
ORACLE = os.path.join(ORACLE_BUILD, "gpx_oracle")


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _stale(out: str, srcs: List[str]) -> bool:
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(s) > t for s in srcs)


def _run_parallel(cmds: List[List[str]]) -> None:
    procs = [(c, subprocess.Popen(c, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)) for c in cmds]
    failed = []
    for c, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            failed.append((c, out))
    if failed:
        msg = "\n\n".join(" ".join(c) + "\n" + out for c, out in failed)
        raise RuntimeError("native build failed:\n" + msg)


def build_library(force: bool = False) -> str:
    """Compile libgpx.so and the gpuexplore tool; returns the library path."""
    os.makedirs(LIBDIR, exist_ok=True)
    srcs_cu = [os.path.join(CSRC, "gpx_explore.cu"), os.path.join(CSRC, "gpx_batch.cu"),
               os.path.join(CSRC, "gpx_por.cu"), os.path.join(CSRC, "gpx_live.cu")]
    srcs_cpp = [os.path.join(CSRC, "gpx_model.cpp")]
    headers = [os.path.join(INCLUDE, "gpx.h"), os.path.join(CSRC, "gpx_model.h"),
               os.path.join(CSRC, "gpx_device.cuh"), os.path.join(CSRC, "gpx_live.h")]
    cli_src = os.path.join(CSRC, "gpuexplore_main.cpp")
    nvcc = _nvcc()
    if force or _stale(LIB, srcs_cu + srcs_cpp + headers):
        objs, cmds = [], []
        for s in srcs_cu + srcs_cpp:
            o = os.path.join(LIBDIR, os.path.basename(s) + ".o")
            objs.append(o)
            cmds.append([nvcc] + ARCH + NVCC_FLAGS + ["-c", s, "-o", o])
        _run_parallel(cmds)
        _run_parallel([[nvcc] + ARCH + ["-shared", "-o", LIB] + objs])
        for o in objs:
            os.remove(o)
    if force or _stale(CLI, [cli_src, LIB] + headers):
        _run_parallel([["g++", "-O2", "-std=c++17", "-I" + INCLUDE, cli_src, "-o", CLI, "-L" + LIBDIR, "-lgpx",
                        "-Wl,-rpath,$ORIGIN"]])
    return LIB


def build_oracle(force: bool = False) -> str:
    """Compile the CPU oracle (single-thread and OpenMP in one binary)."""
    os.makedirs(ORACLE_BUILD, exist_ok=True)
    src = os.path.join(ORACLE_DIR, "gpx_oracle.c")
    if force or _stale(ORACLE, [src]):
        _run_parallel([["gcc", "-O2", "-fopenmp", "-std=gnu11", src, "-o", ORACLE, "-lm"]])
    return ORACLE


def build_all(force: bool = False) -> None:
    build_library(force)
    build_oracle(force)


if __name__ == "__main__":
    build_all(force="--force" in sys.argv)
    print(LIB)
    print(CLI)
    print(ORACLE)
