"""Builds the leela_gb300 CUDA library in-tree (leela_gb300/libleela_gb300.so).

nvcc compiles every translation unit for sm_103a (tcgen05, TMA) in parallel
and links one shared library that exports the C ABI of include/leela_gpu.h.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libleela_gb300.so")
SOURCES = ["lg_api.cu", "fp32_path.cu", "tc_conv.cu", "distill.cu", "ensemble.cu", "weights_io.cu", "gather.cu",
           "latency.cu", "fast_net.cu", "finish.cu"]
NVCC = os.environ.get("NVCC", "nvcc")
FLAGS = ["-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-lineinfo", "-std=c++17",
         "-Xcompiler", "-fPIC", "-Xcompiler", "-fvisibility=hidden"]


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False, extra_flags=None) -> str:
    os.makedirs(BUILD, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    headers.append(os.path.join(os.path.dirname(HERE), "include", "leela_gpu.h"))
    flags = FLAGS + list(extra_flags or [])

    def compile_one(src):
        obj = os.path.join(BUILD, src.replace(".cu", ".o"))
        srcp = os.path.join(CSRC, src)
        if _stale(obj, [srcp] + headers):
            cmd = [NVCC] + flags + ["-c", srcp, "-o", obj]
            if verbose:
                print(" ".join(cmd), flush=True)
            r = subprocess.run(cmd, capture_output=True, text=True)
            if r.returncode != 0:
                raise RuntimeError(f"nvcc failed for {src}:\n{r.stderr}")
        return obj

    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    if _stale(LIB, objs):
        cmd = [NVCC, "-shared", "-o", LIB] + objs + ["-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stderr}")
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
