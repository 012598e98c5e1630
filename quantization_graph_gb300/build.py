"""Builds libqgraph_gb300.so in-tree with nvcc for sm_103a (no torch extension machinery).

Each translation unit is compiled in parallel into quantization_graph_gb300/_build/, then
linked into quantization_graph_gb300/_build/libqgraph_gb300.so. All CUDA sources are compiled
with --fmad=false: the kernels write every fused multiply-add they need explicitly, which is
what makes them reproduce the reference arithmetic bit for bit.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(ROOT, "include")
BUILD = os.environ.get("QG_BUILD_DIR", os.path.join(PKG, "_build"))
LIB = os.path.join(BUILD, "libqgraph_gb300.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CUDA_SOURCES = ["query_prep.cu", "batch_kernels.cu", "search.cu", "encode.cu", "graph_build.cu", "mlp.cu",
                "search_noalloc.cu", "vamana_build.cu", "rotate_gemm.cu"]
CXX_SOURCES = ["bridge.cpp"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _cuda_home(nvcc: str) -> str:
    return os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False, force: bool = False, ptxas_info: bool = False) -> str:
    """Compile and link the library; returns its path."""
    nvcc = _nvcc()
    os.makedirs(BUILD, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    headers.append(os.path.join(INCLUDE, "qgraph_gb300.h"))
    common = ["-std=c++17", "-O3", "-I", INCLUDE, "-I", CSRC]
    jobs = []
    objs = []
    for src in CUDA_SOURCES:
        path = os.path.join(CSRC, src)
        obj = os.path.join(BUILD, src + ".o")
        objs.append(obj)
        if force or _stale(obj, [path] + headers):
            cmd = [nvcc, *ARCH, *common, "-lineinfo", "--fmad=false", "-Xcompiler", "-fPIC",
                   "-Xcompiler", "-ffp-contract=off", "-c", path, "-o", obj]
            if ptxas_info:
                cmd.insert(1, "-Xptxas=-v")
            jobs.append(cmd)
    cuda_inc = os.path.join(_cuda_home(nvcc), "include")
    for src in CXX_SOURCES:
        path = os.path.join(CSRC, src)
        obj = os.path.join(BUILD, src + ".o")
        objs.append(obj)
        if force or _stale(obj, [path] + headers):
            jobs.append(["g++", "-std=c++17", "-O2", "-fPIC", "-ffp-contract=off", "-I", INCLUDE,
                         "-I", CSRC, "-I", cuda_inc, "-c", path, "-o", obj])
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            results = list(ex.map(lambda c: subprocess.run(c, capture_output=True, text=True), jobs))
        for cmd, res in zip(jobs, results):
            if verbose or res.returncode != 0 or ptxas_info:
                sys.stderr.write(" ".join(cmd) + "\n" + res.stdout + res.stderr)
            if res.returncode != 0:
                raise RuntimeError(f"compilation failed: {os.path.basename(cmd[-3])}")
    if force or jobs or _stale(LIB, objs):
        link = [nvcc, *ARCH, "-shared", "-o", LIB, *objs, "-lcudart_static", "-lrt", "-ldl", "-lpthread"]
        res = subprocess.run(link, capture_output=True, text=True)
        if res.returncode != 0:
            sys.stderr.write(" ".join(link) + "\n" + res.stdout + res.stderr)
            raise RuntimeError("link failed")
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv, ptxas_info="--ptxas" in sys.argv))
