"""Builds libespins_gpu.so in-tree for sm_103a (nvcc + g++, no cmake).

The translation units compile in parallel; the result is
``espins_gb300/libespins_gpu.so``.  Rebuilds only when a source is newer.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess

PKG = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(PKG, "csrc")
ROOT = os.path.dirname(PKG)
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libespins_gpu.so")

GENCODE = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr"] + GENCODE
CXX_FLAGS = ["-O2", "-fPIC", "-std=c++17"]

CU_SOURCES = ["esp_kernels.cu", "esp_api.cu", "esp_noalloc.cu", "esp_cluster.cu", "esp_learned.cu", "esp_tile.cu",
              "esp_lp_tc.cu", "esp_gemm_tc.cu"]
CXX_SOURCES = ["esp_tables.cpp"]
HEADERS = ["esp_device.cuh", "esp_kernels.h", "esp_tables.h", "esp_errors.h", "esp_cluster.h", "esp_learned.h",
           "esp_mlp.cuh", "esp_vmf.cuh", "esp_tile.h", "esp_tc.cuh", "esp_lp_tc.cuh", "esp_lp_tc.h"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libespins_gpu.so")


def _sources():
    return ([os.path.join(CSRC, s) for s in CU_SOURCES + CXX_SOURCES + HEADERS]
            + [os.path.join(ROOT, "include", "espins_gpu.h")])


def up_to_date() -> bool:
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(s) <= t for s in _sources())


def build(force: bool = False, verbose: bool = False) -> str:
    if not force and up_to_date():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    nvcc = _nvcc()
    inc = ["-I", CSRC, "-I", os.path.join(ROOT, "include")]
    cuda_inc = os.path.join(os.path.dirname(os.path.dirname(nvcc)), "include")
    jobs = []
    for s in CU_SOURCES:
        obj = os.path.join(BUILD, s + ".o")
        jobs.append([nvcc] + NVCC_FLAGS + inc + ["-c", os.path.join(CSRC, s), "-o", obj])
    for s in CXX_SOURCES:
        obj = os.path.join(BUILD, s + ".o")
        jobs.append([os.environ.get("CXX", "g++")] + CXX_FLAGS + inc + ["-I", cuda_inc, "-c", os.path.join(CSRC, s), "-o", obj])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
        return r.stdout + r.stderr

    with cf.ThreadPoolExecutor(max_workers=len(jobs)) as ex:
        outs = list(ex.map(run, jobs))
    if verbose:
        for o in outs:
            print(o)
    objs = [os.path.join(BUILD, s + ".o") for s in CU_SOURCES + CXX_SOURCES]
    tmp = LIB + ".tmp"
    run([nvcc, "-shared"] + GENCODE + ["-o", tmp] + objs)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True, verbose=True))
