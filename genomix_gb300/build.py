"""Builds libgxgpu.so (CUDA sm_103a + host C++) in-tree.

    python -m genomix_gb300.build          # incremental
    python -m genomix_gb300.build --force

Translation units compile in parallel; the link uses nvcc with the static CUDA runtime.
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libgxgpu.so")
INCLUDE = os.path.join(ROOT, "include")

GENCODE = ["-gencode", "arch=compute_103a,code=sm_103a"]
CUDA_SRCS = ["gx_kernels.cu", "gx_fastq.cu", "gx_job.cu", "gx_batch.cu", "gx_serve.cu", "gx_tune.cu", "gx_graphstats.cu", "gx_noalloc.cu"]
CXX_SRCS = ["gx_formats.cpp"]


def _nvcc():
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.isabs(cand) and os.path.exists(cand) or not os.path.isabs(cand)):
            return cand
    return "nvcc"


def _deps():
    files = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    files.append(os.path.join(INCLUDE, "gxgpu.h"))
    files.append(os.path.abspath(__file__))
    return files


def up_to_date():
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(f) <= t for f in _deps())


def _compile(src):
    obj = os.path.join(BUILD, os.path.basename(src) + ".o")
    if src.endswith(".cu"):
        cmd = [_nvcc(), *GENCODE, "-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-I", INCLUDE,
               "-c", os.path.join(CSRC, src), "-o", obj]
    else:
        cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-I", INCLUDE, "-I", "/usr/local/cuda/include",
               "-c", os.path.join(CSRC, src), "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return obj


def build(force=False, verbose=False):
    """Compiles libgxgpu.so unless it is newer than every source."""
    if not force and up_to_date():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    srcs = CUDA_SRCS + CXX_SRCS
    with ThreadPoolExecutor(max_workers=len(srcs)) as ex:
        objs = list(ex.map(_compile, srcs))
    tmp = LIB + ".tmp"
    cmd = [_nvcc(), *GENCODE, "-shared", "-o", tmp, *objs, "-lpthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    if verbose:
        print("built", LIB)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
