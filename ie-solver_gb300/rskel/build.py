"""Builds the solver's shared library (CUDA kernels for sm_103a + C++ host code).

Compiles every translation unit in ``csrc/`` in parallel and links
``lib/librskel.so`` in-tree.  Host C++ is compiled with floating-point
contraction disabled so the quadtree is identical on x86-64 and aarch64.
Also links ``lib/libfmapeak.so`` (``csrc/fma_peak.cu``), the CUDA-core FMA
peak measurement the benchmark uses as its roofline denominator.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess

PKG = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(PKG, "csrc")
OBJ = os.path.join(PKG, "_build")
LIB_DIR = os.path.join(PKG, "lib")
LIB = os.path.join(LIB_DIR, "librskel.so")
PEAK_LIB = os.path.join(LIB_DIR, "libfmapeak.so")
ROOT = os.path.dirname(PKG)

CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA_HOME, "bin", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

CU_SOURCES = ["id_kernel.cu", "decouple_kernel.cu", "solve_kernels.cu", "border_kernels.cu",
              "fmm.cu", "id_noalloc.cu", "domain.cu", "rank_model.cu",
              "krylov.cu"]
CPP_SOURCES = ["tree.cpp", "solver.cpp", "fmm_plan.cpp"]


def _nvcc():
    if os.path.exists(NVCC):
        return NVCC
    found = shutil.which("nvcc")
    if not found:
        raise RuntimeError("nvcc not found; the solver has no CPU fallback")
    return found


def _compile(src, obj, verbose):
    nvcc = _nvcc()
    path = os.path.join(CSRC, src)
    if src.endswith(".cu"):
        cmd = [nvcc, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
               "-Xcompiler", "-ffp-contract=off", "--expt-relaxed-constexpr",
               "-I", CSRC, "-c", path, "-o", obj]
    else:
        cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-fopenmp", "-Wall",
               "-Wno-unused-function", "-I", CSRC, "-I", os.path.join(CUDA_HOME, "include"),
               "-c", path, "-o", obj]
    if verbose:
        print(" ".join(cmd), flush=True)
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"compile failed: {src}\n{res.stdout}\n{res.stderr}")
    return res.stderr


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose=False, force=False):
    os.makedirs(OBJ, exist_ok=True)
    os.makedirs(LIB_DIR, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".hpp", ".cuh"))]
    headers.append(os.path.join(ROOT, "include", "rskel.h"))
    jobs = []
    objs = []
    for src in CU_SOURCES + CPP_SOURCES:
        obj = os.path.join(OBJ, src.rsplit(".", 1)[0] + ".o")
        objs.append(obj)
        if force or _stale(obj, [os.path.join(CSRC, src)] + headers):
            jobs.append((src, obj))
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        futs = [ex.submit(_compile, s, o, verbose) for s, o in jobs]
        for f in futs:
            warn = f.result()
            if verbose and warn:
                print(warn)
    peak_src = os.path.join(CSRC, "fma_peak.cu")
    if force or _stale(PEAK_LIB, [peak_src]):
        cmd = [_nvcc(), *ARCH, "-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-shared", peak_src,
               "-o", PEAK_LIB, "-lcudart"]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"fma_peak build failed\n{res.stdout}\n{res.stderr}")
    if force or jobs or _stale(LIB, objs):
        cmd = [_nvcc(), *ARCH, "-shared", "-o", LIB, *objs, "-lcudart", "-lgomp", "-Xlinker", "--no-undefined"]
        if verbose:
            print(" ".join(cmd), flush=True)
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"link failed\n{res.stdout}\n{res.stderr}")
    return LIB


if __name__ == "__main__":
    print(build(verbose=True))
