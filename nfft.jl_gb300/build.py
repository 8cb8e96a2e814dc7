"""Build libnfftgb300.so (the C-ABI library) in-tree for sm_103a.

Usage: python nfft.jl_gb300/build.py [--force] [--jobs N]

Each .cu translation unit is compiled by its own nvcc process (in parallel)
and the objects are linked into nfft.jl_gb300/nfftgb300/libnfftgb300.so with
the CUDA runtime linked statically and cuFFT dynamically.
"""
from __future__ import annotations

import argparse
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
OUT = os.path.join(HERE, "nfftgb300", "libnfftgb300.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

SOURCES = ["plan.cu", "precompute.cu", "sort.cu", "deconv.cu", "interp.cu", "spread.cu", "gradk.cu", "batch.cu",
           "directional.cu", "fft.cu", "plain.cu", "noalloc.cu", "autotune.cu", "toeplitz.cu", "direct.cu", "trig.cu", "nnfft.cu",
           "sortnodes.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc_path() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libnfftgb300.so")


def cuda_home(nvcc: str) -> str:
    return os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))


def _deps_mtime() -> float:
    paths = [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [os.path.join(INCLUDE, "nfft_gb300.h")]
    return max(os.path.getmtime(p) for p in paths)


def _compile(nvcc: str, src: str, obj: str, extra: list[str]) -> str:
    cmd = [nvcc, *ARCH, "-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC,-O2",
           "--expt-relaxed-constexpr", "-I", INCLUDE, "-c", src, "-o", obj, *extra]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {os.path.basename(src)}:\n{r.stdout}\n{r.stderr}")
    return r.stderr


def build(force: bool = False, jobs: int | None = None, verbose: bool = False, ptxas_v: bool = False) -> str:
    if not force and os.path.exists(OUT) and os.path.getmtime(OUT) >= _deps_mtime():
        return OUT
    nvcc = nvcc_path()
    home = cuda_home(nvcc)
    os.makedirs(BUILD, exist_ok=True)
    extra = ["-Xptxas", "-v"] if ptxas_v else []
    objs = []
    jobs = jobs or min(len(SOURCES), os.cpu_count() or 4)
    with cf.ThreadPoolExecutor(max_workers=jobs) as ex:
        futs = {}
        for s in SOURCES:
            obj = os.path.join(BUILD, s.replace(".cu", ".o"))
            objs.append(obj)
            futs[ex.submit(_compile, nvcc, os.path.join(CSRC, s), obj, extra)] = s
        for f in cf.as_completed(futs):
            log = f.result()
            if verbose and log:
                print(f"--- {futs[f]}\n{log}", file=sys.stderr)
    libdir = os.path.join(home, "lib64")
    if not os.path.isdir(libdir):
        libdir = os.path.join(home, "lib")
    tmp = OUT + f".tmp{os.getpid()}"
    cmd = [nvcc, *ARCH, "-shared", "-o", tmp, *objs, "-cudart", "static", f"-L{libdir}", "-lcufft",
           "-Xlinker", f"-rpath,{libdir}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, OUT)
    return OUT


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--force", action="store_true")
    ap.add_argument("--jobs", type=int, default=None)
    ap.add_argument("--ptxas-v", action="store_true")
    a = ap.parse_args()
    print(build(force=a.force, jobs=a.jobs, verbose=True, ptxas_v=a.ptxas_v))
