"""Builds libmbgb.so in-tree: the sm_103a kernels and the C-ABI host code.

Translation units compile in parallel; the FP64 kernel unit is built with
--fmad=false so that double arithmetic keeps the reference's rounding steps.
Host C++ is built with -ffp-contract=off so x86 and Arm hosts derive the same
per-frame doubles.
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
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libmbgb.so")
PEAK_LIB = os.path.join(PKG, "libmbgb_peak.so")
CLI = os.path.join(PKG, "mbgb_cli")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _cuda_home() -> str:
    for cand in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if cand and os.path.exists(os.path.join(cand, "bin", "nvcc")):
            return cand
    nvcc = shutil.which("nvcc")
    if nvcc:
        return os.path.dirname(os.path.dirname(nvcc))
    raise RuntimeError("nvcc not found: set CUDA_HOME")


def _units(cuda: str):
    nvcc = os.path.join(cuda, "bin", "nvcc")
    common_cu = [nvcc, "-std=c++17", "-O3", *ARCH, "-lineinfo", "-Xcompiler", "-fPIC,-ffp-contract=off",
                 "-I", INCLUDE, "-I", CSRC]
    common_cpp = ["g++", "-std=c++17", "-O2", "-fPIC", "-ffp-contract=off", "-Wall", "-Wno-unused-function",
                  "-I", INCLUDE, "-I", CSRC, "-I", os.path.join(cuda, "include")]
    yield "render_f64.cu", common_cu + ["--fmad=false"]
    yield "render_f32.cu", common_cu
    yield "noalloc.cu", common_cu
    yield "wave_f64.cu", common_cu + ["--fmad=false"]
    yield "wave_f32.cu", common_cu
    yield "wave_more_f64.cu", common_cu + ["--fmad=false"]
    yield "wave_more_f32.cu", common_cu
    yield "render_more_f64.cu", common_cu + ["--fmad=false"]
    yield "render_more_f32.cu", common_cu
    yield "post.cu", common_cu + ["--fmad=false"]
    yield "capi.cpp", common_cpp
    yield "settings.cpp", common_cpp
    yield "keyframes.cpp", common_cpp
    yield "image_io.cpp", common_cpp


def _sources_newer(target: str) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    for d in (CSRC, INCLUDE):
        for f in os.listdir(d):
            if os.path.getmtime(os.path.join(d, f)) > t:
                return True
    return os.path.getmtime(__file__) > t


def build(force: bool = False, verbose: bool = False) -> str:
    """Compiles every unit and links libmbgb.so; returns its path."""
    if not force and not _sources_newer(LIB):
        return LIB
    cuda = _cuda_home()
    os.makedirs(BUILD, exist_ok=True)
    jobs = []
    for src, cmd in _units(cuda):
        obj = os.path.join(BUILD, src + ".o")
        jobs.append((obj, cmd + ["-c", os.path.join(CSRC, src), "-o", obj]))

    def run(job):
        obj, cmd = job
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        return obj

    with cf.ThreadPoolExecutor(max_workers=len(jobs)) as ex:
        objs = list(ex.map(run, jobs))
    tmp = LIB + ".tmp"
    link = [os.path.join(cuda, "bin", "nvcc"), "-shared", *ARCH, "-o", tmp, *objs, "-cudart", "static"]
    r = subprocess.run(link, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed: {' '.join(link)}\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    # ALU peak microbenchmark (bench.py's roofline denominator), a separate tool library
    peak = [os.path.join(cuda, "bin", "nvcc"), "-std=c++17", "-O3", *ARCH, "-shared", "-Xcompiler", "-fPIC",
            "-o", PEAK_LIB, os.path.join(CSRC, "peak.cu"), "-cudart", "static"]
    r = subprocess.run(peak, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"peak tool build failed: {' '.join(peak)}\n{r.stdout}\n{r.stderr}")
    # the -nogui command-line renderer, linked against the library next to it
    cli = [os.path.join(cuda, "bin", "nvcc"), "-std=c++17", "-O2", "-I", INCLUDE, "-o", CLI,
           os.path.join(CSRC, "cli.cpp"), "-L", PKG, "-lmbgb", "-Xlinker", "-rpath,$ORIGIN", "-cudart", "static"]
    r = subprocess.run(cli, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"mbgb_cli build failed: {' '.join(cli)}\n{r.stdout}\n{r.stderr}")
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
