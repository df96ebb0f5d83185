"""Builds the engine's shared library (jp2lam_gb300/_lib/libjp2g.so) with
nvcc for sm_103a, and the oracle when its sources are present.

The CUDA sources are compiled in parallel, one translation unit each, and
linked into one shared object. Host float code is compiled without FMA
contraction so that the plan's step sizes and PCRD constants round exactly
like the reference's f64 arithmetic.
"""
import concurrent.futures
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_lib")
LIB = os.path.join(OUT_DIR, "libjp2g.so")
SYNTH_LIB = os.path.join(OUT_DIR, "libjp2g_synth.so")
ARCH = "-gencode=arch=compute_103a,code=sm_103a"
SOURCES = ["api.cu", "dwt.cu", "t1.cu", "pcrd.cu", "recon.cu", "t2dev.cu", "plan.cpp", "t2.cpp", "tables.cpp", "noalloc.cu",
           "decode.cpp", "t1dec.cu"]


def nvcc():
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libjp2g.so")


def _compile(src, obj):
    cmd = [nvcc(), "-std=c++17", "-O3", "-lineinfo", ARCH, "--fmad=false",
           "-Xcompiler", "-fPIC,-ffp-contract=off,-O2", "-I", os.path.join(ROOT, "include"),
           "-c", os.path.join(CSRC, src), "-o", obj]
    if src.endswith(".cpp"):
        cmd[1:1] = ["-x", "cu"]
    subprocess.run(cmd, check=True)
    return obj


def build_synth():
    """Host-only page generator (no CUDA needed)."""
    os.makedirs(OUT_DIR, exist_ok=True)
    cxx = shutil.which("g++") or "c++"
    tmp = SYNTH_LIB + ".tmp"
    subprocess.run([cxx, "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-shared",
                    os.path.join(CSRC, "synth.cpp"), "-o", tmp], check=True)
    os.replace(tmp, SYNTH_LIB)
    return SYNTH_LIB


def build(verbose=False):
    os.makedirs(OUT_DIR, exist_ok=True)
    build_synth()
    objs = [os.path.join(OUT_DIR, os.path.splitext(s)[0] + ".o") for s in SOURCES]
    with concurrent.futures.ThreadPoolExecutor(len(SOURCES)) as ex:
        list(ex.map(_compile, SOURCES, objs))
    tmp = LIB + ".tmp"
    subprocess.run([nvcc(), "-shared", ARCH, "-o", tmp] + objs + ["-lcudart"], check=True)
    os.replace(tmp, LIB)
    if verbose:
        print("built", LIB)
    return LIB


def build_oracle():
    mk = os.path.join(ROOT, "oracle", "Makefile")
    if os.path.exists(mk):
        subprocess.run(["make", "-s", "-C", os.path.dirname(mk)], check=True)


if __name__ == "__main__":
    build(verbose=True)
    if "--oracle" in sys.argv:
        build_oracle()
