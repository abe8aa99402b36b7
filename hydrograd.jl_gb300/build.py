"""Build libhydrograd_gb.so in-tree (hydrograd.jl_gb300/build/) for sm_103a.

CUDA sources go through nvcc with one -gencode (compute_103a -> sm_103a);
host C++ sources through g++ with -ffp-contract=off, so that mesh geometry
and bed slopes are computed with exactly the reference's rounding on x86_64
and aarch64 alike.  Translation units compile in parallel.
"""
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "build")
LIB = os.path.join(OUT, "libhydrograd_gb.so")
INCLUDE = os.path.join(ROOT, "include")

CUDA_SOURCES = ["hg_forward_f64.cu", "hg_forward_f32.cu", "hg_adjoint_f64.cu", "hg_adjoint_f32.cu", "hg_noalloc.cu",
                "hg_tsit5.cu", "hg_resistance.cu", "hg_resistance_f32.cu", "hg_final_loss.cu"]
# FP64 parity path: no fused multiply-add, as in the reference (and in the
# Tsit5 stage sums and the FP64 resistance functions, which the oracle forms
# with separate multiplies and adds; their FP32 instantiations,
# hg_resistance_f32.cu, contract).
NO_FMAD = {"hg_forward_f64.cu", "hg_tsit5.cu", "hg_resistance.cu"}
# FP32-compensated path: approximate division/sqrt/log2/exp2 (a few ulp; the
# path's contract is a 1e-5 state error against the FP64 oracle).
FAST_MATH = {"hg_forward_f32.cu", "hg_adjoint_f32.cu"}
CXX_SOURCES = ["hg_mesh.cpp", "hg_capi.cpp", "hg_adjoint.cpp", "hg_tsit5.cpp", "hg_autotune.cpp"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _cuda_home():
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return os.path.dirname(os.path.dirname(os.path.realpath(nvcc))), nvcc


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r.stdout + r.stderr


def _stage_block_define():
    """HG_STAGE_BLOCK: cells per block of the FP32 stage kernels (default 256),
    the same in every translation unit (the host builds the fused stepping's
    per-block tables with it)."""
    v = os.environ.get("HG_STAGE_BLOCK")
    return ["-DHG_STAGE_BLOCK=%d" % int(v)] if v else []


def build(verbose=False):
    cuda_home, nvcc = _cuda_home()
    os.makedirs(OUT, exist_ok=True)
    jobs = []
    objs = []
    for src in CUDA_SOURCES:
        if not os.path.exists(os.path.join(CSRC, src)):
            continue
        obj = os.path.join(OUT, src + ".o")
        objs.append(obj)
        fmad = ["--fmad=false"] if src in NO_FMAD else []
        if src in FAST_MATH and os.environ.get("HG_FAST_MATH", "1") == "1":
            fmad = ["--use_fast_math"]
        if src == "hg_forward_f32.cu" and os.environ.get("HG_STAGE_MIN_BLOCKS"):
            fmad = fmad + ["-DHG_STAGE_MIN_BLOCKS=%d" % int(os.environ["HG_STAGE_MIN_BLOCKS"])]
        fmad = fmad + _stage_block_define()
        jobs.append([nvcc, "-std=c++17", "-O3", *ARCH, *fmad, "-lineinfo", "-Xcompiler", "-fPIC", "-I", INCLUDE,
                     "-c", os.path.join(CSRC, src), "-o", obj])
    for src in CXX_SOURCES:
        obj = os.path.join(OUT, src + ".o")
        objs.append(obj)
        jobs.append(["g++", "-std=c++17", "-O2", "-fPIC", "-ffp-contract=off", "-Wall", "-I", INCLUDE,
                     "-I", os.path.join(cuda_home, "include"), *_stage_block_define(), "-c", os.path.join(CSRC, src),
                     "-o", obj])
    with ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        logs = list(ex.map(_run, jobs))
    if verbose:
        for log in logs:
            if log.strip():
                print(log)
    _run([nvcc, "-shared", *ARCH, "-o", LIB, *objs, "-lcudart_static", "-lrt", "-lpthread", "-ldl"])
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
