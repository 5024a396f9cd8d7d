"""Build the native libraries in-tree for sm_103a.

Outputs (git-ignored):
    cunfft_adjoint_gb300/lib/libcuna_gb300.so  core: kernels + extern "C" cuna2_* API
    cunfft_adjoint_gb300/lib/libcunaf.so       drop-in CUNA float API (C++ names)
    cunfft_adjoint_gb300/lib/libcunad.so       drop-in CUNA double API

Translation units compile in parallel with one -gencode (sm_103a).  compat.cu
is compiled with --use_fast_math, the flag of the reference build, so the
reference's filter arithmetic maps to the same hardware approximations.

Usage: python -m cunfft_adjoint_gb300.build [--force]
"""
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(PKG, "csrc")
LIB = os.path.join(PKG, "lib")
OBJ = os.path.join(PKG, "_build")
INC = os.path.join(os.path.dirname(PKG), "include")

GENCODE = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_COMMON = GENCODE + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-I", INC]

CORE_UNITS = [
    ("runtime.cu", []),
    ("compat.cu", ["--use_fast_math"]),
    ("accurate.cu", []),
    ("batch.cu", []),
    ("lombscargle.cu", []),
]

LIBS = ["libcuna_gb300.so", "libcunaf.so", "libcunad.so"]


def nvcc():
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return exe


def cuda_lib_dir():
    root = os.path.dirname(os.path.dirname(os.path.realpath(nvcc())))
    for d in ("lib64", "lib", os.path.join("targets", "sbsa-linux", "lib"),
              os.path.join("targets", "x86_64-linux", "lib")):
        p = os.path.join(root, d)
        if os.path.exists(os.path.join(p, "libcufft.so")):
            return p
    return os.path.join(root, "lib64")


def _sources():
    srcs = []
    for d in (CSRC, INC):
        for f in os.listdir(d):
            srcs.append(os.path.join(d, f))
    return srcs


def up_to_date():
    outs = [os.path.join(LIB, l) for l in LIBS]
    if not all(os.path.exists(o) for o in outs):
        return False
    newest_src = max(os.path.getmtime(s) for s in _sources())
    return min(os.path.getmtime(o) for o in outs) > newest_src


def _run(cmd, verbose):
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed:\n%s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
    return r


def build(force=False, verbose=False):
    if not force and up_to_date():
        return LIB
    os.makedirs(LIB, exist_ok=True)
    os.makedirs(OBJ, exist_ok=True)
    cudalib = cuda_lib_dir()

    def compile_unit(unit):
        name, extra = unit
        out = os.path.join(OBJ, os.path.splitext(name)[0] + ".o")
        _run([nvcc()] + NVCC_COMMON + extra + ["-c", os.path.join(CSRC, name), "-o", out], verbose)
        return out

    def compile_dropin(prec):
        out = os.path.join(OBJ, "dropin_%s.o" % prec)
        defs = ["-DDOUBLE_PRECISION"] if prec == "d" else []
        # host arithmetic of the drop-in (scale_x) rounds like the reference's
        # on x86 and Arm alike: no fused multiply-add contraction
        _run([nvcc()] + NVCC_COMMON + defs + ["-Xcompiler", "-ffp-contract=off", "-x", "c++", "-c",
                                              os.path.join(CSRC, "dropin.cpp"), "-o", out], verbose)
        return out

    with ThreadPoolExecutor(max_workers=len(CORE_UNITS) + 2) as ex:
        core = list(ex.map(compile_unit, CORE_UNITS))
        dropins = list(ex.map(compile_dropin, ["f", "d"]))

    rpath = ["-Xlinker", "-rpath," + cudalib, "-Xlinker", "-rpath,$ORIGIN"]
    core_so = os.path.join(LIB, "libcuna_gb300.so")
    _run([nvcc()] + GENCODE + ["-shared", "-o", core_so] + core
         + ["-L" + cudalib, "-lcufft"] + rpath, verbose)
    for prec, obj in zip("fd", dropins):
        _run([nvcc()] + GENCODE + ["-shared", "-o", os.path.join(LIB, "libcuna%s.so" % prec), obj,
                                   "-L" + LIB, "-lcuna_gb300"] + rpath, verbose)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
    print("built", LIB)
