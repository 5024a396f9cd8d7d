"""Recipe: build the reference library's own sources for the CPU (oracle only).

Test infrastructure.  Reads src/gridding.cu, src/gaussian_filter.cu,
src/cuna_kernel.cu, src/cufft_utils.cu, src/utils.cu and src/cuna.cpp where
they lie in the reference tree (the directory named by CUNA_REFERENCE_DIR),
rewrites each ``kern<<<grid, block, ...>>>(args)`` launch into
``CUNA_CPU_LAUNCH(grid, block, kern, args)`` on the fly (and drops
src/utils.cu's DOUBLE_PRECISION block, a compare-and-swap atomicAdd for GPUs
without a native double atomic, which the host stand-in replaces), and pipes
the result straight into g++ together with the host stand-ins in
oracle/refcpu/.  No reference source is copied anywhere; the only outputs are
object files and two shared libraries in oracle/_ref/:

    oracle/_ref/libcuna_refcpu_f.so   (float build, like libcunaf.so)
    oracle/_ref/libcuna_refcpu_d.so   (-DDOUBLE_PRECISION, like libcunad.so)

The reference is compiled with BLOCK_SIZE=256 as its Makefile does
(Makefile:16,30).  Differences from the reference's GPU build: libm's correctly
rounded expf/powf/sqrtf instead of --use_fast_math intrinsics (about 1e-7
relative per filter weight in float), no FMA contraction (-ffp-contract=off, so
x86 and Arm hosts give identical bits), and a deterministic atomic order.
cuFFT is replaced by the double-precision DFT stand-in in refcpu/cufft.h.

Usage: python oracle/build_ref.py            (no-op when the reference is absent)
"""
import os
import re
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
SHIM = os.path.join(HERE, "refcpu")
REF_SOURCES = ["gridding.cu", "gaussian_filter.cu", "cuna_kernel.cu", "cufft_utils.cu", "utils.cu", "cuna.cpp"]

_LAUNCH = re.compile(r"(\w+)\s*<<<(.*?)>>>\s*\(", re.S)
_DOUBLE_ATOMIC = re.compile(r"^#ifdef DOUBLE_PRECISION\s*\n.*?^#endif[^\n]*\n", re.S | re.M)


def _rewrite_launches(src: str) -> str:
    def repl(m):
        cfg = [c.strip() for c in m.group(2).split(",")]
        return "CUNA_CPU_LAUNCH((%s), (%s), %s, " % (cfg[0], cfg[1], m.group(1))

    return _LAUNCH.sub(repl, src)


def _drop_double_atomic(src: str) -> str:
    """src/utils.cu:28-44 defines atomicAdd(double *, double) by a CAS loop;
    the host stand-in provides that overload instead."""
    out, n = _DOUBLE_ATOMIC.subn("", src, count=1)
    if n != 1 or "atomicCAS" in out:
        raise RuntimeError("build_ref: the DOUBLE_PRECISION atomicAdd block of utils.cu was not found")
    return out


def reference_dir():
    """The reference tree: CUNA_REFERENCE_DIR when set, else a directory
    named ``reference`` beside this repository."""
    env = os.environ.get("CUNA_REFERENCE_DIR")
    if env:
        return env
    return os.path.join(os.path.dirname(os.path.dirname(HERE)), "reference")


def libs_present():
    return all(os.path.exists(os.path.join(OUT, "libcuna_refcpu_%s.so" % p)) for p in "fd")


def build(verbose=False):
    ref = reference_dir()
    if not os.path.isdir(os.path.join(ref, "src")):
        if verbose:
            print("build_ref: reference tree not present; skipped")
        return False
    os.makedirs(OUT, exist_ok=True)
    inc = os.path.join(ref, "inc")
    base = ["g++", "-std=c++17", "-fext-numeric-literals", "-O2", "-fPIC", "-ffp-contract=off", "-w",
            "-DBLOCK_SIZE=256", "-I", SHIM, "-I", inc,
            "-include", os.path.join(SHIM, "cuda_runtime.h")]

    def compile_one(args):
        name, prec = args
        defs = ["-DDOUBLE_PRECISION"] if prec == "d" else []
        obj = os.path.join(OUT, "%s_%s.o" % (os.path.splitext(name)[0], prec))
        if name == "cuda_cpu_shim.cpp":
            cmd = base + defs + ["-c", os.path.join(SHIM, name), "-o", obj]
            subprocess.run(cmd, check=True)
        else:
            with open(os.path.join(ref, "src", name)) as f:
                src = _rewrite_launches(f.read())
            if name == "utils.cu":
                src = _drop_double_atomic(src)
            cmd = base + defs + ["-x", "c++", "-c", "-", "-o", obj]
            subprocess.run(cmd, input=src.encode(), check=True)
        return obj

    jobs = [(s, p) for p in "fd" for s in REF_SOURCES + ["cuda_cpu_shim.cpp"]]
    with ThreadPoolExecutor(max_workers=8) as ex:
        objs = list(ex.map(compile_one, jobs))
    for p in "fd":
        mine = [o for o in objs if o.endswith("_%s.o" % p)]
        subprocess.run(["g++", "-shared", "-o", os.path.join(OUT, "libcuna_refcpu_%s.so" % p)]
                       + mine + ["-lm"], check=True)
    for o in objs:
        os.remove(o)
    if verbose:
        print("build_ref: built", OUT)
    return True


if __name__ == "__main__":
    sys.exit(0 if build(verbose=True) or True else 1)
