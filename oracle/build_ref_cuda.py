"""Recipe: the reference library's own CUDA build, libcunaf.so / libcunad.so --
the parity target and timed comparator of the GPU path.  Test
infrastructure: nothing in the product links or loads it.

Two steps:

* ``stage()`` -- where the reference tree is available (CUNA_REFERENCE_DIR,
  else a directory named ``reference`` beside this repository), copy its
  ``src/`` and ``inc/`` into ``baseline/_ref/`` (the reference's install
  location: git-ignored, never committed, but it travels with the working
  tree to the machine with the GPU).
* ``build()`` -- compile ``baseline/_ref/{src,inc}`` for sm_103a with the
  reference Makefile's flags (``--use_fast_math``, ``-rdc=true``,
  ``-DBLOCK_SIZE=256``; host code with g++; Makefile:16-33) into
  ``baseline/_ref/lib/<machine>/libcuna{f,d}.so``.  Three shims and nothing
  else (oracle/refcuda/): ``shim.h`` maps names CUDA 13 removed
  (cudaThreadSynchronize, two cufftResult values), ``ovl/complex.h`` gives
  the C99 ``complex`` spelling of inc/cuna.h a C++ meaning, and the
  DOUBLE_PRECISION block of src/utils.cu (a compare-and-swap atomicAdd for
  GPUs older than sm_60, which collides with the native one) is left out of
  the compiled copy.  The reference's sources are otherwise compiled as they
  are.

The libraries export the reference's C++ names, the same names as this
project's drop-in libraries, so callers load them in a separate process
(tests/_refcuda_child.py) or by absolute path with RTLD_LOCAL.

Usage: python oracle/build_ref_cuda.py [--stage]
"""
import os
import platform
import re
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
REF_INSTALL = os.path.join(ROOT, "baseline", "_ref")
SHIM = os.path.join(HERE, "refcuda")
CU = ["cuna_kernel.cu", "gaussian_filter.cu", "gridding.cu", "cufft_utils.cu", "utils.cu"]
CPP = ["cuna.cpp"]
_DOUBLE_ATOMIC = re.compile(r"^#ifdef DOUBLE_PRECISION\s*\n.*?^#endif[^\n]*\n", re.S | re.M)


def reference_dir():
    env = os.environ.get("CUNA_REFERENCE_DIR")
    if env:
        return env
    return os.path.join(os.path.dirname(ROOT), "reference")


def lib_dir(machine=None):
    return os.path.join(REF_INSTALL, "lib", machine or platform.machine())


def lib_path(prec, machine=None):
    return os.path.join(lib_dir(machine), "libcuna%s.so" % prec)


def available():
    return all(os.path.exists(lib_path(p)) for p in "fd")


def stage(verbose=False):
    """Copy the reference's src/ and inc/ into baseline/_ref (no-op without
    the reference tree)."""
    ref = reference_dir()
    if not os.path.isdir(os.path.join(ref, "src")):
        return False
    for sub in ("src", "inc"):
        dst = os.path.join(REF_INSTALL, sub)
        os.makedirs(dst, exist_ok=True)
        for f in os.listdir(os.path.join(ref, sub)):
            s = os.path.join(ref, sub, f)
            d = os.path.join(dst, f)
            if os.path.isfile(s) and (not os.path.exists(d) or os.path.getmtime(d) < os.path.getmtime(s)):
                shutil.copy2(s, d)
    if verbose:
        print("build_ref_cuda: staged", REF_INSTALL)
    return True


def _nvcc():
    return shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"


def _cuda_root():
    return os.path.dirname(os.path.dirname(os.path.realpath(_nvcc())))


def _up_to_date(out):
    srcs = [os.path.join(REF_INSTALL, "src", f) for f in CU + CPP]
    srcs += [os.path.join(SHIM, "shim.h"), os.path.join(SHIM, "ovl", "complex.h"), os.path.abspath(__file__)]
    outs = [os.path.join(out, "libcuna%s.so" % p) for p in "fd"]
    return all(os.path.exists(o) for o in outs) and \
        min(os.path.getmtime(o) for o in outs) > max(os.path.getmtime(s) for s in srcs if os.path.exists(s))


def build(verbose=False, force=False):
    """Compile the staged sources for this machine (no-op when nothing is
    staged).  Returns True when the libraries exist afterwards."""
    src = os.path.join(REF_INSTALL, "src")
    inc = os.path.join(REF_INSTALL, "inc")
    if not all(os.path.exists(os.path.join(src, f)) for f in CU + CPP):
        return False
    out = lib_dir()
    if not force and _up_to_date(out):
        return True
    obj = os.path.join(REF_INSTALL, "build", platform.machine())
    os.makedirs(out, exist_ok=True)
    os.makedirs(obj, exist_ok=True)
    with open(os.path.join(src, "utils.cu")) as f:
        utils, n = _DOUBLE_ATOMIC.subn("", f.read(), count=1)
    if n != 1 or "atomicCAS" in utils:
        raise RuntimeError("build_ref_cuda: the DOUBLE_PRECISION atomicAdd block of utils.cu was not found")
    utils_path = os.path.join(obj, "utils_native_atomics.cu")
    with open(utils_path, "w") as f:
        f.write(utils)
    cuda_inc = os.path.join(_cuda_root(), "include")
    cuda_lib = None
    for d in ("lib64", "lib", os.path.join("targets", "sbsa-linux", "lib"), os.path.join("targets", "x86_64-linux", "lib")):
        if os.path.exists(os.path.join(_cuda_root(), d, "libcufft.so")):
            cuda_lib = os.path.join(_cuda_root(), d)
            break
    cuda_lib = cuda_lib or os.path.join(_cuda_root(), "lib64")
    gencode = ["-gencode", "arch=compute_103a,code=sm_103a"]
    nv = [_nvcc(), "-DBLOCK_SIZE=256", "-DVERSION=\"1.3\"", "--use_fast_math", "-Xcompiler", "-O3", "-Xcompiler",
          "-fpic", "-w"] + gencode + ["-rdc=true", "-include", os.path.join(SHIM, "shim.h"),
                                       "-I", os.path.join(SHIM, "ovl"), "-I", inc]
    cc = ["g++", "-DBLOCK_SIZE=256", "-DVERSION=\"1.3\"", "-fPIC", "-w", "-include", os.path.join(SHIM, "shim.h"),
          "-I", os.path.join(SHIM, "ovl"), "-I", inc, "-I", cuda_inc]

    def run(cmd):
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("build_ref_cuda failed:\n%s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))

    def compile_one(job):
        name, prec = job
        defs = ["-DDOUBLE_PRECISION"] if prec == "d" else []
        o = os.path.join(obj, "%s_%s.o" % (os.path.splitext(name)[0], prec))
        if name in CPP:
            run(cc + defs + ["-c", os.path.join(src, name), "-o", o])
        else:
            path = utils_path if name == "utils.cu" else os.path.join(src, name)
            run(nv + defs + ["-c", path, "-o", o])
        return o

    jobs = [(n_, p) for p in "fd" for n_ in CU + CPP]
    with ThreadPoolExecutor(max_workers=len(jobs)) as ex:
        objs = dict(zip(jobs, ex.map(compile_one, jobs)))
    for p in "fd":
        dev = [objs[(n_, p)] for n_ in CU]
        dl = os.path.join(obj, "dlink_%s.o" % p)
        run([_nvcc()] + gencode + ["-Xcompiler", "-fpic", "-dlink"] + dev + ["-o", dl])
        run(["g++", "-shared", "-o", os.path.join(out, "libcuna%s.so" % p)] + dev + [objs[("cuna.cpp", p)], dl,
            "-L" + cuda_lib, "-lcudart", "-lcufft", "-lm", "-Wl,-rpath," + cuda_lib])
    if verbose:
        print("build_ref_cuda: built", out)
    return True


if __name__ == "__main__":
    if "--stage" in sys.argv:
        stage(verbose=True)
    ok = build(verbose=True, force="--force" in sys.argv)
    print("reference CUDA build:", "ok" if ok else "nothing staged")
