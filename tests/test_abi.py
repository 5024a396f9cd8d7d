"""CPU tests of the C-ABI boundary: the libraries build for sm_103a, load
without a GPU, and export every symbol the headers in include/ declare (the
drop-in libraries under the reference's C++ linkage names).  No compute call
is made here."""
import ctypes
import os
import re
import subprocess

import pytest

from conftest import ROOT

INC = os.path.join(ROOT, "include")

# C++ linkage names of the reference's host API (inc/cuna.h, inc/cuna_filter.h,
# inc/cuna_typedefs.h, inc/cuna_utils.h, inc/cufft_utils.h) in its float build;
# the double build replaces f/float2 by d/double2.
DROPIN_F = [
    "_Z14cunfft_adjointPKfS0_PCfiij",
    "_Z24cunfft_adjoint_from_planP4plan",
    "_Z18cunfft_adjoint_rawPKfS0_P6float2iiPK17filter_properties",
    "_Z24cunfft_adjoint_raw_asyncPKfS0_P6float2iiPK17filter_propertiesP11CUstream_st",
    "_Z34cunfft_adjoint_raw_async_bootstrapPKfS0_P6float2iiiPK17filter_propertiesP11CUstream_stj",
    "_Z34cunfft_adjoint_raw_async_bootstrapPKfS0_P6float2iiiPK17filter_propertiesP11CUstream_st",
    "_Z26generate_filter_propertiesPKfiiPP17filter_propertiesS3_",
    "_Z33generate_pinned_filter_propertiesPKfiiP17filter_propertiesS2_P11CUstream_st",
    "_Z21set_filter_propertiesP4plan",
    "_Z22free_filter_propertiesP17filter_propertiesS0_",
    "_Z9init_planP4planPKfS2_iij",
    "_Z9free_planP4plan",
    "_Z10print_planP4plan",
    "_Z15performGriddingP4plan",
    "_Z11performFFTsP4plan",
    "_Z16normalizeResultsP4plan",
    "_Z16copyResultsToCPUP4plan",
    "_Z7scale_xPfi",
    "_Z14nextPowerOfTwoj",
    "_Z7secondsl",
    "_Z17launchDummyKernelv",
    "_Z14printComplex_dP6float2iP8_IO_FILE",
    "_Z11printReal_dPfiP8_IO_FILE",
    "_Z12printComplexP6float2iP8_IO_FILE",
    "_Z9printRealPfiP8_IO_FILE",
    "_Z15cufftParseError13cufftResult_t",
    "_Z15checkCufftError13cufftResult_t",
]


def _to_double(sym):
    return (sym.replace("PKf", "PKd").replace("PCf", "PCd").replace("P6float2", "P7double2")
            .replace("_Z7scale_xPfi", "_Z7scale_xPdi").replace("PfiP8", "PdiP8"))


DROPIN_D = [_to_double(s) for s in DROPIN_F]


def _exports(path):
    out = subprocess.run(["nm", "-D", "--defined-only", path], capture_output=True, text=True,
                         check=True).stdout
    return {l.split()[-1] for l in out.splitlines() if " T " in l}


def test_libraries_build_and_load(native_built):
    from cunfft_adjoint_gb300 import _lib
    for p in _lib.library_paths():
        assert os.path.exists(p)
    lib = _lib.core()
    assert lib.cuna2_version().decode().startswith("cuna-gb300")
    assert lib.cuna2_status_string(1) == b"CUNA2_ERROR_INVALID_VALUE"


def test_core_exports_every_cuna2_declaration(native_built):
    from cunfft_adjoint_gb300 import _lib
    decl = set(re.findall(r"\b(cuna2_\w+)\s*\(", open(os.path.join(INC, "cuna2.h")).read()))
    assert decl, "no declarations parsed"
    exported = _exports(_lib.library_paths()[0])
    missing = sorted(decl - exported)
    assert not missing, missing
    # and the Python bindings declare a signature for each
    assert decl <= set(_lib.CORE_SIGNATURES)


@pytest.mark.parametrize("prec,names", [("f", DROPIN_F), ("d", DROPIN_D)])
def test_dropin_exports_reference_names(native_built, prec, names):
    from cunfft_adjoint_gb300 import _lib
    exported = _exports(os.path.join(_lib.LIB_DIR, "libcuna%s.so" % prec))
    missing = [s for s in names if s not in exported]
    assert not missing, missing
    lib = _lib.dropin(prec)
    for s in names:
        getattr(lib, s)  # resolvable through dlsym


def test_dropin_headers_declare_every_name():
    """Each function named in DROPIN_F is declared in include/*.h."""
    text = "".join(open(os.path.join(INC, f)).read() for f in os.listdir(INC) if f.endswith(".h"))
    for s in DROPIN_F:
        name = re.match(r"_Z\d+([A-Za-z_]+?)(?=P|v|j|l|13|$)", s)
        m = re.match(r"_Z(\d+)", s)
        fname = s[len(m.group(0)):len(m.group(0)) + int(m.group(1))]
        assert re.search(r"\b%s\s*\(" % fname, text), fname


def test_reference_names_match_reference_build():
    """When the reference's own sources were built for the CPU here
    (oracle/build_ref.py), its host API names are exactly DROPIN_F/D."""
    from oracle.oracle import RefCPU
    for prec, names in (("f", DROPIN_F), ("d", DROPIN_D)):
        if not RefCPU.available(prec):
            pytest.skip("reference build not present")
        ref = _exports(os.path.join(ROOT, "oracle", "_ref", "libcuna_refcpu_%s.so" % prec))
        api = [s for s in names if not s.startswith(("_Z7scale_x", "_Z14nextPowerOfTwo", "_Z7seconds",
                                                    "_Z17launchDummy", "_Z14printComplex_d",
                                                    "_Z11printReal_d", "_Z12printComplex",
                                                    "_Z9printReal", "_Z34cunfft_adjoint_raw_async_bootstrap"))
               or s.endswith("stj")]
        # utils.cu / cuna.cpp are not part of the CPU build; the unseeded
        # bootstrap overload is declared by the reference but never defined
        api = [s for s in api if not s.startswith(("_Z14cunfft_adjoint", "_Z9init_plan", "_Z9free_plan",
                                                   "_Z10print_plan"))]
        missing = [s for s in api if s not in ref]
        assert not missing, missing


def test_struct_layouts():
    from cunfft_adjoint_gb300 import _lib
    assert ctypes.sizeof(_lib.FilterPropertiesF32) == 40
    assert _lib.FilterPropertiesF32.E1.offset == 16
    assert ctypes.sizeof(_lib.FilterPropertiesF64) == 48
    assert _lib.FilterPropertiesF64.E1.offset == 24


def test_no_oracle_in_product():
    """The product package never imports or links the oracle."""
    pkg = os.path.join(ROOT, "cunfft_adjoint_gb300")
    for dirpath, _, files in os.walk(pkg):
        for f in files:
            if f.endswith((".py", ".cu", ".cuh", ".cpp", ".h")):
                txt = open(os.path.join(dirpath, f)).read()
                assert "oracle" not in txt.replace("the oracle", ""), os.path.join(dirpath, f)


_C_EXAMPLE = r"""#include <stdio.h>
#include <stdlib.h>
#include <cuda_runtime.h>
#include "cuna2.h"

/* t_d: n doubles, y_d: n floats, F_d: nf float2 values, all in device memory */
int transform_series(const double *t_d, const float *y_d, float2 *F_d, int64_t n, double t0, double T,
                     cudaStream_t stream, int count) {
  cuna2_plan plan;
  float best_ms = 0.f;
  if (cuna2_plan_create(&plan, CUNA2_F32, (int64_t)1 << 20, 4, 12) != CUNA2_SUCCESS) {
    fprintf(stderr, "cuna2: %s\n", cuna2_last_error());
    return 1;
  }
  /* once, on a representative input and before any graph capture */
  if (cuna2_plan_autotune(plan, t_d, y_d, F_d, n, t0, T, stream, 5, &best_ms) != CUNA2_SUCCESS ||
      cuna2_plan_set_graph(plan, 1) != CUNA2_SUCCESS) {
    fprintf(stderr, "cuna2: %s\n", cuna2_last_error());
    cuna2_plan_destroy(plan);
    return 1;
  }
  for (int i = 0; i < count; ++i)
    if (cuna2_adjoint(plan, t_d, y_d, F_d, n, t0, T, stream) != CUNA2_SUCCESS) {
      fprintf(stderr, "cuna2: %s\n", cuna2_last_error());
      break;
    }
  cuna2_plan_destroy(plan);
  printf("%lld bounded waits ran out\n", cuna2_wait_timeouts());
  return 0;
}
"""


def test_c_header_compiles_as_c(tmp_path):
    """include/cuna2.h is plain C: the accurate-mode example of the
    integration guide compiles as C11 with every warning an error."""
    import shutil
    import subprocess
    gcc = shutil.which("gcc")
    cuda_inc = "/usr/local/cuda/include"
    if not gcc or not os.path.exists(os.path.join(cuda_inc, "cuda_runtime.h")):
        pytest.skip("gcc or the CUDA headers are not installed")
    src = tmp_path / "example.c"
    src.write_text(_C_EXAMPLE)
    out = subprocess.run([gcc, "-std=c11", "-Wall", "-Werror", "-c", str(src), "-I", INC, "-I", cuda_inc,
                          "-o", str(tmp_path / "example.o")], capture_output=True, text=True)
    assert out.returncode == 0, out.stderr
