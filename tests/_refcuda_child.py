"""Run the reference's own CUDA build (baseline/_ref/lib/<machine>/libcuna{f,d}.so,
made by oracle/build_ref_cuda.py) on request files and write its outputs.

Helper of tests/test_gpu_refcuda.py, run as a child process: the reference
library exports the same C++ names as this project's drop-in libraries and
terminates its process on any CUDA error, so it gets a process of its own.

    python tests/_refcuda_child.py <lib_dir> <request.npz> <out.npz> ...

A request holds: prec ('f' or 'd'), op ('adjoint', 'window' or
'bootstrap'), x, y, ng, and for the bootstrap nbs and seed.  The output
holds the filter properties (b, normfac, rf, E1, E2, E3), the result F of a
first call and `noise`, the relative L2 difference of a second, identical
call from the first (the reference sums with float atomics, so its own
results vary from run to run), and `max_noise`, the largest absolute
difference over the largest |F|.
"""
import ctypes
import os
import sys

import numpy as np
import torch


def _fields(dt):
    v = ctypes.c_float if dt == np.float32 else ctypes.c_double
    return [("b", v), ("normfac", v), ("filter_radius", ctypes.c_int), ("E1", ctypes.c_void_p),
            ("E2", ctypes.c_void_p), ("E3", ctypes.c_void_p)]


class FPf(ctypes.Structure):
    _fields_ = _fields(np.float32)


class FPd(ctypes.Structure):
    _fields_ = _fields(np.float64)


def _sym(lib, name, args):
    fn = getattr(lib, name)
    fn.restype = None
    fn.argtypes = args
    return fn


def run_case(lib_dir, req):
    prec = str(req["prec"])
    dt = np.float32 if prec == "f" else np.float64
    ct = torch.complex64 if prec == "f" else torch.complex128
    lib = ctypes.CDLL(os.path.join(lib_dir, "libcuna%s.so" % prec), mode=ctypes.RTLD_LOCAL)
    cudart = ctypes.CDLL("libcudart.so.13")
    cudart.cudaMemcpy.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int]
    P, I = ctypes.c_void_p, ctypes.c_int
    c = prec
    cx = "P6float2" if prec == "f" else "P7double2"
    gen = _sym(lib, "_Z26generate_filter_propertiesPK%siiPP17filter_propertiesS3_" % c, [P, I, I, P, P])
    raw = _sym(lib, "_Z18cunfft_adjoint_rawPK%sS0_%siiPK17filter_properties" % (c, cx), [P, P, P, I, I, P])
    boot = _sym(lib, "_Z34cunfft_adjoint_raw_async_bootstrapPK%sS0_%siiiPK17filter_propertiesP11CUstream_stj"
                % (c, cx), [P, P, P, I, I, I, P, P, ctypes.c_uint])
    free_fp = _sym(lib, "_Z22free_filter_propertiesP17filter_propertiesS0_", [P, P])
    x = torch.as_tensor(np.ascontiguousarray(req["x"], dt), device="cuda")
    op = str(req["op"])
    y = None if op == "window" else torch.as_tensor(np.ascontiguousarray(req["y"], dt), device="cuda")
    n, ng = x.numel(), int(req["ng"])
    h, d = P(), P()
    gen(x.data_ptr(), n, ng, ctypes.byref(h), ctypes.byref(d))
    fp = (FPf if prec == "f" else FPd).from_address(h.value)
    out = {"b": np.array(fp.b, dt), "normfac": np.array(fp.normfac, dt), "rf": np.array(fp.filter_radius)}
    for k, cnt in (("E1", n), ("E2", n), ("E3", fp.filter_radius)):
        a = np.empty(cnt, dt)
        assert cudart.cudaMemcpy(a.ctypes.data, getattr(fp, k), a.nbytes, 2) == 0
        out[k] = a
    runs = []
    for _ in range(2):
        if op == "bootstrap":
            nbs, seed = int(req["nbs"]), int(req["seed"])
            f = torch.zeros(nbs * ng, dtype=ct, device="cuda")
            boot(x.data_ptr(), y.data_ptr(), f.data_ptr(), n, ng, nbs, d, None, seed)
        else:
            f = torch.zeros(ng, dtype=ct, device="cuda")
            raw(x.data_ptr(), None if y is None else y.data_ptr(), f.data_ptr(), n, ng, d)
        torch.cuda.synchronize()
        runs.append(f)
    diff = runs[1] - runs[0]
    out["noise"] = np.array(float(torch.linalg.vector_norm(diff) / torch.linalg.vector_norm(runs[0])))
    out["max_noise"] = np.array(float(diff.abs().max() / runs[0].abs().max()))
    out["F"] = runs[0].cpu().numpy()
    free_fp(d, h)
    return out


def main():
    lib_dir = sys.argv[1]
    args = sys.argv[2:]
    for req_path, out_path in zip(args[0::2], args[1::2]):
        req = np.load(req_path)
        np.savez(out_path, **run_case(lib_dir, req))
    print("done", len(args) // 2)


if __name__ == "__main__":
    main()
