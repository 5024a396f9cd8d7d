"""Generate the golden vectors in tests/golden/*.npz.

Each fixture holds seeded inputs and the outputs of the reference library's
OWN sources (src/gaussian_filter.cu, src/gridding.cu, src/cuna_kernel.cu),
compiled for the CPU by oracle/build_ref.py and driven through
oracle.oracle.RefCPU:

    generate_filter_properties -> b, normfac, filter_radius, E1, E2, E3
    fast_gridding              -> grid   (f_hat after gridding, before the FFT)
    cunfft_adjoint_raw         -> F      (gridding + CUFFT_INVERSE + normalize)
    fast_gridding_bootstrap / cunfft_adjoint_raw_async_bootstrap for the
    bootstrap fixtures.

and, in tests/golden/host/, the reference's host-side functions
(src/utils.cu, src/cuna_kernel.cu:137-145):

    host_utils.npz   scale_x on float and double arrays (sorted, unsorted,
                     one and two elements, Julian dates) and nextPowerOfTwo
                     on edge values
    plan_*.npz       init_plan + cunfft_adjoint_from_plan, read back with
                     copyResultsToCPU (f_hat and, with
                     CALCULATE_WINDOW_FUNCTION, f_hat_win)

Run where the reference source tree is available (the fixtures it writes
are committed, so the tests need no reference tree):
    python oracle/build_ref.py && python tests/golden/make_golden.py [--host-only]
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
from oracle import build_ref  # noqa: E402
from oracle.oracle import RefCPU  # noqa: E402


def scaled_times(rng, n, sort=True):
    """Increasing times rescaled to [-1/2, 1/2] like scale_x (src/utils.cu:84-93)."""
    t = rng.uniform(0.0, 1.0, n)
    if sort:
        t = np.sort(t)
    return (t - t.min()) / (t.max() - t.min()) - 0.5 if n > 1 else np.zeros(1)


CASES = [
    # name, prec, n, ng, kind, options
    ("f32_n1000_ng2048", "f", 1000, 2048, "plain", {}),
    ("f32_cfg1_n10000_ng32768", "f", 10000, 32768, "plain", {"cfg1": True}),
    ("f64_n2000_ng8192", "d", 2000, 8192, "plain", {}),
    ("f64_n500_ng1024", "d", 500, 1024, "plain", {}),
    ("f32_window_n1000_ng2048", "f", 1000, 2048, "plain", {"window": True}),
    ("f32_nonpow2_n1000_ng3000", "f", 1000, 3000, "plain", {}),
    ("f32_edges_accumulate_n64_ng256", "f", 64, 256, "plain", {"edges": True, "accumulate": True}),
    ("f64_edges_accumulate_n64_ng256", "d", 64, 256, "plain", {"edges": True, "accumulate": True}),
    ("f32_single_sample_ng16", "f", 1, 16, "plain", {}),
    ("f32_boot_n500_ng1024_nbs8", "f", 500, 1024, "boot", {"nbs": 8, "seed": 12345}),
    ("f64_boot_n300_ng1024_nbs4", "d", 300, 1024, "boot", {"nbs": 4, "seed": 7}),
    ("f32_boot_edges_n64_ng256_nbs3", "f", 64, 256, "boot", {"nbs": 3, "seed": 4000000000, "edges": True}),
    ("f32_boot_window_n200_ng512_nbs2", "f", 200, 512, "boot", {"nbs": 2, "seed": 99, "window": True}),
]


def make_case(idx, name, prec, n, ng, kind, opt):
    rng = np.random.default_rng(1000 + idx)
    dt = np.float32 if prec == "f" else np.float64
    if opt.get("cfg1"):
        t = np.sort(rng.uniform(0.0, 1.0, n))
        x = (t - t[0]) / (t[-1] - t[0]) - 0.5
        y = np.sin(2 * np.pi * 137 * t) + rng.normal(0, 0.5, n)
    else:
        x = scaled_times(rng, n)
        y = np.cos(2 * np.pi * 10.0 * (x + 0.5) - 0.5) + rng.uniform(0, 1, n)
    if opt.get("edges"):
        # exact end points, values just outside [-1/2, 1/2] and a duplicate cell
        x[:6] = [-0.5, 0.5, -0.5000001, 0.5000001, -0.51, 0.53]
        x[6] = x[7]
    x = x.astype(dt)
    y = None if opt.get("window") else y.astype(dt)
    R = RefCPU(prec)
    out = {"x": x, "n": n, "ng": ng}
    if y is not None:
        out["y"] = y
    b, nf, rf, E1, E2, E3 = R.filter_properties(x, ng)
    out.update(b=b, normfac=nf, rf=rf, E1=E1, E2=E2, E3=E3)
    if kind == "plain":
        f0 = None
        if opt.get("accumulate"):
            ct = np.complex64 if prec == "f" else np.complex128
            f0 = (rng.normal(0, 0.1, ng) + 1j * rng.normal(0, 0.1, ng)).astype(ct)
            out["f_hat0"] = f0
        out["grid"] = R.fast_gridding(x, y, ng, f0)
        out["F"] = R.adjoint_raw(x, y, ng, f0)
        out["F_async"] = R.adjoint_raw(x, y, ng, f0, async_=True)
    else:
        nbs, seed = opt["nbs"], opt["seed"]
        out.update(nbs=nbs, seed=seed)
        out["grid"] = R.fast_gridding_bootstrap(x, y, ng, nbs, seed)
        out["F"] = R.adjoint_bootstrap(x, y, ng, nbs, seed)
    return out


HOST_DIR = os.path.join(HERE, "host")

SCALE_X_INPUTS = [
    [3.0, 4.0, 5.0, 7.0],
    [-0.5, -0.1, 0.2, 0.5],
    [0.0, 1.0],
    [42.0],
    [2451545.0, 2451545.25, 2451546.125, 2451600.0, 2451999.75],
    [5.0, 1.0, 3.0, 2.0],
]

PLAN_CASES = [
    # name, prec, n, ng, flags
    ("plan_f32_n1000_ng2048", "f", 1000, 2048, 0),
    ("plan_f32_window_n800_ng1024", "f", 800, 1024, 0x04),
    ("plan_f64_n600_ng2048", "d", 600, 2048, 0x04),
]


def make_host():
    os.makedirs(HOST_DIR, exist_ok=True)
    out = {}
    rng = np.random.default_rng(77)
    inputs = SCALE_X_INPUTS + [list(np.sort(rng.uniform(0, 100, 257))), list(rng.normal(0, 3, 64))]
    for prec, dt in (("f", np.float32), ("d", np.float64)):
        R = RefCPU(prec)
        for i, v in enumerate(inputs):
            x = np.asarray(v, dt)
            out["scale_x_%s_%d_in" % (prec, i)] = x
            out["scale_x_%s_%d_out" % (prec, i)] = R.scale_x(x)
    vals = np.array([0, 1, 2, 3, 4, 5, 7, 8, 9, 1000, 1023, 1024, 1025, 65535, 65536, 65537,
                     2 ** 30, 2 ** 30 + 1, 2 ** 31 - 1, 2 ** 31, 2 ** 31 + 1, 2 ** 32 - 1], np.uint64)
    out["next_pow2_in"] = vals.astype(np.uint32)
    out["next_pow2_out"] = np.array([RefCPU("f").next_power_of_two(int(v)) for v in vals], np.uint32)
    path = os.path.join(HOST_DIR, "host_utils.npz")
    np.savez_compressed(path, **out)
    print("wrote", os.path.relpath(path), os.path.getsize(path), "bytes")
    for idx, (name, prec, n, ng, flags) in enumerate(PLAN_CASES):
        rng = np.random.default_rng(500 + idx)
        dt = np.float32 if prec == "f" else np.float64
        x = scaled_times(rng, n).astype(dt)
        y = (np.sin(2 * np.pi * 7.0 * (x + 0.5)) + rng.normal(0, 0.3, n)).astype(dt)
        f, w = RefCPU(prec).plan_adjoint(x, y, ng, flags)
        rec = {"x": x, "y": y, "n": n, "ng": ng, "flags": flags, "f_hat": f}
        if w is not None:
            rec["f_hat_win"] = w
        path = os.path.join(HOST_DIR, name + ".npz")
        np.savez_compressed(path, **rec)
        print("wrote", os.path.relpath(path), os.path.getsize(path), "bytes")


def main():
    if not RefCPU.available("f") or not RefCPU.available("d"):
        if not build_ref.build(verbose=True):
            sys.exit("reference tree not available; cannot generate golden vectors")
    if "--host-only" not in sys.argv:
        for idx, (name, prec, n, ng, kind, opt) in enumerate(CASES):
            out = make_case(idx, name, prec, n, ng, kind, opt)
            path = os.path.join(HERE, name + ".npz")
            np.savez_compressed(path, **out)
            print("wrote", os.path.relpath(path), os.path.getsize(path), "bytes")
    make_host()


if __name__ == "__main__":
    main()
