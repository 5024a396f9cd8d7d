"""Benchmark: adjoint NFFTs per second on one GB300 (and N replicas).

Workload (default, `--workload large`): one light curve of N = 1,000,000
samples in 10 seasonal windows of 200 d over 3650 d, y = three sinusoids
(periods 0.7, 3.3, 41 d; amplitudes 1, 0.3, 0.1) + N(0, 1) noise, Nf = 2^20
output frequencies, oversampling R = 4, Gaussian half-width m = 12, float32
gridding/FFT with the 64-bit fixed-point phase reduction (accurate mode).  A
step is one adjoint NFFT of one such input set.  16 independent input sets
(192 MB of t and y) rotate across steps, so the inputs of a step are not in
the 129 MB L2 from the previous use.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Multi-GPU: the transform of one light curve does not shard; `--gpus N` under
torchrun runs N independent replicas ("replicas only"), value = the sum.

The reference arm (`--impl reference`) times the reference's pipeline (its
compat arithmetic: R_f = 6 float filter, non-periodic grid of ng = R*Nf cells,
unnormalised inverse FFT, deconvolution) as the multi-threaded CPU program of
the oracle, on the host cores of the machine that runs the benchmark; the
reference has no CPU implementation of its own, and its CUDA sources are not
shipped with this package.
"""
import argparse
import json
import math
import os
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "adjoint NFFTs/sec & HBM GB/s on 1 GB300 at ≤1e-5 rel err vs FP64 NDFT, batched vs plain"
UNIT = "NFFT/s"

WORKLOADS = {
    "large": dict(n=1_000_000, nf=1 << 20, R=4, m=12, T=3650.0,
                  name="large single-series: N=1e6 in 10 seasonal windows over 3650 d, "
                       "Nf=2^20, R=4, m=12"),
    "plain": dict(n=10_000, nf=1 << 14, R=2, m=8, T=1.0,
                  name="plain single-series: N=1e4 sorted U[0,1), Nf=16384, R=2, m=8"),
}
NSETS = 16


def make_inputs(wl, seed, nsets):
    """nsets independent input sets of the workload (seeded)."""
    rng = np.random.default_rng(seed)
    n = wl["n"]
    ts, ys = [], []
    for _ in range(nsets):
        if wl is WORKLOADS["large"]:
            win = rng.integers(0, 10, n)
            t = win * 365.0 + rng.uniform(0, 200.0, n)
            y = (np.sin(2 * np.pi * t / 0.7) + 0.3 * np.sin(2 * np.pi * t / 3.3)
                 + 0.1 * np.sin(2 * np.pi * t / 41.0) + rng.normal(0, 1.0, n))
        else:
            t = np.sort(rng.uniform(0, 1.0, n))
            y = np.sin(2 * np.pi * 137 * t) + rng.normal(0, 0.5, n)
        ts.append(t)
        ys.append(y)
    return ts, ys


def ndft_check(t, y, F, nf, T, nbins=64, seed=0):
    """Relative L2 error of F on `nbins` random bins against a direct FP64 sum
    (numpy, chunked)."""
    rng = np.random.default_rng(seed)
    k = np.sort(rng.choice(np.arange(-nf // 2, nf // 2), nbins, replace=False))
    x = t / T - 0.5
    D = np.zeros(nbins, np.complex128)
    for a in range(0, len(x), 200_000):
        ph = np.outer(k, x[a:a + 200_000])
        ph -= np.rint(ph)
        D += np.exp(2j * np.pi * ph) @ y[a:a + 200_000].astype(np.float64)
    G = F[k + nf // 2].astype(np.complex128)
    return float(np.linalg.norm(G - D) / np.linalg.norm(D))


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during a timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index, interval_ms=50):
        self.index, self.interval = index, interval_ms
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q, "--format=csv,noheader,nounits",
                 "-lms", str(self.interval)], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
        time.sleep(0.15)
        return self

    def __exit__(self, *a):
        time.sleep(0.1)
        if self.proc:
            self.proc.terminate()
            try:
                self.out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                self.out = ""
        else:
            self.out = ""

    def summary(self):
        rows = [l.split(",") for l in self.out.strip().splitlines() if l.count(",") >= 8]
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"], "samples": 0}
        sm = [float(r[1]) for r in rows if r[1].strip().replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].strip().replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for r in rows:
            for nm, v in zip(names, r[5:9]):
                if "Active" in v and "Not" not in v:
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(rows)}


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def stage_bytes(n, ng, nf, rec_bytes=16, elem=4):
    """Algorithmic DRAM bytes per launch of each stage of the accurate path
    (float32 unless elem=8): every input read once, every output written
    once.  Records are duplicated for the ~2m/TL samples near tile edges;
    that factor is ignored (it is < 1%)."""
    L = ng // 2
    c = 2 * elem
    return {
        "bin_local": 8 * n + elem * n + rec_bytes * n,       # read t, y; write records (chunk-local order)
        "bin_count": 16 * n,                                 # read t; write the 64-bit phases
        "scan_tiles": 0,
        "bin_scatter": 8 * n + elem * n + rec_bytes * n,     # read phases, y; write records
        "grid": rec_bytes * n + elem * ng,                    # read records; write real grid
        "fft_colpass": 2 * c * L,                            # read + write the packed grid
        "fft_rowpass": c * L + c * nf,                       # read packed grid; write F
        "nfft_small": 8 * n + elem * n + c * nf,
    }


def batched_legs(dev, steps, which=("bootstrap", "uneven"), plain=True, batch_schedule=None, uneven_series=4096):
    """Batched forms: bootstrap (N=5000, 1024 resamples, Nf=32768, R=2, m=8)
    and an uneven batch (4096 series, N log-uniform in [100, 1e5], Nf =
    nextpow2(4N) capped at 2^18, R=2, m=8), float32, CUDA-graph replay.
    Returns NFFT/s for each (CUDA events, inputs resident)."""
    import torch
    from cunfft_adjoint_gb300.nfft import AdjointNFFT, BatchAdjointNFFT
    out = {}
    rng = np.random.default_rng(3)
    # bootstrap
    n, nbs, nf = 5000, 1024, 32768
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    if "bootstrap" in which:
        t = rng.uniform(0, 100.0, n)
        y = (np.sin(2 * np.pi * t / 2.1) + rng.normal(0, 0.3, n)).astype(np.float32)
        plan = AdjointNFFT(nf, 2, 8, torch.float32, device=dev)
        td, yd = torch.as_tensor(t, device=dev), torch.as_tensor(y, device=dev)
        F = torch.empty((nbs, nf), dtype=torch.complex64, device=dev)
        for i in range(3):
            plan.bootstrap(td, yd, nbs, i, 0.0, 100.0, out=F)
        # one CUDA graph replayed for every call, its draw seed updated per call
        plan.set_graph(True)
        for i in range(3):
            plan.bootstrap(td, yd, nbs, 100 + i, 0.0, 100.0, out=F)
        torch.cuda.synchronize()
        k = max(20, min(200, steps // 10))
        e0.record()
        for i in range(k):
            plan.bootstrap(td, yd, nbs, i, 0.0, 100.0, out=F)
        e1.record()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / k
        # algorithmic HBM bytes per call: draw weights written and read, t and y
        # read, records written and read, each resample's real grid written,
        # read and written by the column pass, read by the row pass, spectrum
        # written (the grids of 1024 resamples, 268 MB, exceed L2)
        ng = 2 * nf
        bcall = 8 * n * nbs + 12 * n + 32 * n + nbs * (16 * ng + 8 * nf)
        peak, pk = peaks()
        out["bootstrap"] = {"workload": "N=5000, 1024 resamples, Nf=32768, R=2, m=8", "value": nbs * 1000.0 / ms,
                            "unit": UNIT, "ms_per_call": ms, "calls": k,
                            "graph": "one captured graph per argument set, a new draw seed every call",
                            "hbm": {"algorithmic_bytes_per_call": bcall, "gbs": bcall / ms / 1e6,
                                    "frac_of_peak": bcall / ms / 1e6 / peak, "peak": peak, "peak_kind": pk}}
        if plain:
            # plain per-resample path: one single-series transform per resample
            # (resampled inputs prepared outside the timed region)
            plan.set_graph(False)  # eager single-series calls, one per resample
            draws = [rng.integers(0, n, n) for _ in range(max(64, min(256, steps // 8)))]
            tds = [td[torch.as_tensor(d, device=dev)] for d in draws]
            yds = [yd[torch.as_tensor(d, device=dev)] for d in draws]
            Fp = torch.empty(nf, dtype=torch.complex64, device=dev)
            for i in range(8):
                plan.adjoint(tds[i], yds[i], 0.0, 100.0, out=Fp)
            torch.cuda.synchronize()
            e0.record()
            for i in range(len(tds)):
                plan.adjoint(tds[i], yds[i], 0.0, 100.0, out=Fp)
            e1.record()
            torch.cuda.synchronize()
            msp = e0.elapsed_time(e1) / len(tds)
            out["bootstrap"]["plain_value"] = 1000.0 / msp
            out["bootstrap"]["batched_over_plain"] = out["bootstrap"]["value"] / (1000.0 / msp)
        del F, plan
    if "uneven" in which:
        # uneven batch (its own seeded stream)
        rng = np.random.default_rng(4)
        ns = uneven_series
        nser = np.exp(rng.uniform(np.log(100), np.log(1e5), ns)).astype(np.int64)
        nfs = np.minimum(2 ** np.ceil(np.log2(4 * nser)).astype(np.int64), 1 << 18)
        Ts = np.exp(rng.uniform(np.log(10), np.log(3000), ns))
        tt = np.concatenate([rng.uniform(0, Ts[i], nser[i]) for i in range(ns)])
        yy = rng.normal(0, 1, int(nser.sum())).astype(np.float32)
        bp = BatchAdjointNFFT(nser, nfs, 2, 8, np.zeros(ns), Ts, torch.float32, device=dev, graph=True)
        tdd, ydd = torch.as_tensor(tt, device=dev), torch.as_tensor(yy, device=dev)
        # the batch's own autotuner picks the tile size and gridding form,
        # unless the caller fixes them (launch lists of one schedule)
        if batch_schedule:
            bp.set_schedule(*batch_schedule)
            blt, bgm = bp.schedule
        else:
            blt, bgm, _ = bp.autotune(tdd, ydd, reps=3)
        FF = torch.empty(int(nfs.sum()), dtype=torch.complex64, device=dev)
        for i in range(3):
            bp(tdd, ydd, out=FF)
        torch.cuda.synchronize()
        k = max(20, min(100, steps // 20))
        e0.record()
        for i in range(k):
            bp(tdd, ydd, out=FF)
        e1.record()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / k
        # algorithmic HBM bytes per call: every series reads t and y and writes
        # its spectrum; series with grids above 2^15 cells (the one-CTA limit)
        # also write and read their records, write their grid, read and write
        # it in the column pass and read it in the row pass
        big = 2 * nfs > (1 << 15)
        bcall = int((12 * nser + 8 * nfs).sum() + (32 * nser[big] + 16 * 2 * nfs[big]).sum())
        peak, pk = peaks()
        out["uneven"] = {"workload": "%d series, N log-U[100,1e5] (total %d), Nf=nextpow2(4N)<=2^18, R=2, m=8"
                         % (ns, int(nser.sum())), "value": ns * 1000.0 / ms, "unit": UNIT, "ms_per_call": ms, "calls": k,
                         "schedule": {"log_tile": blt, "grid_method": ["gather", "scatter", "fixed"][bgm]},
                         "graph": True,
                         "hbm": {"algorithmic_bytes_per_call": bcall, "gbs": bcall / ms / 1e6,
                                 "frac_of_peak": bcall / ms / 1e6 / peak, "peak": peak, "peak_kind": pk}}
        if not plain:
            return out
        # plain per-series path: one single-series plan call per series (plans
        # cached per Nf, inputs resident), same series
        plans = {}
        offs = np.concatenate([[0], np.cumsum(nser)])
        foffs = np.concatenate([[0], np.cumsum(nfs)])
        def plain_all():
            for i in range(ns):
                p_ = plans.get(int(nfs[i]))
                if p_ is None:
                    p_ = plans[int(nfs[i])] = AdjointNFFT(int(nfs[i]), 2, 8, torch.float32, device=dev)
                p_.adjoint(tdd[offs[i]:offs[i + 1]], ydd[offs[i]:offs[i + 1]], 0.0, float(Ts[i]),
                           out=FF[foffs[i]:foffs[i + 1]])
        plain_all()
        torch.cuda.synchronize()
        e0.record()
        plain_all()
        e1.record()
        torch.cuda.synchronize()
        msp = e0.elapsed_time(e1)
        out["uneven"]["plain_value"] = ns * 1000.0 / msp
        out["uneven"]["batched_over_plain"] = out["uneven"]["value"] / out["uneven"]["plain_value"]
    return out


def autograd_leg(dev, steps):
    """Differentiable path: a batch of 64 series (N=2e5 sorted on [0,500),
    Nf=2^18, R=2, m=10, float32), loss sum_k w_k |F_k|^2, forward + backward
    (dL/dt, dL/dy) per step; CUDA events, inputs resident."""
    import torch
    from cunfft_adjoint_gb300.autograd import BatchedAdjointNFFT
    B, N, nf, T = 64, 200_000, 1 << 18, 500.0
    rng = np.random.default_rng(5)
    t = torch.as_tensor(np.sort(rng.uniform(0, T, (B, N)), axis=1), device=dev)
    y = torch.as_tensor(rng.normal(0, 1, (B, N)).astype(np.float32), device=dev)
    w = torch.as_tensor(rng.uniform(0, 1, (B, nf)).astype(np.float32), device=dev)
    op = BatchedAdjointNFFT(B, N, nf, 2, 10, np.zeros(B), np.full(B, T), torch.float32, dev)

    def step():
        tt, yy = t.detach().requires_grad_(True), y.detach().requires_grad_(True)
        F = op(tt, yy)
        (w * (F.real ** 2 + F.imag ** 2)).sum().backward()
        return tt.grad, yy.grad

    for _ in range(3):
        step()
    torch.cuda.synchronize()
    k = max(20, min(100, steps // 20))
    a0, a1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a0.record()
    for _ in range(k):
        step()
    a1.record()
    torch.cuda.synchronize()
    ms = a0.elapsed_time(a1) / k
    # plain per-series path: the single-series differentiable function, one
    # forward and one backward per series
    from cunfft_adjoint_gb300.autograd import adjoint_nfft
    from cunfft_adjoint_gb300.nfft import AdjointNFFT
    plan = AdjointNFFT(nf, 2, 10, torch.float32, device=dev)

    def plain_step():
        for b in range(B):
            tb, yb = t[b].detach().requires_grad_(True), y[b].detach().requires_grad_(True)
            F = adjoint_nfft(tb, yb, plan, 0.0, T)
            (w[b] * (F.real ** 2 + F.imag ** 2)).sum().backward()

    plain_step()
    torch.cuda.synchronize()
    kp = max(5, min(20, steps // 100))
    a0.record()
    for _ in range(kp):
        plain_step()
    a1.record()
    torch.cuda.synchronize()
    msp = a0.elapsed_time(a1) / kp
    return {"workload": "64 series x N=2e5, Nf=2^18, R=2, m=10, loss sum w|F|^2, forward + backward (t, y)",
            "value": B * 1000.0 / ms, "unit": "series/s (forward+backward)", "ms_per_batch": ms, "steps": k,
            "plain_value": B * 1000.0 / msp, "plain_ms_per_batch": msp, "plain_steps": kp,
            "batched_over_plain": msp / ms,
            "plain": "per series: the single-series autograd function, one forward and one backward"}


def cpu_baseline(wl, budget_s=20.0):
    """The reference pipeline on the host cores (oracle CPU program)."""
    from oracle import oracle
    n, ng = wl["n"], wl["R"] * wl["nf"]
    ts, ys = make_inputs(wl, 99, 1)
    t = ts[0]
    x = ((t - t.min()) / (t.max() - t.min()) - 0.5).astype(np.float32)
    y = ys[0].astype(np.float32)
    p = oracle.CpuPipeline(n, ng)
    p.run(x, y)  # warm-up (page-in, thread pool)
    done, t0 = 0, time.perf_counter()
    while True:
        p.run(x, y)
        done += 1
        el = time.perf_counter() - t0
        if el > budget_s or done >= 50:
            break
    return {"value": done / el, "unit": UNIT, "cores": oracle.num_threads(), "kind": "port",
            "sample": "%d transforms of the workload (N=%d, ng=%d, reference compat math, float) "
                      "by the oracle's multi-threaded CPU pipeline" % (done, n, ng),
            "seconds": round(el, 3), "beside": cpu_beside(wl, t, ys[0])}


def cpu_beside(wl, t, y, budget_s=1.5):
    """Rows reported beside the CPU baseline, each a bounded sample on the
    same host cores: the CPU pipeline on the plain (N = 1e4, ng = 32768) and
    bootstrap-resample (N = 5000, ng = 65536) shapes, the FP64 direct NDFT of
    the large workload (256 frequencies, rate extrapolated to all Nf) and
    scipy's FFT of the large grid as a cross-check of the FFT share."""
    from oracle import oracle
    out = {}

    def rate(fn):
        fn()
        done, t0 = 0, time.perf_counter()
        while True:
            fn()
            done += 1
            el = time.perf_counter() - t0
            if el > budget_s or done >= 200:
                return done / el

    rng = np.random.default_rng(5)
    for tag, n, ng in (("plain_nfft_per_s", 10_000, 32768), ("bootstrap_resamples_per_s", 5000, 65536)):
        x = rng.uniform(-0.5, 0.5, n).astype(np.float32)
        v = rng.normal(0, 1, n).astype(np.float32)
        p = oracle.CpuPipeline(n, ng)
        out[tag] = rate(lambda: p.run(x, v))
    k = np.arange(-128, 128)
    t0 = time.perf_counter()
    oracle.ndft(t, y, 0.0, wl["T"], k)
    el = time.perf_counter() - t0
    out["ndft_fp64_seconds_per_transform"] = el * wl["nf"] / len(k)
    try:
        import scipy.fft
        g = (rng.normal(size=wl["R"] * wl["nf"]) + 0j).astype(np.complex64)
        out["scipy_fft_ms"] = 1000.0 / rate(lambda: scipy.fft.ifft(g, workers=oracle.num_threads()))
    except ImportError:
        out["scipy_fft_ms"] = None
    return out


def reference_cuda_leg(dev, steps, wl):
    """The reference's OWN CUDA build (baseline/_ref, compiled for sm_103a by
    oracle/build_ref_cuda.py from its sources with its Makefile's flags) on
    the workload's inputs in the reference's units (x = t/T - 1/2, float,
    ng = R*nf, its fixed filter radius 6), timed with CUDA events:

    * as_is: cunfft_adjoint_raw_async as it ships, a cuFFT plan created and
      destroyed inside every call (src/cuna_kernel.cu:188-232);
    * kernels: its gridding and normalisation kernels (performGridding,
      normalizeResults, src/cuna_kernel.cu:52-117) around one cuFFT C2C
      inverse whose plan is made once -- the reference's arithmetic without
      its per-call plan;
    * bootstrap: cunfft_adjoint_raw_async_bootstrap, 1024 resamples of
      N = 5000 on ng = 65536 (src/cuna_kernel.cu:236-289);

    beside this library's drop-in entry points (cuna2_compat_adjoint_f32,
    cuna2_compat_bootstrap_f32) on the same inputs, with the relative L2
    difference of the two results."""
    import ctypes
    import platform
    import torch
    from cunfft_adjoint_gb300 import _lib
    libdir = os.path.join(ROOT, "baseline", "_ref", "lib", platform.machine())
    path = os.path.join(libdir, "libcunaf.so")
    if not os.path.exists(path):
        return {"unavailable": "the reference's CUDA build is not in baseline/_ref (oracle/build_ref_cuda.py)"}
    ref = ctypes.CDLL(path, mode=ctypes.RTLD_LOCAL)
    P, I = ctypes.c_void_p, ctypes.c_int
    gen = ref._Z26generate_filter_propertiesPKfiiPP17filter_propertiesS3_
    gen.argtypes, gen.restype = [P, I, I, P, P], None
    raw = ref._Z24cunfft_adjoint_raw_asyncPKfS0_P6float2iiPK17filter_propertiesP11CUstream_st
    raw.argtypes, raw.restype = [P, P, P, I, I, P, P], None
    boot = ref._Z34cunfft_adjoint_raw_async_bootstrapPKfS0_P6float2iiiPK17filter_propertiesP11CUstream_stj
    boot.argtypes, boot.restype = [P, P, P, I, I, I, P, P, ctypes.c_uint], None
    init_plan = ref._Z9init_planP4planPKfS2_iij
    init_plan.argtypes, init_plan.restype = [P, P, P, I, I, ctypes.c_uint], None
    grid = ref._Z15performGriddingP4plan
    norm = ref._Z16normalizeResultsP4plan
    free_plan = ref._Z9free_planP4plan
    for f in (grid, norm, free_plan):
        f.argtypes, f.restype = [P], None
    cufft = ctypes.CDLL("libcufft.so.12")
    L = _lib.core()
    n, nf, R, T = wl["n"], wl["nf"], wl["R"], wl["T"]
    ng = R * nf
    ts, ys = make_inputs(wl, 4242, 1)
    x_h = (ts[0] / T - 0.5).astype(np.float32)
    y_h = ys[0].astype(np.float32)
    x = torch.as_tensor(x_h, device=dev)
    y = torch.as_tensor(y_h, device=dev)
    st = torch.cuda.default_stream(dev)  # the reference's kernels run on the legacy default stream
    K = max(10, min(50, steps))

    def timed(fn, k):
        for _ in range(3):
            fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(st)
        for _ in range(k):
            fn()
        e1.record(st)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / k

    with torch.cuda.stream(st):
        h, d = P(), P()
        gen(x.data_ptr(), n, ng, ctypes.byref(h), ctypes.byref(d))
        f_ref = torch.zeros(ng, dtype=torch.complex64, device=dev)
        raw(x.data_ptr(), y.data_ptr(), f_ref.data_ptr(), n, ng, d, None)
        f_ref2 = torch.zeros(ng, dtype=torch.complex64, device=dev)
        raw(x.data_ptr(), y.data_ptr(), f_ref2.data_ptr(), n, ng, d, None)
        fp = _lib.FilterPropertiesF32()
        E = [torch.empty(k, dtype=torch.float32, device=dev) for k in (n, n, 6)]
        fp.E1, fp.E2, fp.E3 = E[0].data_ptr(), E[1].data_ptr(), E[2].data_ptr()
        dfp = torch.zeros(ctypes.sizeof(fp), dtype=torch.uint8, device=dev)
        _lib.check(L.cuna2_compat_filter_f32(x.data_ptr(), n, ng, ctypes.byref(fp), dfp.data_ptr(), None))
        f_ours = torch.zeros(ng, dtype=torch.complex64, device=dev)
        _lib.check(L.cuna2_compat_adjoint_f32(x.data_ptr(), y.data_ptr(), f_ours.data_ptr(), n, ng,
                                              dfp.data_ptr(), None))
        torch.cuda.synchronize()
        a, b = f_ours.cpu().numpy().astype(np.complex128), f_ref.cpu().numpy().astype(np.complex128)
        parity = float(np.linalg.norm(a - b) / np.linalg.norm(b))
        noise = float(np.linalg.norm(f_ref2.cpu().numpy().astype(np.complex128) - b) / np.linalg.norm(b))
        del f_ref2
        as_is = timed(lambda: raw(x.data_ptr(), y.data_ptr(), f_ref.data_ptr(), n, ng, d, None), K)
        ours = timed(lambda: _lib.check(L.cuna2_compat_adjoint_f32(x.data_ptr(), y.data_ptr(), f_ours.data_ptr(),
                                                                    n, ng, dfp.data_ptr(), None)), K)
        # the reference's kernels around a cuFFT plan made once
        libc = ctypes.CDLL(None)
        libc.malloc.restype = P
        libc.malloc.argtypes = [ctypes.c_size_t]
        pp = libc.malloc(96)
        init_plan(pp, x_h.ctypes.data, y_h.ctypes.data, n, ng, 0)
        g_f_hat = ctypes.c_void_p.from_address(pp + 32).value
        hplan = ctypes.c_int()
        assert cufft.cufftPlan1d(ctypes.byref(hplan), ng, 0x29, 1) == 0  # CUFFT_C2C
        exec_c2c = cufft.cufftExecC2C
        exec_c2c.argtypes = [ctypes.c_int, P, P, I]

        def kernels():
            grid(pp)
            exec_c2c(hplan.value, g_f_hat, g_f_hat, 1)  # CUFFT_INVERSE
            norm(pp)

        kern = timed(kernels, K)
        cufft.cufftDestroy(hplan.value)
        free_plan(pp)
        # bootstrap: 1024 resamples of N = 5000 on ng = 65536
        nb, nbs, ngb = 5000, 1024, 65536
        rng = np.random.default_rng(77)
        tb = rng.uniform(0, 100, nb)
        xb = torch.as_tensor(((tb - tb.min()) / (tb.max() - tb.min()) - 0.5).astype(np.float32), device=dev)
        yb = torch.as_tensor((np.sin(2 * np.pi * tb / 2.1) + rng.normal(0, 0.3, nb)).astype(np.float32), device=dev)
        hb, db = P(), P()
        gen(xb.data_ptr(), nb, ngb, ctypes.byref(hb), ctypes.byref(db))
        fb_ref = torch.zeros(nbs * ngb, dtype=torch.complex64, device=dev)
        boot(xb.data_ptr(), yb.data_ptr(), fb_ref.data_ptr(), nb, ngb, nbs, db, None, 7)
        fpb = _lib.FilterPropertiesF32()
        Eb = [torch.empty(k, dtype=torch.float32, device=dev) for k in (nb, nb, 6)]
        fpb.E1, fpb.E2, fpb.E3 = Eb[0].data_ptr(), Eb[1].data_ptr(), Eb[2].data_ptr()
        dfpb = torch.zeros(ctypes.sizeof(fpb), dtype=torch.uint8, device=dev)
        _lib.check(L.cuna2_compat_filter_f32(xb.data_ptr(), nb, ngb, ctypes.byref(fpb), dfpb.data_ptr(), None))
        fb_ours = torch.zeros(nbs * ngb, dtype=torch.complex64, device=dev)
        _lib.check(L.cuna2_compat_bootstrap_f32(xb.data_ptr(), yb.data_ptr(), fb_ours.data_ptr(), nb, ngb, nbs,
                                                dfpb.data_ptr(), 7, None))
        torch.cuda.synchronize()
        bpar = float(torch.linalg.vector_norm(fb_ours - fb_ref) / torch.linalg.vector_norm(fb_ref))
        kb = max(5, min(20, steps))
        b_ref = timed(lambda: boot(xb.data_ptr(), yb.data_ptr(), fb_ref.data_ptr(), nb, ngb, nbs, db, None, 7), kb)
        b_ours = timed(lambda: _lib.check(L.cuna2_compat_bootstrap_f32(
            xb.data_ptr(), yb.data_ptr(), fb_ours.data_ptr(), nb, ngb, nbs, dfpb.data_ptr(), 7, None)), kb)
        del fb_ref, fb_ours
    return {
        "build": "reference sources compiled for sm_103a with its Makefile flags (--use_fast_math, -rdc, "
                 "BLOCK_SIZE=256), cuFFT %s" % "12",
        "workload": "%s; reference units: x = t/T - 1/2 (float32), ng = %d, filter radius 6" % (wl["name"], ng),
        "as_is": {"ms_per_call": as_is, "value": 1000.0 / as_is, "unit": UNIT, "calls": K,
                  "note": "cuFFT plan created and destroyed inside every call, as the reference does"},
        "kernels": {"ms_per_call": kern, "value": 1000.0 / kern, "unit": UNIT, "calls": K,
                    "note": "performGridding + cufftExecC2C (plan made once) + normalizeResults"},
        "ours_dropin": {"ms_per_call": ours, "value": 1000.0 / ours, "unit": UNIT,
                        "api": "cuna2_compat_adjoint_f32 (the drop-in's arithmetic)"},
        "ours_over_as_is": as_is / ours, "ours_over_kernels": kern / ours,
        "parity_rel_l2": parity, "reference_noise_floor": noise,
        "bootstrap": {"resamples": nbs, "n": nb, "ng": ngb, "reference_ms_per_call": b_ref, "ours_ms_per_call": b_ours,
                      "reference_resamples_per_s": nbs * 1000.0 / b_ref, "ours_resamples_per_s": nbs * 1000.0 / b_ours,
                      "ours_over_reference": b_ref / b_ours, "parity_rel_l2": bpar},
    }


def dist_setup(backend):
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch.distributed as dist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group(backend)
    return ws, rank, local


def max_over_ranks(ms, ws, device=None):
    """The slowest rank's time (the contract's max over ranks); ws == 1: ms."""
    if ws <= 1:
        return ms
    import torch
    import torch.distributed as dist
    t = torch.tensor([ms], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_value(ms, steps, ws):
    """Whole-job NFFT/s: every rank runs `steps` transforms in the max time."""
    return ws * steps / (ms / 1000.0)


def reference_arm(args, wl):
    ws, rank, local = int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0")), 0
    if rank != 0:
        return
    from oracle import oracle
    n, ng = wl["n"], wl["R"] * wl["nf"]
    ts, ys = make_inputs(wl, 7, 2)
    xs = [((t - t.min()) / (t.max() - t.min()) - 0.5).astype(np.float32) for t in ts]
    yv = [y.astype(np.float32) for y in ys]
    p = oracle.CpuPipeline(n, ng)
    t_est = time.perf_counter()
    p.run(xs[0], yv[0])
    one = time.perf_counter() - t_est
    for w in range(min(args.warmup, 2)):
        p.run(xs[w % 2], yv[w % 2])
    steps = args.steps
    cap = max(1, int(120.0 / max(one, 1e-6)))
    timed = min(steps, cap)
    t0 = time.perf_counter()
    for s in range(timed):
        p.run(xs[s % 2], yv[s % 2])
    el = time.perf_counter() - t0
    value = timed / el
    sample = ("%d transforms (N=%d, ng=%d, reference compat math, float) by the oracle's "
              "multi-threaded CPU pipeline%s" % (timed, n, ng, "" if timed == steps else
                                                 "; %d of %d requested steps, capped at ~120 s" % (timed, steps)))
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": timed, "warmup": args.warmup, "ms_per_step": 1000.0 * el / timed,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded)",
            "config": {"workload": wl["name"], "n": n, "ng": ng, "nf": wl["nf"], "R": wl["R"],
                       "cache": "two input sets alternate; CPU run"},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": oracle.num_threads(), "kind": "port",
                             "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def f64_leg(dev, args, wl, ts, ys, td, stream):
    """The same workload through a float64 plan (graph replay, one stream)."""
    import torch
    from cunfft_adjoint_gb300 import _lib
    from cunfft_adjoint_gb300.nfft import AdjointNFFT
    L = _lib.core()
    nf, R, m, T = wl["nf"], wl["R"], wl["m"], wl["T"]
    plan64 = AdjointNFFT(nf, R, m, torch.float64, device=dev)
    yd64 = [torch.as_tensor(y, dtype=torch.float64, device=dev) for y in ys[:4]]
    if not args.no_autotune:
        plan64.autotune(td[0], yd64[0], 0.0, T, reps=2)
    if not args.no_graph:
        _lib.check(L.cuna2_plan_set_graph(plan64._h, 1))
    n64 = len(yd64)
    F64 = torch.empty(nf, dtype=torch.complex128, device=dev)
    with torch.cuda.stream(stream):
        for s in range(8):
            plan64.adjoint(td[s % n64], yd64[s % n64], 0.0, T, out=F64)
    torch.cuda.synchronize()
    k64 = max(10, min(200, args.steps // 10))
    a0, a1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with torch.cuda.stream(stream):
        a0.record(stream)
        for s in range(k64):
            plan64.adjoint(td[s % n64], yd64[s % n64], 0.0, T, out=F64)
        a1.record(stream)
    torch.cuda.synchronize()
    ms64 = a0.elapsed_time(a1) / k64
    err64 = ndft_check(ts[0], ys[0], plan64.adjoint(td[0], yd64[0], 0.0, T).cpu().numpy(), nf, T)
    return {"value": 1000.0 / ms64, "unit": UNIT, "ms_per_step": ms64, "rel_err_vs_fp64_ndft": err64, "steps": k64}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--warmup", type=int, default=50)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="large", choices=sorted(WORKLOADS))
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-graph", action="store_true")
    ap.add_argument("--no-autotune", action="store_true")
    ap.add_argument("--streams", type=int, default=3, help="concurrent streams, one plan each")
    ap.add_argument("--no-side-legs", action="store_true", help="skip the float64 and batched legs")
    ap.add_argument("--only", choices=["bootstrap", "uneven", "autograd", "f64"],
                    help="run one batched leg alone (no plain leg) and print its result")
    ap.add_argument("--nsets", type=int, default=NSETS, help="rotating input sets (default 16: 192 MB > L2)")
    ap.add_argument("--batch-schedule", default=None, metavar="LOG_TILE,FORM",
                    help="uneven leg: this schedule (e.g. 12,fixed) instead of the batch autotuner")
    ap.add_argument("--uneven-series", type=int, default=4096,
                    help="uneven leg: number of series (fewer for small profiler captures)")
    args = ap.parse_args()
    if args.batch_schedule:
        lt_, gm_ = args.batch_schedule.split(",")
        args.batch_schedule = (int(lt_), {"gather": 0, "scatter": 1, "fixed": 2}[gm_])
    wl = WORKLOADS[args.workload]
    if args.impl == "reference":
        return reference_arm(args, wl)
    if args.only == "f64":
        import torch
        dev = torch.device("cuda", 0)
        ts, ys = make_inputs(wl, 0, 4)
        td = [torch.as_tensor(t, device=dev) for t in ts]
        print(json.dumps(f64_leg(dev, args, wl, ts, ys, td, torch.cuda.Stream(dev))), flush=True)
        return
    if args.only:
        import torch
        dev = torch.device("cuda", 0)
        res = autograd_leg(dev, args.steps) if args.only == "autograd" else \
            batched_legs(dev, args.steps, (args.only,), plain=False, batch_schedule=args.batch_schedule,
                         uneven_series=args.uneven_series)[args.only]
        print(json.dumps(res), flush=True)
        return

    import torch
    from cunfft_adjoint_gb300 import _lib
    from cunfft_adjoint_gb300.nfft import AdjointNFFT

    ws, rank, local = dist_setup("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    n, nf, R, m, T = wl["n"], wl["nf"], wl["R"], wl["m"], wl["T"]
    ng = R * nf
    nsets = max(1, args.nsets)
    ts, ys = make_inputs(wl, 1000 + rank, nsets)
    td = [torch.as_tensor(t, dtype=torch.float64, device=dev) for t in ts]
    yd = [torch.as_tensor(y.astype(np.float32), device=dev) for y in ys]
    nstr = max(1, args.streams)
    Fd = [torch.empty(nf, dtype=torch.complex64, device=dev) for _ in range(nstr)]
    plan = AdjointNFFT(nf, R, m, torch.float32, device=dev)
    L = _lib.core()
    # the plan's own autotuner picks the tile size and gridding form on input set 0
    schedule = plan.autotune(td[0], yd[0], 0.0, T, reps=5)[:2] if not args.no_autotune else plan.schedule
    # independent series stream through one plan per CUDA stream (a plan's
    # workspace serves one stream at a time); the others copy the schedule
    plans = [plan] + [AdjointNFFT(nf, R, m, torch.float32, device=dev) for _ in range(nstr - 1)]
    streams = [torch.cuda.current_stream(dev)] + [torch.cuda.Stream(dev) for _ in range(nstr - 1)]
    for p_ in plans[1:]:
        _lib.check(L.cuna2_plan_set_schedule(p_._h, *plan.schedule))
        _lib.check(L.cuna2_plan_set_binning(p_._h, plan.binning))
    if not args.no_graph:
        for p_ in plans:
            _lib.check(L.cuna2_plan_set_graph(p_._h, 1))
    stream = streams[0]

    def step(s, ns=nstr):
        k = s % ns
        _lib.check(L.cuna2_adjoint(plans[k]._h, td[s % nsets].data_ptr(), yd[s % nsets].data_ptr(),
                                   Fd[k].data_ptr(), n, 0.0, T, streams[k].cuda_stream))

    # every (plan, input set) pair gets its graph before timing
    for s in range(max(args.warmup, 3) + nsets * nstr):
        step(s)
    for s in range(nsets):
        step(s, 1)
    torch.cuda.synchronize()
    # accuracy of one output against a direct FP64 sum
    err = ndft_check(ts[0], ys[0].astype(np.float32), plan.adjoint(td[0], yd[0], 0.0, T).cpu().numpy(), nf, T)

    def timed(ns, k):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(streams[0])
        for st in streams[1:ns]:
            st.wait_event(e0)
        for s in range(k):
            step(s, ns)
        for st in streams[1:ns]:
            ev = torch.cuda.Event()
            ev.record(st)
            streams[0].wait_event(ev)
        e1.record(streams[0])
        torch.cuda.synchronize()
        return e0.elapsed_time(e1)

    if ws > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        ms = timed(nstr, args.steps)
    ms = max_over_ranks(ms, ws, dev)
    if ws > 1:
        torch.distributed.barrier()
    ms_step = ms / args.steps
    value = replica_value(ms, args.steps, ws)
    ms1 = timed(1, args.steps) / args.steps  # one stream: the per-transform latency

    # per-launch durations: cuna2_plan_profile replays the transform as a CUDA
    # graph with an event node after every launch (launches serialised), so
    # each duration is one kernel's, timed on the device; a 512 MB read ahead
    # of each replay evicts the inputs from L2, as in the timed loop
    import ctypes
    stage_ms = (ctypes.c_float * 16)()
    names = (ctypes.c_char_p * 16)()
    nst = ctypes.c_int()
    acc = {}
    reps = 10
    evict = torch.zeros(128 << 20, dtype=torch.float32, device=dev)
    for r in range(reps):
        s = (r * 5) % nsets
        with torch.cuda.stream(stream):
            evict.sum()
        _lib.check(L.cuna2_plan_profile(plan._h, td[s].data_ptr(), yd[s].data_ptr(), Fd[0].data_ptr(), n, 0.0, T,
                                        stream.cuda_stream or None, stage_ms, names, 16, ctypes.byref(nst)))
        for i in range(nst.value):
            acc.setdefault(names[i].decode(), []).append(stage_ms[i])
    stages = {k: float(np.median(v)) for k, v in acc.items()}
    # every profiled interval includes one event node's gap: take it out
    gap = stages.pop("event_gap", 0.0)
    stages = {k: max(v - gap, 0.0) for k, v in stages.items()}
    # the gridding kernel's own launch time (the roofline's kernel): one
    # transform in which the gridding launch repeats back to back between two
    # events on the plan's stream, on the records of that transform
    gms = ctypes.c_float()
    grid_runs = []
    for r in range(5):
        s = (r * 3) % nsets
        with torch.cuda.stream(stream):
            evict.sum()
        _lib.check(L.cuna2_plan_time_grid(plan._h, td[s].data_ptr(), yd[s].data_ptr(), Fd[0].data_ptr(), n, 0.0, T,
                                          50, stream.cuda_stream or None, ctypes.byref(gms)))
        grid_runs.append(gms.value)
    grid_ms = float(np.median(grid_runs))
    del evict

    # comparator: cuFFT's real-to-complex transform of the same ng-point real
    # grid (torch.fft.rfft), L2-resident like the grid our two passes work on;
    # ours also unpack, deconvolve and centre the spectrum
    g_real = torch.randn(ng, device=dev)
    with torch.cuda.stream(stream):
        for _ in range(5):
            torch.fft.rfft(g_real)
        c0, c1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        c0.record(stream)
        for _ in range(50):
            torch.fft.rfft(g_real)
        c1.record(stream)
    torch.cuda.synchronize()
    fft_cmp = {"cufft_r2c_ms": c0.elapsed_time(c1) / 50,
               "ours_ms": stages.get("fft_colpass", 0.0) + stages.get("fft_rowpass", 0.0),
               "points": ng, "note": "cuFFT R2C alone; ours includes unpack, deconvolution and centring"}
    del g_real
    sb = stage_bytes(n, ng, nf)
    dom = "grid"  # the largest share of the transform in the launch lists (profiles/)
    peak, peak_kind = peaks()
    ach = sb.get(dom, 0) / (grid_ms * 1e-3) / 1e9
    # DRAM bytes per gridding launch, from the one-pass ncu launch list of
    # the same bench command with this stream count (profiles/)
    traffic, traffic_src = None, None
    tfile = os.path.join(ROOT, "profiles", "traffic_large.json")
    if os.path.exists(tfile):
        tj = json.load(open(tfile))
        entry = tj.get("streams_%d" % nstr)
        if entry:
            traffic = entry.get(dom)
            traffic_src = "%s (%d streams)" % (tj.get("source", "profiles/traffic_large.json"), nstr)
    total_bytes = sum(sb[k] for k in stages if k in sb)
    kernels_per_step = len([k for k in stages if k != "start"])

    # e2e: the same transforms through the host-buffer C-ABI entry from pinned
    # host arrays, H2D copy of t, y and D2H copy of F inside every step: a
    # stream of series spread over the same plans and streams
    # (cuna2_adjoint_host_async), so one series' copies overlap another's
    # transform, as a caller streaming many series would run it
    th = [torch.as_tensor(t).pin_memory() for t in ts[:4]]
    yh = [torch.as_tensor(y.astype(np.float32)).pin_memory() for y in ys[:4]]
    nh = len(th)
    e2e_steps = max(1, min(args.steps, 200))
    hplans, hstreams = plans, streams
    nh2 = nstr
    Fh = [torch.empty(nf, dtype=torch.complex64).pin_memory() for _ in range(nh2)]

    def host_step(s):
        k = s % nh2
        _lib.check(L.cuna2_adjoint_host_async(hplans[k]._h, th[s % nh].data_ptr(), yh[s % nh].data_ptr(),
                                              Fh[k].data_ptr(), n, 0.0, T, hstreams[k].cuda_stream))

    for s in range(8):
        host_step(s)
    torch.cuda.synchronize()
    h0, h1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    h0.record(hstreams[0])
    for st in hstreams[1:]:
        st.wait_event(h0)
    for s in range(e2e_steps):
        host_step(s)
    for st in hstreams[1:]:
        j1 = torch.cuda.Event()
        j1.record(st)
        hstreams[0].wait_event(j1)
    h1.record(hstreams[0])
    torch.cuda.synchronize()
    e2e_ms = h0.elapsed_time(h1) / e2e_steps
    # the host link's own floor for the same bytes: the same copies on the
    # same streams with no transform between them
    tdev = [torch.empty(n, dtype=torch.float64, device=dev) for _ in range(nh2)]
    ydev = [torch.empty(n, dtype=torch.float32, device=dev) for _ in range(nh2)]
    fdev = [torch.empty(nf, dtype=torch.complex64, device=dev) for _ in range(nh2)]

    def copy_step(s):
        k = s % nh2
        with torch.cuda.stream(hstreams[k]):
            tdev[k].copy_(th[s % nh], non_blocking=True)
            ydev[k].copy_(yh[s % nh], non_blocking=True)
            Fh[k].copy_(fdev[k], non_blocking=True)

    for s in range(8):
        copy_step(s)
    torch.cuda.synchronize()
    copy_ms = None
    for _ in range(2):  # the better of two runs: a floor
        h0.record(hstreams[0])
        for st in hstreams[1:]:
            st.wait_event(h0)
        for s in range(e2e_steps):
            copy_step(s)
        for st in hstreams[1:]:
            j1 = torch.cuda.Event()
            j1.record(st)
            hstreams[0].wait_event(j1)
        h1.record(hstreams[0])
        torch.cuda.synchronize()
        c_ms = h0.elapsed_time(h1) / e2e_steps
        copy_ms = c_ms if copy_ms is None else min(copy_ms, c_ms)
    del tdev, ydev, fdev
    # the blocking single-call form, for reference
    for s in range(3):
        _lib.check(L.cuna2_adjoint_host(plan._h, th[s % nh].data_ptr(), yh[s % nh].data_ptr(), Fh[0].data_ptr(), n,
                                        0.0, T, stream.cuda_stream or None))
    b0 = time.perf_counter()
    nb = max(1, min(args.steps, 50))
    for s in range(nb):
        _lib.check(L.cuna2_adjoint_host(plan._h, th[s % nh].data_ptr(), yh[s % nh].data_ptr(), Fh[0].data_ptr(), n,
                                        0.0, T, stream.cuda_stream or None))
    blocking_ms = (time.perf_counter() - b0) * 1000.0 / nb

    # float64 side by side (same workload, double plan)
    f64 = f64_leg(dev, args, wl, ts, ys, td, stream) if rank == 0 and not args.no_side_legs else None

    r1 = reference_cuda_leg(dev, args.steps, wl) if rank == 0 and not args.no_side_legs else None

    batched = batched_legs(dev, args.steps) if rank == 0 and not args.no_side_legs else None
    if batched is not None:
        batched["autograd"] = autograd_leg(dev, args.steps)

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        cpu = cpu_baseline(wl)

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
            "config": {"workload": wl["name"], "n": n, "nf": nf, "R": R, "m": m, "ng": ng,
                       "mode": "accurate (fixed-point phase, float32 gridding+FFT)",
                       "cache": "%d rotating input sets (%.0f MB of t,y; L2 is 129 MB)" %
                                (nsets, nsets * n * 12 / 1e6),
                       "graph": not args.no_graph, "parallelism": "replicas" if ws > 1 else "single",
                       "streams": nstr,
                       "schedule": {"log_tile": schedule[0],
                                    "grid_method": ["gather", "scatter", "fixed"][schedule[1]]}},
            "rel_err_vs_fp64_ndft": err,
            "single_stream": {"value": ws * 1000.0 / ms1, "ms_per_step": ms1},
            "roofline": {"bound": "hbm", "kernel": "grid (k_grid_acc, gather gridding)", "achieved": ach,
                         "peak": peak, "peak_kind": peak_kind, "unit": "GB/s", "frac": ach / peak,
                         "traffic": traffic, "traffic_source": traffic_src,
                         "algorithmic_bytes": sb.get(dom, 0),
                         "kernel_ms": grid_ms,
                         "timing": "mean of 50 back-to-back launches of the gridding kernel on one transform's "
                                   "records, CUDA events on the plan's stream (cuna2_plan_time_grid), median of 5"},
            "stages_ms": stages,
            "stages_note": "per-launch device time, launches serialised (graph replay with an event after each "
                           "launch, the event nodes' own gap of %.4f ms taken out); the timed step overlaps "
                           "launches (dependent launch) and streams, so the stages sum to more than "
                           "ms_per_step" % gap,
            "pipeline_gbs": total_bytes / (ms_step * 1e-3) / 1e9,
            # compulsory traffic only: t and y in, the spectrum out
            "compulsory_gbs": (n * 12 + nf * 8) / (ms_step * 1e-3) / 1e9,
            # reported, not a roofline: 2m taps x 3 flops per sample (recurrence
            # product + fused multiply-add) + 5 L log2 L for the packed L = ng/2
            # complex FFT
            "flops_per_transform": 2 * m * 3 * n + 5 * (ng // 2) * int(np.log2(ng // 2)),
            "tflops": (2 * m * 3 * n + 5 * (ng // 2) * int(np.log2(ng // 2))) / (ms_step * 1e-3) / 1e12,
            "fft_vs_cufft": fft_cmp,
            "e2e": {"value": 1000.0 / e2e_ms, "unit": UNIT, "ms_per_step": e2e_ms, "steps": e2e_steps,
                    "h2d_bytes_per_step": n * 12, "d2h_bytes_per_step": nf * 8,
                    "copy_only_ms_per_step": copy_ms, "frac_of_copy_bound": copy_ms / e2e_ms,
                    "api": "cuna2_adjoint_host_async, one plan per stream, %d streams, pinned host buffers" % nstr,
                    "blocking_call_ms": blocking_ms},
            "gpu_launches": kernels_per_step * args.steps,
            "clocks": clk.summary(),
            "f64": f64,
            "r1_reference_cuda": r1,
            "batched": batched,
            "cpu_baseline": cpu,
        }
        print(json.dumps(line), flush=True)
    if ws > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
