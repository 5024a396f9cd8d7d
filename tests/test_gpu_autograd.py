"""GPU tests of the differentiable path: the hand-written backward
(cuna2_adjoint_backward, and cuna2_adjoint_backward_batch for a batch of 64
series) against the FP64 direct-sum gradient of the oracle, and autograd
through AdjointNFFTFunction against central finite differences (h = 1e-4) of
a float64 plan on the differentiable workload's shape.

Loss used by the autograd tests: L = sum_k w_k |F_k|^2, w_k ~ U[0, 1)."""
import numpy as np
import pytest
import torch

from conftest import rel_l2

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def mods(native_built):
    from cunfft_adjoint_gb300 import autograd, nfft
    return nfft, autograd


CASES = [
    # n, nf, R, m, dtype, tol            (small fused path / four-step path)
    (3000, 4096, 2, 8, torch.float32, 2e-5),
    (3000, 2048, 4, 12, torch.float64, 1e-9),
    (60000, 1 << 16, 2, 8, torch.float32, 2e-5),
    (40000, 1 << 15, 4, 12, torch.float64, 1e-9),
]


@pytest.mark.parametrize("n,nf,R,m,dtype,tol", CASES)
def test_backward_vs_fp64_gradient(mods, oracle_lib, n, nf, R, m, dtype, tol):
    nfft, _ = mods
    rng = np.random.default_rng(n + nf)
    T = 500.0
    t = np.sort(rng.uniform(0, T, n))
    y = rng.normal(0, 1, n)
    g = (rng.normal(0, 1, nf) + 1j * rng.normal(0, 1, nf))
    plan = nfft.AdjointNFFT(nf, R, m, dtype)
    td = torch.as_tensor(t, device="cuda")
    yd = torch.as_tensor(y, dtype=dtype, device="cuda")
    gd = torch.as_tensor(g, dtype=plan.cdtype, device="cuda")
    gy, gt = plan.backward(td, yd, gd, 0.0, T)
    torch.cuda.synchronize()
    sel = np.sort(rng.choice(n, 256, replace=False))
    k = np.arange(-nf // 2, nf // 2)
    ry, rt = oracle_lib.ndft_grad(t[sel], yd.cpu().numpy().astype(np.float64)[sel], 0.0, T, k, g)
    assert rel_l2(gy.cpu().numpy()[sel], ry) < tol
    assert rel_l2(gt.cpu().numpy()[sel], rt) < tol


def _loss(F, w):
    return (w * (F.real ** 2 + F.imag ** 2)).sum()


def test_autograd_matches_finite_differences(mods):
    """Central differences of L(y, t) with h = 1e-4 on 256 random coordinates
    of y and 256 of t, on the differentiable workload's shape (N = 2e5, t
    sorted in [0, 500), Nf = 2^18, R = 2, m = 10) with a float64 plan, whose
    kernel error (about exp(-pi m sqrt(1 - 1/R)) = 2e-10) leaves the
    differences meaningful."""
    nfft, ag = mods
    rng = np.random.default_rng(5)
    n, nf, T = 200_000, 1 << 18, 500.0
    t = torch.as_tensor(np.sort(rng.uniform(0, T, n)), device="cuda")
    y = torch.as_tensor(rng.normal(0, 1, n), device="cuda")
    w = torch.as_tensor(rng.uniform(0, 1, nf), device="cuda")
    plan = nfft.AdjointNFFT(nf, 2, 10, torch.float64)
    tt, yy = t.clone().requires_grad_(True), y.clone().requires_grad_(True)
    _loss(ag.adjoint_nfft(tt, yy, plan, 0.0, T), w).backward()
    h = 1e-4
    idx = rng.choice(n, 256, replace=False)

    def central(arr, j, step):
        a = arr.clone(); a[j] += step
        b = arr.clone(); b[j] -= step
        if arr is y:
            lp, lm = _loss(plan(t, a, 0.0, T), w), _loss(plan(t, b, 0.0, T), w)
        else:
            lp, lm = _loss(plan(a, y, 0.0, T), w), _loss(plan(b, y, 0.0, T), w)
        return float((lp - lm) / (2 * step))

    with torch.no_grad():
        fd_y = np.array([central(y, j, h) for j in idx])
        fd_t = np.array([central(t, j, h) for j in idx])
        fd_t2 = np.array([central(t, j, h / 2) for j in idx])
    # L is quadratic in y: the central difference is exact up to rounding
    assert rel_l2(yy.grad.cpu().numpy()[idx], fd_y) < 1e-6
    # in t the phase of the top frequency turns 2 pi (nf/2) h / T = 0.16 rad per
    # step, so the difference itself carries a third-derivative term of about
    # 1e-3; the Richardson combination (4 D(h/2) - D(h)) / 3 removes it
    gt = tt.grad.cpu().numpy()[idx]
    assert rel_l2(gt, fd_t) < 1e-2
    assert rel_l2(gt, (4 * fd_t2 - fd_t) / 3) < 5e-5


def test_autograd_float32_cfg5_shape(mods, oracle_lib):
    """N = 2e5, t sorted in [0, 500), Nf = 2^18, R = 2, m = 10, float32:
    autograd gradients of L = sum w |F|^2 against the FP64 direct-sum gradient
    (same upstream g = 2 w F) on 256 random coordinates."""
    nfft, ag = mods
    rng = np.random.default_rng(9)
    n, nf, T = 200_000, 1 << 18, 500.0
    t = np.sort(rng.uniform(0, T, n))
    y = rng.normal(0, 1, n).astype(np.float32)
    w = rng.uniform(0, 1, nf)
    plan = nfft.AdjointNFFT(nf, 2, 10, torch.float32)
    tt = torch.as_tensor(t, device="cuda").requires_grad_(True)
    yy = torch.as_tensor(y, device="cuda").requires_grad_(True)
    F = ag.adjoint_nfft(tt, yy, plan, 0.0, T)
    wd = torch.as_tensor(w, dtype=torch.float32, device="cuda")
    _loss(F, wd).backward()
    g = 2.0 * w * F.detach().cpu().numpy().astype(np.complex128)
    sel = np.sort(rng.choice(n, 256, replace=False))
    ry, rt = oracle_lib.ndft_grad(t[sel], y[sel].astype(np.float64), 0.0, T, np.arange(-nf // 2, nf // 2), g)
    assert rel_l2(yy.grad.cpu().numpy()[sel], ry) < 1e-4
    assert rel_l2(tt.grad.cpu().numpy()[sel], rt) < 1e-4


def test_batched_op_matches_per_series(mods):
    """BatchedAdjointNFFT (batched forward, batched VJP) equals the per-series
    autograd function for values and both gradients, on a batch of 64 series
    of the differentiable workload's shape (N = 2e5, Nf = 2^18, R = 2,
    m = 10, float32)."""
    nfft, ag = mods
    rng = np.random.default_rng(17)
    B, N, nf = 64, 200_000, 1 << 18
    t0 = rng.uniform(0, 10, B)
    T = rng.uniform(200, 500, B)
    t = torch.as_tensor(t0[:, None] + np.sort(rng.uniform(0, 1, (B, N)), axis=1) * T[:, None], device="cuda")
    y = torch.as_tensor(rng.normal(0, 1, (B, N)), dtype=torch.float32, device="cuda")
    w = torch.as_tensor(rng.uniform(0, 1, (B, nf)), dtype=torch.float32, device="cuda")
    op = ag.BatchedAdjointNFFT(B, N, nf, 2, 10, t0, T)
    tt, yy = t.clone().requires_grad_(True), y.clone().requires_grad_(True)
    F = op(tt, yy)
    _loss(F, w).backward()
    plan = nfft.AdjointNFFT(nf, 2, 10, torch.float32)
    for b in range(B):
        tb, yb = t[b].clone().requires_grad_(True), y[b].clone().requires_grad_(True)
        Fb = ag.adjoint_nfft(tb, yb, plan, t0[b], T[b])
        _loss(Fb, w[b]).backward()
        assert rel_l2(F[b].detach().cpu().numpy(), Fb.detach().cpu().numpy()) < 1e-6
        assert rel_l2(yy.grad[b].cpu().numpy(), yb.grad.cpu().numpy()) < 1e-6
        assert rel_l2(tt.grad[b].cpu().numpy(), tb.grad.cpu().numpy()) < 1e-6


def test_batched_gradients_vs_fp64(mods, oracle_lib):
    """The batched backward of 64 series (cuna2_adjoint_backward_batch) against
    the FP64 direct-sum gradient for 4 of the series on 256 coordinates each,
    with per-series t0 and T."""
    nfft, ag = mods
    rng = np.random.default_rng(23)
    B, N, nf = 64, 200_000, 1 << 18
    t0 = rng.uniform(0, 100, B)
    T = rng.uniform(400, 600, B)
    t = t0[:, None] + np.sort(rng.uniform(0, 1, (B, N)), axis=1) * T[:, None]
    y = rng.normal(0, 1, (B, N)).astype(np.float32)
    g = (rng.normal(0, 1, (B, nf)) + 1j * rng.normal(0, 1, (B, nf)))
    plan = nfft.AdjointNFFT(nf, 2, 10, torch.float32)
    gy, gt = plan.backward_batch(torch.as_tensor(t, device="cuda"), torch.as_tensor(y, device="cuda"),
                                 torch.as_tensor(g, dtype=torch.complex64, device="cuda"), t0, T)
    torch.cuda.synchronize()
    gy, gt = gy.cpu().numpy(), gt.cpu().numpy()
    k = np.arange(-nf // 2, nf // 2)
    for b in (0, 17, 40, 63):
        sel = np.sort(rng.choice(N, 256, replace=False))
        gc = g[b].astype(np.complex64).astype(np.complex128)
        ry, rt = oracle_lib.ndft_grad(t[b][sel], y[b][sel].astype(np.float64), t0[b], T[b], k, gc)
        assert rel_l2(gy[b][sel], ry) < 2e-5, b
        assert rel_l2(gt[b][sel], rt) < 2e-5, b
