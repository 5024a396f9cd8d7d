"""GPU tests of the differentiable path: the hand-written backward
(cuna2_adjoint_backward) against the FP64 direct-sum gradient of the oracle,
and autograd through AdjointNFFTFunction against central finite differences
(h = 1e-4) of a float64 plan.

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
    (float64 plan, four-step path)."""
    nfft, ag = mods
    rng = np.random.default_rng(5)
    n, nf, T = 20000, 1 << 14, 500.0
    t = torch.as_tensor(np.sort(rng.uniform(0, T, n)), device="cuda")
    y = torch.as_tensor(rng.normal(0, 1, n), device="cuda")
    w = torch.as_tensor(rng.uniform(0, 1, nf), device="cuda")
    plan = nfft.AdjointNFFT(nf, 2, 12, torch.float64)
    tt, yy = t.clone().requires_grad_(True), y.clone().requires_grad_(True)
    _loss(ag.adjoint_nfft(tt, yy, plan, 0.0, T), w).backward()
    h = 1e-4
    idx = rng.choice(n, 128, replace=False)
    fd_y, fd_t = [], []
    with torch.no_grad():
        for j in idx:
            for arr, out in ((y, fd_y), (t, fd_t)):
                a = arr.clone(); a[j] += h
                b = arr.clone(); b[j] -= h
                if arr is y:
                    lp = _loss(plan(t, a, 0.0, T), w); lm = _loss(plan(t, b, 0.0, T), w)
                else:
                    lp = _loss(plan(a, y, 0.0, T), w); lm = _loss(plan(b, y, 0.0, T), w)
                out.append(float((lp - lm) / (2 * h)))
    assert rel_l2(yy.grad.cpu().numpy()[idx], np.array(fd_y)) < 1e-6
    # central differences carry h^2 f'''/6 ~ 2e-5 relative for frequencies up to nf/(2T)
    assert rel_l2(tt.grad.cpu().numpy()[idx], np.array(fd_t)) < 1e-4


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
    """BatchedAdjointNFFT (batched forward, per-series VJP) equals the
    per-series autograd function for values and both gradients."""
    nfft, ag = mods
    rng = np.random.default_rng(17)
    B, N, nf = 6, 20000, 1 << 14
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
