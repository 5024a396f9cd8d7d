"""GPU tests of the multi-channel transform (fused window-function channel)
and of the generalised Lomb-Scargle periodogram built on it."""
import numpy as np
import pytest
import torch

from conftest import rel_l2

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def mods(native_built):
    from cunfft_adjoint_gb300 import lombscargle, nfft
    return nfft, lombscargle


@pytest.mark.parametrize("n,nf", [(3000, 4096), (100_000, 1 << 17)])
def test_multi_channel_equals_single_and_window(mods, oracle_lib, n, nf):
    nfft, _ = mods
    rng = np.random.default_rng(n)
    t = rng.uniform(0, 50.0, n)
    y = rng.normal(0, 1, n).astype(np.float32)
    plan = nfft.AdjointNFFT(nf, 2, 8, torch.float32)
    td = torch.as_tensor(t, device="cuda")
    Y = torch.stack([torch.as_tensor(y, device="cuda"), torch.ones(n, device="cuda")])
    F = plan.multi(td, Y, 0.0, 50.0)
    F0 = plan(td, Y[0], 0.0, 50.0)
    torch.cuda.synchronize()
    assert rel_l2(F[0].cpu().numpy(), F0.cpu().numpy()) < 1e-6
    k = np.sort(rng.choice(np.arange(-nf // 2, nf // 2), 256, replace=False))
    W = oracle_lib.ndft(t, np.ones(n), 0.0, 50.0, k)
    assert rel_l2(F[1].cpu().numpy()[k + nf // 2], W) < 1e-5


def _ls_direct(t, y, dy, freqs):
    w = 1.0 / dy ** 2
    w = w / w.sum()
    ybar = (w * y).sum()
    YY = (w * (y - ybar) ** 2).sum()
    P = np.empty(len(freqs))
    for a in range(0, len(freqs), 256):
        om = 2 * np.pi * freqs[a:a + 256, None]
        c, s = np.cos(om * t), np.sin(om * t)
        YC = (w * (y - ybar) * c).sum(1)
        YS = (w * (y - ybar) * s).sum(1)
        C, S = (w * c).sum(1), (w * s).sum(1)
        CC = (w * c * c).sum(1) - C * C
        SS = (w * s * s).sum(1) - S * S
        CS = (w * c * s).sum(1) - C * S
        D = CC * SS - CS * CS
        P[a:a + 256] = (SS * YC ** 2 + CC * YS ** 2 - 2 * CS * YC * YS) / (YY * D)
    return P


@pytest.mark.parametrize("dtype,tol", [(torch.float64, 1e-8), (torch.float32, 1e-4)])
def test_lomb_scargle_vs_direct(mods, dtype, tol):
    _, ls = mods
    rng = np.random.default_rng(3)
    n, nfreq = 2000, 3000
    t = np.sort(rng.uniform(0, 100.0, n))
    dy = rng.uniform(0.2, 0.6, n)
    y = np.sin(2 * np.pi * t / 2.1) + rng.normal(0, 1, n) * dy
    df = 1.0 / (5 * 100.0)
    P = ls.lomb_scargle(torch.as_tensor(t, device="cuda"), torch.as_tensor(y, dtype=dtype, device="cuda"),
                        torch.as_tensor(dy, dtype=dtype, device="cuda"), nfreq, df, t0=0.0,
                        m=12 if dtype == torch.float64 else 8, R=4 if dtype == torch.float64 else 2)
    torch.cuda.synchronize()
    freqs = df * np.arange(1, nfreq + 1)
    D = _ls_direct(t, y, dy, freqs)
    assert rel_l2(P.cpu().numpy(), D) < tol
    # the injected period is the highest peak
    assert abs(freqs[int(np.argmax(P.cpu().numpy()))] - 1 / 2.1) < 2 * df
