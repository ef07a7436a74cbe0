"""Spectrum -> RF epilogue (``fsg_irfft_gate``, replacing the irfft + gate of
simus.py:336-367) against NumPy's FP64 irfft and the reference's gate formula."""

import numpy as np
import pytest

from tests import _golden as G
from tests._gpu import np64, require_gpu, torch

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _gpu():
    require_gpu()


class _Plan:
    def __init__(self, n_fft):
        self.n_fft = n_fft


def _spectrum(rng, n_full, E, k0, kc, nb=1):
    s = np.zeros((nb, n_full, E), dtype=np.complex128)
    s[:, k0:k0 + kc] = rng.standard_normal((nb, kc, E)) + 1j * rng.standard_normal((nb, kc, E))
    return s


def _ref_rf(s, n_fft, gate):
    rf = np.fft.irfft(np.conj(s), n=n_fft, axis=-2)[..., : (n_fft + 1) // 2, :]
    if gate:
        mag = np.abs(rf)
        rel = mag / (mag.max(axis=(-2, -1), keepdims=True) + 1e-30)
        rf = rf * 0.5 * (1.0 + np.tanh((rel - 1e-5) / 1e-6))
    return rf


@pytest.mark.parametrize("n_fft,k0,kc", [(2004, 180, 635), (3544, 310, 1142), (64, 0, 33), (63, 0, 32), (100, 40, 11)])
def test_irfft_matches_numpy(n_fft, k0, kc):
    from fastsimus_gb300.simus import irfft_and_threshold

    rng = np.random.default_rng(n_fft)
    n_full = n_fft // 2 + 1
    E = 70
    s = _spectrum(rng, n_full, E, k0, kc)[0]
    t = torch.as_tensor(s.astype(np.complex64), device="cuda")
    got = np64(irfft_and_threshold(t, _Plan(n_fft), k_first=k0, k_count=kc, gate=False))
    ref = _ref_rf(s.astype(np.complex64).astype(np.complex128), n_fft, gate=False)
    err = G.rel_l2(got, ref)
    print(f"n_fft {n_fft} band [{k0},{k0 + kc}): relL2 {err:.2e}")
    assert err < 2e-6
    # reading the whole spectrum (zeros outside the band) gives the same result
    full = np64(irfft_and_threshold(t, _Plan(n_fft), gate=False))
    assert G.rel_l2(full, ref) < 2e-6


def test_gate_per_frame_peak_batch():
    from fastsimus_gb300.simus import irfft_and_threshold

    rng = np.random.default_rng(3)
    n_fft, k0, kc, E = 2004, 180, 635, 64
    s = _spectrum(rng, n_fft // 2 + 1, E, k0, kc, nb=3)
    s[1] *= 1e3  # frames with very different peaks are gated independently
    s[2, :, :] *= np.exp(-np.arange(E) / 4.0)[None, :]
    s = s.astype(np.complex64).astype(np.complex128)
    t = torch.as_tensor(s.astype(np.complex64), device="cuda")
    got = np64(irfft_and_threshold(t, _Plan(n_fft), k_first=k0, k_count=kc))
    ref = _ref_rf(s, n_fft, gate=True)
    for b in range(3):
        err = G.rel_l2(got[b], ref[b])
        assert err < 2e-6, (b, err)


def test_simus_rf_uses_epilogue_and_matches_golden():
    import fastsimus_gb300 as F

    g = G.load("simus_cfg1_full")
    res = F.simus(g.scatterers, g.rc, g.delays, g.params, g.medium, fs=g.fs, tx_apodization=g.apod)
    err = G.rel_l2(np64(res.rf), g.rf)
    print(f"cfg1 RF through the epilogue: relL2 {err:.2e}")
    assert err < 1e-5
