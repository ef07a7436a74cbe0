"""GPU beamforming (fastsimus_gb300.beamform, libfsgb300 fsg_rf2iq / fsg_das / fsg_dasmtx)
against the FP64 oracle (oracle/das_fp64.py), plus simus -> rf2iq -> das on a point target.

Tolerances: rf2iq runs its IIR filter in FP32 (rel-L2 <= 2e-5 against scipy's FP64 filtfilt);
delay-and-sum forms distances and I/Q phases in FP32, whose rounding at ~400 wavelengths of
path is ~1e-4 rad (rel-L2 <= 1e-3)."""

import math

import numpy as np
import pytest

from oracle import das_fp64 as D
from tests._gpu import np64, require_gpu, torch

pytestmark = pytest.mark.gpu

FC, C = 5e6, 1540.0


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.mark.parametrize("fs,bw,tau", [(20e6, None, 0.0), (31.25e6, 3e6, 1.3e-6)])
def test_rf2iq_matches_oracle(fs, bw, tau):
    require_gpu()
    from fastsimus_gb300.beamform import rf2iq

    rng = np.random.default_rng(3)
    rf = rng.standard_normal((3, 700, 24)).astype(np.float32)
    got = np64(rf2iq(torch.as_tensor(rf, device="cuda"), fs, FC, bw, tau))
    for f in range(3):
        ref = D.rf2iq(rf[f].astype(np.float64), fs, FC, bw, tau)
        assert _rel(got[f], ref) < 2e-5
    one = np64(rf2iq(rf[1], fs, FC, bw, tau))
    assert one.shape == (700, 24)
    assert _rel(one, got[1]) < 1e-7


def _setup(n_el=24, radius=math.inf, n_s=600, n_frames=3, seed=5):
    rng = np.random.default_rng(seed)
    pitch = 0.3e-3
    iq = (rng.standard_normal((n_frames, n_s, n_el)) + 1j * rng.standard_normal((n_frames, n_s, n_el)))
    xe, ze, _ = D.element_frame(n_el, pitch, radius)
    delays = []
    for k, ang in enumerate(np.linspace(-8, 8, n_frames)):
        d = (xe * np.sin(np.deg2rad(ang)) + ze * np.cos(np.deg2rad(ang))) / C
        d = d - d.min()
        if k == 1:
            d[3] = np.nan  # an element that does not fire
        delays.append(d)
    xs = np.linspace(-3e-3, 3.5e-3, 20)
    zs = np.linspace(4e-3, 16e-3, 16)
    x, z = np.meshgrid(xs, zs)
    return iq, np.stack(delays), x, z, pitch


@pytest.mark.parametrize("method", ["linear", "nearest"])
@pytest.mark.parametrize("fnumber", [1.7, 0.0, None])
@pytest.mark.parametrize("radius", [math.inf, 40e-3])
def test_das_matches_oracle(method, fnumber, radius):
    require_gpu()
    from fastsimus_gb300.beamform import DasParam, das

    fs = 20e6
    iq, delays, x, z, pitch = _setup(radius=radius)
    param = DasParam(fc=FC, pitch=pitch, Nelements=24, width=0.25e-3, radius=radius, c=C, fs=fs, fnumber=fnumber)
    fn = D.default_fnumber(0.25e-3, FC, C) if fnumber is None else fnumber
    got = np64(das(torch.as_tensor(iq.astype(np.complex64), device="cuda"), x, z, delays, param, method))
    q = iq.astype(np.complex64).astype(np.complex128)
    ref = D.das(q, x, z, delays, n_elements=24, pitch=pitch, radius=radius, c=C, fs=fs, fc=FC, fnumber=fn,
                method=method)
    assert got.shape == x.shape
    if method == "linear":
        assert _rel(got, ref) < 1e-3
    else:
        # nearest sample: a tap whose fractional sample lies within FP32 rounding (~1e-4
        # sample) of k + 1/2 may round the other way; with white test signals one such tap
        # moves its pixel by O(1).  Most pixels agree to FP32 rounding; the few others move
        # the whole image by ~1e-2.
        err = np.abs(got - ref) / np.maximum(np.abs(ref), 1e-3 * np.abs(ref).max())
        assert np.median(err) < 1e-4 and np.mean(err > 1e-3) < 0.05
        assert _rel(got, ref) < 3e-2


@pytest.mark.parametrize("method", ["linear", "nearest"])
def test_dasmtx_matches_oracle_and_das(method):
    require_gpu()
    from fastsimus_gb300.beamform import DasParam, das, dasmtx

    fs = 20e6
    iq, delays, x, z, pitch = _setup()
    q = iq.astype(np.complex64)
    param = DasParam(fc=FC, pitch=pitch, Nelements=24, width=0.25e-3, c=C, fs=fs, fnumber=1.2, TXdelay=delays[1])
    m = dasmtx(1j * np.array(q[1].shape), x, z, param, method)
    assert m.layout == torch.sparse_csr and m.shape == (x.size, 600 * 24)
    # the signal itself (a GPU tensor) instead of its shape gives the same matrix
    m_t = dasmtx(torch.as_tensor(q[1], device="cuda"), x, z, param, method)
    assert torch.equal(m_t.values(), m.values()) and torch.equal(m_t.col_indices(), m.col_indices())
    dense = np64(m.to_dense())
    # oracle rows are in C order of the grid; the matrix's in Fortran order, as pymust.dasmtx's
    ref = D.das_weights(600, x.reshape(-1, order="F"), z.reshape(-1, order="F"), delays[1], n_elements=24,
                        pitch=pitch, radius=math.inf, c=C, fs=fs, fc=FC, fnumber=1.2, method=method)
    if method == "linear":
        assert np.max(np.abs(dense - ref)) < 2e-3 * np.max(np.abs(ref))
    else:  # taps at rounding ties may pick the neighbouring sample (see test_das_matches_oracle)
        assert np.mean(np.abs(dense - ref) > 2e-3 * np.max(np.abs(ref))) < 1e-4
    # the reference's usage: (M @ iq.flatten(order="F")).reshape(grid, order="F") equals das
    # (das rotates by transmit and receive phases separately, the matrix by their sum: both
    # FP32, so they agree to the FP32 phase rounding of each)
    vec = torch.as_tensor(q[1].reshape(-1, order="F"), device="cuda")
    img_m = np64(m @ vec).reshape(x.shape, order="F")
    img = np64(das(torch.as_tensor(q[1], device="cuda"), x, z, delays[1], param, method))
    assert _rel(img_m, img) < (2e-4 if method == "linear" else 3e-2)


def test_simus_rf2iq_das_images_a_point_scatterer():
    require_gpu()
    from fastsimus_gb300 import simus_compute, simus_precompute
    from fastsimus_gb300 import workloads as W
    from fastsimus_gb300.beamform import DasParam, das, rf2iq

    p, m = W.cfg1_probe(), W.cfg1_medium()
    pos = np.array([[1.5e-3, 14e-3]])
    fs = 4 * p.freq_center
    delays = [np.asarray(d, dtype=np.float64) for d in W.plane_wave_delays(p, m, [-6.0, 0.0, 6.0])]
    plan = simus_precompute(pos, np.ones(1), delays[0], p, m, fs=fs)  # one plan: equal record lengths
    frames = [simus_compute(pos, np.ones(1), d, plan, p, m).rf for d in delays]
    fs = plan.n_fft * float(plan.selected_freqs[1] - plan.selected_freqs[0])  # the RF's exact sample rate
    iq = rf2iq(torch.stack(frames), fs, p.freq_center)
    xs = np.linspace(-2e-3, 5e-3, 71)
    zs = np.linspace(11e-3, 17e-3, 61)
    x, z = np.meshgrid(xs, zs)
    img = np64(das(iq, x, z, np.stack(delays), DasParam.from_params(p, m, fs=fs)).abs())
    iz, ix = np.unravel_index(np.argmax(img), img.shape)
    lam = m.speed_of_sound / p.freq_center
    assert abs(xs[ix] - pos[0, 0]) < lam and abs(zs[iz] - pos[0, 1]) < lam / 2


def test_bad_arguments_raise():
    require_gpu()
    from fastsimus_gb300.beamform import DasParam, das, rf2iq

    with pytest.raises(ValueError):
        rf2iq(np.zeros((10, 4), np.float32), 20e6, FC)  # fewer samples than the filter padding
    param = DasParam(fc=FC, pitch=0.3e-3, Nelements=8, width=0.25e-3, c=C, fs=20e6)
    with pytest.raises(ValueError):
        das(np.zeros((100, 7), np.complex64), np.zeros(3), np.ones(3), np.zeros(7), param)  # wrong channel count
    with pytest.raises(ValueError):
        das(np.zeros((100, 8), np.complex64), np.zeros(3), np.ones(3), np.zeros(8), param, method="cubic")
