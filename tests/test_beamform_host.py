"""Host-side logic of the GPU beamformer (fastsimus_gb300.beamform), on the CPU: the f-number
rule, the filter design handed to fsg_rf2iq, and the Fortran pixel order of dasmtx rows."""

import math

import numpy as np
import pytest

torch = pytest.importorskip("torch")
scipy_signal = pytest.importorskip("scipy.signal")

from fastsimus_gb300 import beamform as B  # noqa: E402
from oracle import das_fp64 as D  # noqa: E402


@pytest.mark.parametrize("width", [1e-9, 0.1e-3, 0.27e-3, 0.6e-3])
def test_default_fnumber_matches_oracle(width):
    assert B.default_fnumber(width, 5.2e6, 1540.0) == pytest.approx(D.default_fnumber(width, 5.2e6, 1540.0), rel=1e-12)


@pytest.mark.parametrize("fs,bw", [(20e6, None), (31.25e6, 3e6)])
def test_lowpass_sections_are_the_rf2iq_butterworth(fs, bw):
    sos, zi = B._lowpass(fs, 5e6, bw)
    assert sos.shape == (3, 6) and zi.shape == (3, 2)
    assert np.all(sos[:, 3] == 1.0)
    b, a, _ = D.butter_lowpass(fs, 5e6, bw)
    x = np.random.default_rng(0).standard_normal(400)
    # same transfer function as the oracle's (b, a) form
    np.testing.assert_allclose(scipy_signal.sosfilt(sos, x), scipy_signal.lfilter(b, a, x), rtol=1e-9, atol=1e-11)
    # steady state: a constant input stays constant from the first sample
    y, _ = scipy_signal.sosfilt(sos, np.ones(50), zi=zi)
    np.testing.assert_allclose(y, np.ones(50), atol=1e-12)


def test_pixel_rows_follow_fortran_order_and_invert():
    x, z = np.meshgrid(np.arange(3.0), 10 + np.arange(4.0))  # (4, 3)
    pix, shape = B._pixels(x, z, torch.device("cpu"))
    assert shape == (4, 3)
    np.testing.assert_array_equal(pix[:, 0].numpy(), x.reshape(-1, order="F"))
    np.testing.assert_array_equal(pix[:, 1].numpy(), z.reshape(-1, order="F"))
    img = B._from_fortran(pix[:, 0] + 100 * pix[:, 1], shape)
    np.testing.assert_array_equal(img.numpy(), x + 100 * z)


def test_das_param_from_transducer_params():
    from fastsimus_gb300 import workloads as W

    p, m = W.cfg2_probe(), W.cfg2_medium()
    dp = B.DasParam.from_params(p, m)
    assert dp.Nelements == 128 and dp.fc == p.freq_center and dp.fs == 4 * p.freq_center
    assert dp.c == m.speed_of_sound and math.isinf(dp.radius)
