"""CPU checks of the beamforming oracle (oracle/das_fp64.py): envelope recovery by rf2iq,
the f-number rule, and a point target imaged at its position by rf2iq + DAS."""

from math import pi

import numpy as np

from oracle import das_fp64 as D

FC, FS, C = 5e6, 20e6, 1540.0


def test_rf2iq_recovers_envelope_and_phase():
    n = np.arange(1200)
    t = n / FS
    env = np.exp(-(((t - 30e-6) / 6e-6) ** 2))
    phi = 0.7
    rf = (env * np.cos(2 * pi * FC * t + phi))[:, None] * np.array([1.0, -2.0])
    iq = D.rf2iq(rf, FS, FC)
    mid = slice(400, 800)
    assert np.allclose(np.abs(iq[mid, 0]), env[mid], atol=2e-3)
    assert np.allclose(iq[mid, 1], -2.0 * iq[mid, 0], atol=1e-12)
    peak = np.argmax(np.abs(iq[:, 0]))
    assert abs(np.angle(iq[peak, 0] * np.exp(-1j * phi))) < 1e-2


def test_default_fnumber_limits():
    # a point-like element radiates like cos(theta): -3 dB at 45 degrees, f-number 1/2
    assert abs(D.default_fnumber(1e-9, FC, C) - 0.5) < 1e-9
    # wider elements are more directive: larger f-number
    lam = C / FC
    assert D.default_fnumber(lam, FC, C) > D.default_fnumber(lam / 2, FC, C) > 0.5


def _point_target_iq(n_el, pitch, pos, delays, n_s):
    """I/Q of a point scatterer at pos for one firing: a Gaussian-enveloped tone arriving at
    (d_tx + d_rx) / c on each element, demodulated by the oracle."""
    xe = (np.arange(n_el) - (n_el - 1) / 2) * pitch
    d_rx = np.hypot(pos[0] - xe, pos[1])
    d_tx = np.min(C * delays + d_rx)
    t = np.arange(n_s)[:, None] / FS
    tau = (d_tx + d_rx)[None, :] / C
    rf = np.exp(-(((t - tau) / 0.3e-6) ** 2)) * np.cos(2 * pi * FC * (t - tau))
    return D.rf2iq(rf, FS, FC)


def test_point_target_is_imaged_at_its_position():
    n_el, pitch = 32, 0.3e-3
    pos = (1.2e-3, 12e-3)
    xe = (np.arange(n_el) - (n_el - 1) / 2) * pitch
    frames, delays = [], []
    for ang in (-5.0, 0.0, 5.0):
        d = xe * np.sin(np.deg2rad(ang)) / C
        d -= d.min()
        delays.append(d)
        frames.append(_point_target_iq(n_el, pitch, pos, d, 500))
    xs = np.linspace(-3e-3, 3e-3, 61)
    zs = np.linspace(9e-3, 15e-3, 61)
    x, z = np.meshgrid(xs, zs)
    img = D.das(np.stack(frames), x, z, np.stack(delays), n_elements=n_el, pitch=pitch, radius=np.inf, c=C,
                fs=FS, fc=FC, fnumber=1.0)
    iz, ix = np.unravel_index(np.argmax(np.abs(img)), img.shape)
    assert abs(xs[ix] - pos[0]) <= 1.5 * (xs[1] - xs[0]) and abs(zs[iz] - pos[1]) <= 1.5 * (zs[1] - zs[0])
