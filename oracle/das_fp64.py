"""FP64 NumPy restatement of the beamforming that consumes simulated RF (test infrastructure only).

The reference's validation tests turn simulated RF into images with PyMUST
(``tests/_picmus_phantom_shared.py:407-460``): ``pymust.rf2iq(rf, fs, fc)`` per firing, then
``pymust.dasmtx(1j * iq.shape, x_grid, z_grid, param)`` and a sparse product with the IQ
flattened in Fortran order, summed over firings.  PyMUST (``pymust==0.1.9``, ``uv.lock:2135-2137``)
is not installed here, so this module restates the published MUST algorithms (Garcia,
MUST toolbox, ``rf2iq`` and ``dasmtx``) as this package implements them; parity with PyMUST
itself is unpinned.

* ``rf2iq``: down-mixing by ``exp(-2 pi i fc (n / fs + tau))``, then a zero-phase 5th-order
  Butterworth low-pass with normalised cut-off ``Wn = min(2 fc / fs, 0.5)`` (or ``B / fs`` for a
  given bandwidth B in Hz) applied forward and backward (``scipy.signal.filtfilt``, odd
  padding of ``3 (order + 1)`` samples, steady-state initial conditions), times 2.
* ``dasmtx``: for pixel p and element e, transmit distance
  ``d_tx(p) = min_e (c tau_e + |p - x_e|)`` over the elements that fire (NaN delay = off),
  receive distance ``|p - x_e|``, delay ``t = (d_tx + d_rx) / c``, fractional sample
  ``s = (t - t0) fs`` (0-based), linear interpolation between samples floor(s) and floor(s) + 1
  (or the nearest sample), both inside the record; for I/Q signals the weight is multiplied by
  ``exp(2 pi i fc t)``.  Receive aperture: the element takes part when the pixel lies in front
  of it with ``|lateral| <= axial / (2 f#)`` in the element's frame (``f# <= 0``: every element).
  The column of sample i of element e is ``e n_samples + i`` (Fortran order of the
  ``(n_samples, n_elements)`` signal).
* default f-number: ``1 / (2 tan(alpha))`` with alpha the angle at which the soft-baffle element
  directivity ``sinc(w sin(alpha) / lambda) cos(alpha)`` at fc falls to ``1 / sqrt(2)``.
"""

from __future__ import annotations

from math import asin, atan2, cos, inf, isinf, pi, sin, sqrt, tan

import numpy as np
import scipy.signal


def butter_lowpass(fs, fc, bandwidth=None, order=5):
    """Coefficients (b, a) and steady-state initial conditions of the rf2iq low-pass."""
    wn = min(2.0 * fc / fs, 0.5) if bandwidth is None else bandwidth / fs
    b, a = scipy.signal.butter(order, wn)
    return b, a, scipy.signal.lfilter_zi(b, a)


def rf2iq(rf, fs, fc, bandwidth=None, tau=0.0):
    """I/Q components of RF ``(n_samples, n_channels)`` (complex128, same shape)."""
    rf = np.asarray(rf, dtype=np.float64)
    n = rf.shape[0]
    t = np.arange(n) / fs + tau
    iq = rf * np.exp(-2j * pi * fc * t).reshape((n,) + (1,) * (rf.ndim - 1))
    b, a, _ = butter_lowpass(fs, fc, bandwidth)
    return scipy.signal.filtfilt(b, a, iq, axis=0) * 2.0


def element_frame(n_elements, pitch, radius):
    """Element centres (x, z) and angles (radians, 0 for a linear array)."""
    if isinf(radius):
        x = (np.arange(n_elements) - (n_elements - 1) / 2.0) * pitch
        return x, np.zeros(n_elements), np.zeros(n_elements)
    half = asin(pitch / 2.0 / radius)
    chord = 2.0 * radius * sin(half * (n_elements - 1))
    apex = sqrt(radius * radius - (chord / 2.0) ** 2)
    theta = np.linspace(atan2(-chord / 2.0, apex), atan2(chord / 2.0, apex), n_elements)
    return radius * np.sin(theta), radius * np.cos(theta) - apex, theta


def default_fnumber(element_width, fc, c):
    """f-number from the -3 dB angle of the soft-baffle element directivity at fc."""
    lam = c / fc

    def directivity(alpha):
        return np.sinc(element_width / lam * sin(alpha)) * cos(alpha)

    lo, hi = 0.0, pi / 2.0
    for _ in range(80):
        mid = 0.5 * (lo + hi)
        if directivity(mid) > 1.0 / sqrt(2.0):
            lo = mid
        else:
            hi = mid
    return 1.0 / (2.0 * tan(0.5 * (lo + hi)))


def das_weights(n_samples, x, z, tx_delays, *, n_elements, pitch, radius, c, fs, fc, fnumber, t0=0.0,
                iq=True, method="linear"):
    """Dense DAS matrix rows, ``(n_pixels, n_samples * n_elements)`` complex128.

    ``x``/``z`` are pixel coordinates (any shape, flattened in C order)."""
    px = np.asarray(x, dtype=np.float64).reshape(-1)
    pz = np.asarray(z, dtype=np.float64).reshape(-1)
    xe, ze, te = element_frame(n_elements, pitch, radius)
    d = np.sqrt((px[:, None] - xe[None, :]) ** 2 + (pz[:, None] - ze[None, :]) ** 2)
    tx = np.asarray(tx_delays, dtype=np.float64)
    on = ~np.isnan(tx)
    d_tx = np.min(np.where(on[None, :], c * np.where(on, tx, 0.0)[None, :] + d, inf), axis=1)
    t = (d_tx[:, None] + d) / c
    s = (t - t0) * fs
    ax = (px[:, None] - xe) * np.sin(te) + (pz[:, None] - ze) * np.cos(te)
    lat = (px[:, None] - xe) * np.cos(te) - (pz[:, None] - ze) * np.sin(te)
    inside = ax > 0 if fnumber > 0 else np.ones_like(ax, dtype=bool)
    if fnumber > 0:
        inside &= np.abs(lat) <= ax / (2.0 * fnumber)
    rot = np.exp(2j * pi * fc * t) if iq else np.ones_like(t)
    m = np.zeros((px.size, n_samples * n_elements), dtype=np.complex128)
    rows = np.arange(px.size)[:, None].repeat(n_elements, axis=1)
    cols0 = np.arange(n_elements)[None, :] * n_samples
    if method == "linear":
        i0 = np.floor(s)
        w = s - i0
        ok = inside & (i0 >= 0) & (i0 + 1 <= n_samples - 1)
        i0 = np.where(ok, i0, 0).astype(np.int64)
        np.add.at(m, (rows[ok], (cols0 + i0)[ok]), ((1.0 - w) * rot)[ok])
        np.add.at(m, (rows[ok], (cols0 + i0 + 1)[ok]), (w * rot)[ok])
    elif method == "nearest":
        i = np.floor(s + 0.5)
        ok = inside & (i >= 0) & (i <= n_samples - 1)
        i = np.where(ok, i, 0).astype(np.int64)
        np.add.at(m, (rows[ok], (cols0 + i)[ok]), rot[ok])
    else:
        raise ValueError(f"unknown interpolation method {method!r}")
    return m


def das(iq_frames, x, z, tx_delays_frames, **kw):
    """Compounded image: sum over firings of ``das_weights @ iq.flatten(order="F")``.

    ``iq_frames`` is ``(n_frames, n_samples, n_elements)``; returns complex128 of x's shape."""
    iq_frames = np.asarray(iq_frames)
    img = np.zeros(np.asarray(x).size, dtype=np.complex128)
    for f in range(iq_frames.shape[0]):
        m = das_weights(iq_frames.shape[1], x, z, tx_delays_frames[f], **kw)
        img += m @ iq_frames[f].reshape(-1, order="F")
    return img.reshape(np.asarray(x).shape)
