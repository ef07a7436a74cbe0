"""Host-side FP64 planning: spectra, array geometry, frequency selection and the simus/pfield plans.

Everything here is cheap O(S*E) or O(F) host work that fixes the static shapes of a sweep
(number of selected frequencies, frequency step, irfft length).  It follows the reference's
planning code exactly, because the plan decides which frequencies exist at all:

* ``pulse_spectrum`` / ``probe_spectrum``  -- spectrum.py:24-107
* ``element_positions``                    -- utils/geometry.py:18-88 (linear x in float32,
  as NumPy 2 promotion makes it there)
* ``subelement_offsets``                   -- _pfield_math.py:40-67
* ``select_frequencies``                   -- _pfield_math.py:121-162, :250-261
* ``two_way_pulse_duration``               -- simus.py:49-104
* ``simus_precompute`` / ``SimusPlan``     -- simus.py:135-260
* ``pfield_precompute`` / ``PfieldPlan``   -- pfield.py:58-82, :223-298

Scatterer/grid arrays may be NumPy arrays or torch tensors (CPU or CUDA); the max-distance
pass runs where the data lives, in float64, in chunks.
"""

from __future__ import annotations

from math import ceil, inf, log, log2, pi
from typing import NamedTuple

import numpy as np

from fastsimus_gb300.params import MediumParams, TransducerParams

NEPER_TO_DB = 20.0 / log(10.0)

_DEFAULT_MEDIUM = MediumParams()


def pulse_spectrum(angular_freq, freq_center, tx_n_wavelengths=1.0):
    """Spectrum of a windowed sine of ``tx_n_wavelengths`` cycles (spectrum.py:24-50)."""
    duration = tx_n_wavelengths / freq_center
    wc = 2.0 * pi * freq_center
    w = np.asarray(angular_freq, dtype=np.float64)
    return 1j * (np.sinc(duration * (w - wc) / 2.0 / pi) - np.sinc(duration * (w + wc) / 2.0 / pi))


def probe_spectrum(angular_freq, freq_center, bandwidth=0.75):
    """One-way generalized-normal probe response (spectrum.py:53-107)."""
    if not (0.0 < bandwidth < 2.0):
        raise ValueError(f"bandwidth must be in (0, 2.0), got {bandwidth!r}")
    wc = 2.0 * pi * freq_center
    wb = bandwidth * wc
    shape = log(126) / log(2.0 * wc / wb)
    sigma = wb / 2.0 / (log(2) ** (1.0 / shape))
    w = np.asarray(angular_freq, dtype=np.float64)
    return np.sqrt(np.exp(-((np.abs(w - wc) / sigma) ** shape)))


def element_positions(n_elements: int, pitch: float, radius: float):
    """Element centres (E,2), angular positions (E,) or None, apex offset (utils/geometry.py:18-88)."""
    if radius == inf:
        idx = np.arange(n_elements, dtype=np.float32)
        x = (idx - (n_elements - 1) / 2) * pitch  # stays float32, as in the reference
        z = np.zeros(n_elements)
        return np.stack([x.astype(np.float64), z], axis=-1), None, 0.0
    half = np.arcsin(pitch / 2 / radius)
    total = half * (n_elements - 1)
    chord = 2 * radius * np.sin(total)
    apex = float(np.sqrt(radius**2 - (chord / 2) ** 2))
    t0 = float(np.arctan2(-chord / 2, apex))
    t1 = float(np.arctan2(chord / 2, apex))
    theta = np.linspace(t0, t1, n_elements)
    return np.stack([radius * np.sin(theta), radius * np.cos(theta) - apex], axis=-1), theta, apex


def subelement_offsets(element_width: float, n_sub: int, theta_e):
    """Sub-element centroid offsets (E, U, 2) relative to element centres (_pfield_math.py:40-67)."""
    seg = element_width / n_sub
    offs = np.asarray([-element_width / 2.0 + seg / 2.0 + i * seg for i in range(n_sub)]).reshape(1, n_sub)
    theta_e = np.asarray(theta_e, dtype=np.float64)
    return np.stack([offs * np.cos(theta_e)[:, None], offs * np.sin(-theta_e)[:, None]], axis=-1)


def source_positions(params: TransducerParams, n_sub: int):
    """FP64 (E*U, 2) source positions element-major (src = e*U + u), theta_e (E,), apex offset."""
    epos, theta_e, apex = element_positions(params.n_elements, params.pitch, params.radius)
    if theta_e is None:
        theta_e = np.zeros(params.n_elements)
    offs = subelement_offsets(params.element_width, n_sub, theta_e)
    src = (epos[:, None, :] + offs).reshape(-1, 2)
    return src, theta_e, apex


class FrequencyPlan(NamedTuple):
    selected_freqs: np.ndarray
    pulse_spectrum: np.ndarray
    probe_spectrum: np.ndarray
    freq_step: float


def select_frequencies(fc, bandwidth, tx_n_wavelengths, db_thresh, max_freq_step) -> FrequencyPlan:
    """Keep the contiguous band where |pulse*probe| exceeds ``db_thresh`` dB of its peak on
    ``linspace(0, 2 fc, 2 ceil(fc/df) + 1)`` (_pfield_math.py:121-162)."""
    n = int(2 * ceil(fc / max_freq_step) + 1)
    freqs = np.linspace(0, 2 * fc, n)
    step = float(freqs[1])
    w = 2.0 * pi * freqs
    mag = np.abs(pulse_spectrum(w, fc, tx_n_wavelengths) * probe_spectrum(w, fc, bandwidth))
    above = 20.0 * np.log10(1e-200 + mag / np.max(mag)) > db_thresh
    if not above.any():
        i0 = i1 = 0
    else:
        i0 = int(np.argmax(above))
        i1 = n - 1 - int(np.argmax(above[::-1]))
    sel = freqs[i0 : i1 + 1]
    ws = 2.0 * pi * sel
    return FrequencyPlan(sel, pulse_spectrum(ws, fc, tx_n_wavelengths), probe_spectrum(ws, fc, bandwidth), step)


def two_way_pulse_duration(freq_center, bandwidth, tx_n_wavelengths) -> float:
    """Duration of the pulse-echo pulse above 1/1023 of its peak (simus.py:49-104)."""
    dt = 1e-9
    df = freq_center / tx_n_wavelengths / 32
    n_fft = 2 ** ceil(log2(1.0 / dt / 2.0 / df))
    w = 2.0 * pi * np.linspace(0, 1.0 / dt / 2.0, n_fft)
    two_way = pulse_spectrum(w, freq_center, tx_n_wavelengths) * probe_spectrum(w, freq_center, bandwidth) ** 2
    pulse = np.fft.fftshift(np.fft.irfft(two_way))
    pulse = pulse / np.max(np.abs(pulse))
    above = pulse > (1.0 / 1023)
    n = above.shape[0]
    if not above.any():
        return tx_n_wavelengths / freq_center
    idx1 = int(np.argmax(above))
    idx2 = n - 1 - int(np.argmax(above[::-1]))
    trim = min(idx1 + 1, 2 * n_fft - 1 - idx2 - 1)
    return float(pulse[-trim : trim - 2 : -1].shape[0] * dt)


def _is_torch(a) -> bool:
    return type(a).__module__.startswith("torch")


def max_distance(points, targets: np.ndarray, *, clip_min: float | None = None) -> float:
    """max over (point, target) of the Euclidean distance, in float64, chunked over points.

    ``points`` is (..., 2) NumPy or torch (CPU/CUDA); ``targets`` is (T, 2) FP64 NumPy.
    """
    if _is_torch(points):
        import torch

        p = points.reshape(-1, 2).to(torch.float64)
        t = torch.as_tensor(targets, dtype=torch.float64, device=p.device)
        best = torch.zeros((), dtype=torch.float64, device=p.device)
        chunk = max(1, (1 << 24) // max(1, t.shape[0]))
        for i in range(0, p.shape[0], chunk):
            q = p[i : i + chunk]
            d2 = (q[:, None, 0] - t[None, :, 0]) ** 2 + (q[:, None, 1] - t[None, :, 1]) ** 2
            best = torch.maximum(best, d2.max())
        m = float(torch.sqrt(best))
    else:
        p = np.asarray(points, dtype=np.float64).reshape(-1, 2)
        m = 0.0
        chunk = max(1, (1 << 22) // max(1, targets.shape[0]))
        for i in range(0, p.shape[0], chunk):
            q = p[i : i + chunk]
            d2 = (q[:, None, 0] - targets[None, :, 0]) ** 2 + (q[:, None, 1] - targets[None, :, 1]) ** 2
            m = max(m, float(np.sqrt(d2.max())))
    if clip_min is not None:
        m = max(m, clip_min)
    return m


def _auto_n_sub(params: TransducerParams, c: float, element_splitting):
    if element_splitting is not None:
        return int(element_splitting)
    lam_min = c / (params.freq_center * (1.0 + params.bandwidth / 2.0))
    return ceil(params.element_width / lam_min)


def _nan_clean_max(delays) -> float:
    if _is_torch(delays):
        d = delays.detach().to("cpu").double().numpy()
    else:
        d = np.asarray(delays, dtype=np.float64)
    d = np.where(np.isnan(d), 0.0, d)
    return float(np.max(d)) if d.size else 0.0


class SimusPlan(NamedTuple):
    """Static quantities of a simus sweep (simus.py:135-162)."""

    selected_freqs: np.ndarray
    pulse_spectrum: np.ndarray
    probe_spectrum: np.ndarray
    n_sub: int
    seg_length: float
    correction_factor: float
    n_freq_full: int
    freq_idx_start: int
    n_fft: int


def simus_precompute(scatterers, rc, delays, params: TransducerParams, medium: MediumParams = _DEFAULT_MEDIUM, *,
                     fs: float | None = None, tx_n_wavelengths: float = 1.0, db_thresh: float = -60.0,
                     element_splitting: int | None = None, frequency_step: float = 1.0) -> SimusPlan:
    """Round-trip frequency plan (simus.py:165-260).

    df = 1 / 2 / (2 max_d / c + max delay), with max_d over scatterer x element-centre
    distances plus the two-way pulse length; n_freq_full = 2 ceil(fc/df) + 1;
    n_fft = ceil(fs / 2 / fc * (n_freq_full - 1)).
    """
    c = medium.speed_of_sound
    fc = params.freq_center
    if fs is None:
        fs = 4.0 * fc
    n_sub = _auto_n_sub(params, c, element_splitting)
    seg = params.element_width / n_sub
    epos, _, _ = element_positions(params.n_elements, params.pitch, params.radius)
    max_d = max_distance(scatterers, epos)
    if tx_n_wavelengths != float("inf"):
        max_d = max_d + two_way_pulse_duration(fc, params.bandwidth, tx_n_wavelengths) * c
    df = 1.0 / 2.0 / (2.0 * max_d / c + _nan_clean_max(delays))
    df = float(frequency_step) * df
    n_full = int(2 * ceil(fc / df) + 1)
    fp = select_frequencies(fc, params.bandwidth, tx_n_wavelengths, db_thresh, df)
    dfa = fp.freq_step
    idx0 = round(float(fp.selected_freqs[0]) / dfa) if dfa > 0 else 0
    corr = (1.0 if tx_n_wavelengths == float("inf") else dfa) * params.element_width
    n_fft = ceil(fs / 2.0 / fc * (n_full - 1))
    return SimusPlan(fp.selected_freqs, fp.pulse_spectrum, fp.probe_spectrum, n_sub, seg, corr, n_full, idx0, n_fft)


class PfieldPlan(NamedTuple):
    """Static quantities of a pfield sweep (pfield.py:58-82)."""

    selected_freqs: np.ndarray
    pulse_spectrum: np.ndarray
    probe_spectrum: np.ndarray
    n_sub: int
    seg_length: float
    correction_factor: float


def pfield_precompute(positions, delays, params: TransducerParams, medium: MediumParams = _DEFAULT_MEDIUM, *,
                      tx_n_wavelengths: float = 1.0, db_thresh: float = -60.0,
                      element_splitting: int | None = None, frequency_step: float = 1.0) -> PfieldPlan:
    """One-way frequency plan (pfield.py:223-298): df = 1 / (max r / c + max delay), with r the
    lambda/2-clipped distance from every grid point to every sub-element."""
    c = medium.speed_of_sound
    size = positions.numel() if _is_torch(positions) else np.asarray(positions).size
    if size == 0:
        raise ValueError("Grid has no points")
    n_sub = _auto_n_sub(params, c, element_splitting)
    seg = params.element_width / n_sub
    src, _, _ = source_positions(params, n_sub)
    max_r = max_distance(positions, src, clip_min=c / params.freq_center / 2.0)
    df = 1.0 / (max_r / c + _nan_clean_max(delays))
    df = float(frequency_step) * df
    fp = select_frequencies(params.freq_center, params.bandwidth, tx_n_wavelengths, db_thresh, df)
    corr = (1.0 if tx_n_wavelengths == float("inf") else fp.freq_step) * params.element_width
    return PfieldPlan(fp.selected_freqs, fp.pulse_spectrum, fp.probe_spectrum, n_sub, seg, corr)
