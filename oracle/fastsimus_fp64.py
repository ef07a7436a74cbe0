"""FP64 NumPy restatement of the reference simus/pfield path (test infrastructure only).

Each function names the reference file and lines it restates (paths are relative to the
reference project root, ``src/fast_simus/...``).  The arithmetic follows the reference
step for step, including its dtype quirks (linear-array element x positions are formed in
float32, ``utils/geometry.py:33-37``), so results agree with the reference to FP64 rounding.

Parameters are duck-typed: any object exposing the reference's ``TransducerParams`` /
``MediumParams`` attributes (``freq_center``, ``pitch``, ``n_elements``, ``element_width``,
``radius``, ``bandwidth``, ``baffle``; ``speed_of_sound``, ``attenuation``) is accepted.
"""

from __future__ import annotations

from math import ceil, inf, log, log2, pi
from typing import NamedTuple

import numpy as np

NEPER_TO_DB = 20.0 / log(10.0)  # _pfield_math.py:21
BAFFLE_SOFT = "soft"
BAFFLE_RIGID = "rigid"


def _baffle_kind(baffle):
    """Map a baffle value to ("soft"|"rigid"|"float", value); transducer_params.py:10-20, :61-67."""
    if isinstance(baffle, str):
        b = str(baffle).lower()
        if b in ("soft", "rigid"):
            return b, 0.0
        raise ValueError(f"unknown baffle {baffle!r}")
    return "float", float(baffle)


# --------------------------------------------------------------------------------------
# spectrum.py
# --------------------------------------------------------------------------------------


def pulse_spectrum(angular_freq, freq_center, tx_n_wavelengths=1.0):
    """Windowed-sine pulse spectrum; spectrum.py:24-50."""
    duration = tx_n_wavelengths / freq_center
    wc = 2.0 * pi * freq_center
    lower = duration * (angular_freq - wc) / 2.0 / pi
    upper = duration * (angular_freq + wc) / 2.0 / pi
    return 1j * (np.sinc(lower) - np.sinc(upper))


def probe_spectrum(angular_freq, freq_center, bandwidth=0.75):
    """One-way generalized-normal probe response; spectrum.py:53-107."""
    if not (0.0 < bandwidth < 2.0):
        raise ValueError(f"bandwidth must be in (0, 2.0), got {bandwidth!r}")
    wc = 2.0 * pi * freq_center
    wb = bandwidth * wc
    shape = log(126) / log(2.0 * wc / wb)
    sigma = wb / 2.0 / (log(2) ** (1.0 / shape))
    sq = np.exp(-((np.abs(angular_freq - wc) / sigma) ** shape))
    return np.sqrt(sq)


# --------------------------------------------------------------------------------------
# utils/geometry.py, _pfield_math.py
# --------------------------------------------------------------------------------------


def element_positions(n_elements, pitch, radius):
    """Element centres, angles and apex offset; utils/geometry.py:18-88.

    Linear arrays: ``arange(..., dtype=float32) - (N-1)/2`` times ``pitch`` stays float32
    under NumPy 2 promotion (utils/geometry.py:33-37); z is float64 zeros.
    """
    if radius == inf:
        idx = np.arange(n_elements, dtype=np.float32)
        x = (idx - (n_elements - 1) / 2) * pitch  # float32 (weak python scalars)
        z = np.zeros(n_elements)
        theta = None
        apex = 0.0
    else:
        half = np.asin(np.asarray(pitch / 2 / radius))
        total = half * (n_elements - 1)
        chord = np.asarray(2 * radius) * np.sin(total)
        apex_arr = np.sqrt(np.asarray(radius**2) - (chord / 2) ** 2)
        apex = float(apex_arr)
        t0 = float(np.atan2(-chord / 2, apex_arr))
        t1 = float(np.atan2(chord / 2, apex_arr))
        theta = np.linspace(t0, t1, n_elements)
        z = np.asarray(radius) * np.cos(theta) - apex
        x = np.asarray(radius) * np.sin(theta)
    return np.stack([x, z], axis=-1), theta, apex


def subelement_centroids(element_width, n_sub, theta_e):
    """Sub-element centroid offsets; _pfield_math.py:40-67."""
    seg = element_width / n_sub
    offs = np.asarray([-element_width / 2.0 + seg / 2.0 + i * seg for i in range(n_sub)])
    offs2 = np.reshape(offs, (1, n_sub))
    dx = offs2 * np.cos(theta_e)[:, None]
    dz = offs2 * np.sin(-theta_e)[:, None]
    return np.stack([dx, dz], axis=-1)


def distances_and_angles(points, sub_offsets, element_pos, theta_e, c, fc):
    """Clipped distance, sin(theta), theta; _pfield_math.py:70-118."""
    delta = points[..., None, None, :] - sub_offsets - element_pos[:, None, :]
    dx = delta[..., 0]
    dz = delta[..., 1]
    d = np.sqrt(dx**2 + dz**2)
    dmin = np.asarray(c / fc / 2.0)
    dc = np.where(d < dmin, dmin, d)
    eps = np.asarray(1e-16)
    theta = np.asin((dx + eps) / (d + eps)) - theta_e[:, None]
    return dc, np.sin(theta), theta


def obliquity_factor(theta, baffle):
    """Baffle obliquity with the 1e-16 horizon floor; _pfield_math.py:165-199."""
    kind, val = _baffle_kind(baffle)
    if kind == "soft":
        ob = np.cos(theta)
    elif kind == "float":
        ct = np.cos(theta)
        ob = ct / (ct + val)
    else:
        ob = np.ones(theta.shape)
    return np.where(np.abs(theta) >= np.asarray(pi / 2), np.asarray(1e-16), ob)


def init_exponentials(freq_start, c, attenuation, distances, obliquity, freq_step):
    """Initial term and per-step multiplier of the frequency recurrence; _pfield_math.py:202-247."""
    k0 = 2.0 * pi * freq_start / c
    a0 = attenuation / NEPER_TO_DB * freq_start / 1e6 * 1e2
    kr = np.asarray(k0) * distances
    two_pi = np.asarray(2.0 * pi)
    phase = kr - two_pi * np.floor(kr / two_pi)
    init = np.exp(np.asarray(-a0) * distances + np.asarray(1j) * phase)
    dk = 2.0 * pi * freq_step / c
    da = attenuation / NEPER_TO_DB * freq_step / 1e6 * 1e2
    step = np.exp(np.asarray(-da + 1j * dk) * distances)
    init = init * obliquity / np.sqrt(distances)
    return init, step


class FrequencyPlan(NamedTuple):
    selected_freqs: np.ndarray
    pulse_spectrum: np.ndarray
    probe_spectrum: np.ndarray
    freq_step: float


def first_last_true(mask):
    """First/last True index; _pfield_math.py:250-261."""
    n = mask.shape[0]
    if n == 0:
        return 0, 0
    mi = np.asarray(mask, dtype=np.int32)
    first = int(np.argmax(mi))
    if int(np.max(mi)) == 0:
        return 0, 0
    last = n - 1 - int(np.argmax(mi[::-1]))
    return first, last


def select_frequencies(fc, bandwidth, tx_n_wavelengths, db_thresh, max_freq_step):
    """-dB band selection on linspace(0, 2fc); _pfield_math.py:121-162."""
    n = int(2 * ceil(fc / max_freq_step) + 1)
    freqs = np.linspace(0, 2 * fc, n)
    step = float(freqs[1])
    w = np.asarray(2.0 * pi) * freqs
    mag = np.abs(pulse_spectrum(w, fc, tx_n_wavelengths) * probe_spectrum(w, fc, bandwidth))
    gain = 20.0 * np.log10(np.asarray(1e-200) + mag / np.max(mag))
    i0, i1 = first_last_true(gain > db_thresh)
    sel = freqs[i0 : i1 + 1]
    ws = np.asarray(2.0 * pi) * sel
    return FrequencyPlan(sel, pulse_spectrum(ws, fc, tx_n_wavelengths), probe_spectrum(ws, fc, bandwidth), step)


# --------------------------------------------------------------------------------------
# simus.py, _simus_strategies.py
# --------------------------------------------------------------------------------------


def two_way_pulse_duration(fc, bandwidth, tx_n_wavelengths):
    """Two-way pulse length from an irfft of pulse*probe^2; simus.py:49-104."""
    dt = 1e-9
    df = fc / tx_n_wavelengths / 32
    p = ceil(log2(1.0 / dt / 2.0 / df))
    n_fft = 2**p
    w = 2.0 * pi * np.linspace(0, 1.0 / dt / 2.0, n_fft)
    two_way = pulse_spectrum(w, fc, tx_n_wavelengths) * probe_spectrum(w, fc, bandwidth) ** 2
    pulse = np.fft.fftshift(np.fft.irfft(two_way))
    pulse = pulse / np.max(np.abs(pulse))
    above = pulse > (1.0 / 1023)
    n = above.shape[0]
    idx = np.arange(n)
    idx1 = int(np.min(np.where(above, idx, np.asarray(n))))
    idx2 = int(np.max(np.where(above, idx, np.asarray(-1))))
    if idx1 >= n:
        return tx_n_wavelengths / fc
    trim = min(idx1 + 1, 2 * n_fft - 1 - idx2 - 1)
    trimmed = pulse[-trim : trim - 2 : -1]
    return float(trimmed.shape[0] * dt)


class SimusPlan(NamedTuple):
    """Fields of simus.py:135-162."""

    selected_freqs: np.ndarray
    pulse_spectrum: np.ndarray
    probe_spectrum: np.ndarray
    n_sub: int
    seg_length: float
    correction_factor: float
    n_freq_full: int
    freq_idx_start: int
    n_fft: int


def _auto_n_sub(params, c, element_splitting):
    if element_splitting is not None:
        return element_splitting
    lam_min = c / (params.freq_center * (1.0 + params.bandwidth / 2.0))
    return ceil(params.element_width / lam_min)


def simus_precompute(scatterers, rc, delays, params, medium, *, fs=None, tx_n_wavelengths=1.0,
                     db_thresh=-60.0, element_splitting=None, frequency_step=1.0):
    """Round-trip frequency plan; simus.py:165-260."""
    c = medium.speed_of_sound
    fc = params.freq_center
    if fs is None:
        fs = 4.0 * fc
    delays = np.asarray(delays, dtype=np.float64)
    dclean = np.where(np.isnan(delays), np.asarray(0.0), delays)
    n_sub = _auto_n_sub(params, c, element_splitting)
    seg = params.element_width / n_sub
    epos, _, _ = element_positions(params.n_elements, params.pitch, params.radius)
    scatterers = np.asarray(scatterers, dtype=np.float64)
    x = scatterers[..., 0]
    z = scatterers[..., 1]
    d2 = (np.reshape(x, (-1, 1)) - epos[:, 0]) ** 2 + (np.reshape(z, (-1, 1)) - epos[:, 1]) ** 2
    max_d = float(np.max(np.sqrt(d2)))
    if tx_n_wavelengths != float("inf"):
        max_d = max_d + two_way_pulse_duration(fc, params.bandwidth, tx_n_wavelengths) * c
    df = 1.0 / 2.0 / (2.0 * max_d / c + float(np.max(dclean)))
    df = float(frequency_step) * df
    n_full = int(2 * ceil(fc / df) + 1)
    fp = select_frequencies(fc, params.bandwidth, tx_n_wavelengths, db_thresh, df)
    dfa = fp.freq_step
    idx0 = round(float(fp.selected_freqs[0]) / dfa) if dfa > 0 else 0
    corr = 1.0 if tx_n_wavelengths == float("inf") else dfa
    corr = corr * params.element_width
    n_fft = ceil(fs / 2.0 / fc * (n_full - 1))
    return SimusPlan(fp.selected_freqs, fp.pulse_spectrum, fp.probe_spectrum, n_sub, seg, corr, n_full, idx0, n_fft)


def _prepare_simus_sweep(scat, dclean, apod, plan, params, medium, full_frequency_directivity):
    """Sweep set-up; simus.py:263-333."""
    epos, theta_e, apex = element_positions(params.n_elements, params.pitch, params.radius)
    if theta_e is None:
        theta_e = np.zeros(params.n_elements)
    c = medium.speed_of_sound
    offs = subelement_centroids(params.element_width, plan.n_sub, theta_e)
    x = scat[..., 0]
    z = scat[..., 1]
    is_out = z < 0
    if params.radius != inf:
        is_out = is_out | ((x**2 + (z + apex) ** 2) <= params.radius**2)
    dist, sin_t, theta = distances_and_angles(scat, offs, epos, theta_e, c, params.freq_center)
    ob = obliquity_factor(theta, params.baffle)
    f0 = plan.selected_freqs[0]
    nf = plan.selected_freqs.shape[0]
    fstep = (plan.selected_freqs[1] - plan.selected_freqs[0]) if nf > 1 else np.asarray(0.0)
    init, step = init_exponentials(f0, c, medium.attenuation, dist, ob, fstep)
    if not full_frequency_directivity:
        kc = 2.0 * pi * params.freq_center / c
        init = init * np.sinc(np.asarray(kc * plan.seg_length / 2.0) * sin_t / pi)
    da0 = np.exp(np.asarray(1j * 2.0 * pi) * f0 * dclean) * apod
    dstep = np.exp(np.asarray(1j * 2.0 * pi) * fstep * dclean)
    wn = np.asarray(2.0 * pi) * plan.selected_freqs / c
    return init, step, da0, dstep, is_out, wn, sin_t


def _simus_sweep(init, step, da0, dstep, rc, is_out, wn, pulse, probe, seg, sin_t, ffd):
    """Per-frequency TX -> scatter -> RX chain; _simus_strategies.py:23-77 (step body) and
    :80-140 (loop driver)."""
    spectra = pulse * probe
    nf = int(wn.shape[0])
    ne = init.shape[1]
    out = np.zeros((nf, ne), dtype=init.dtype)
    phase = init
    da = da0
    for k in range(nf):
        if ffd:
            dirk = np.sinc(wn[k] * seg / 2.0 * sin_t / pi)
            rp = np.mean(phase * dirk, axis=-1)
        else:
            rp = np.mean(phase, axis=-1)
        p = spectra[k] * (rp @ da[..., None])[..., 0]
        p = np.where(is_out, np.asarray(0.0 + 0j), p)
        out[k, :] = probe[k] * ((rc * p) @ rp)
        phase = phase * step
        da = da * dstep
    return out


def _clean(delays, apod, n):
    delays = np.asarray(delays, dtype=np.float64)
    apod = np.ones(n) if apod is None else np.asarray(apod, dtype=np.float64)
    nan = np.isnan(delays)
    return np.where(nan, np.asarray(0.0), delays), np.where(nan, np.asarray(0.0), apod)


def simus_spectrum_selected(scatterers, rc, delays, plan, params, medium, *, tx_apodization=None,
                            full_frequency_directivity=False):
    """Selected-band spectrum (F, E) before the correction factor: what simus.py:470-488
    returns from the PYTHON strategy."""
    dclean, apod = _clean(delays, tx_apodization, params.n_elements)
    scat = np.asarray(scatterers, dtype=np.float64).reshape(-1, 2)
    rcf = np.asarray(rc, dtype=np.float64).reshape(-1)
    init, step, da0, dstep, is_out, wn, sin_t = _prepare_simus_sweep(
        scat, dclean, apod, plan, params, medium, full_frequency_directivity)
    return _simus_sweep(init, step, da0, dstep, rcf, is_out, wn, plan.pulse_spectrum, plan.probe_spectrum,
                        plan.seg_length, sin_t, full_frequency_directivity)


def irfft_and_threshold(spect_selected, plan, n_elements, gate=True):
    """Zero-pad into the full band, irfft of the conjugate, smooth -100 dB gate; simus.py:336-367."""
    nsel = spect_selected.shape[0]
    full = np.zeros((plan.n_freq_full, n_elements), dtype=spect_selected.dtype)
    full[plan.freq_idx_start : plan.freq_idx_start + nsel, :] = spect_selected
    rf = np.fft.irfft(np.conj(full), n=plan.n_fft, axis=0)
    rf = rf[: (plan.n_fft + 1) // 2, ...]
    if gate:
        th = 1e-5
        peak = np.max(np.abs(rf))
        rel = np.abs(rf) / (peak + np.asarray(1e-30))
        rf = rf * (0.5 * (1.0 + np.tanh((rel - th) / (th / 10.0))))
    return rf, full


class SimusResult(NamedTuple):
    rf: np.ndarray
    spectrum: np.ndarray


def simus_compute(scatterers, rc, delays, plan, params, medium, *, tx_apodization=None,
                  full_frequency_directivity=False, gate=True):
    """simus.py:392-495 on the PYTHON strategy."""
    sel = simus_spectrum_selected(scatterers, rc, delays, plan, params, medium, tx_apodization=tx_apodization,
                                  full_frequency_directivity=full_frequency_directivity)
    sel = sel * np.asarray(plan.correction_factor)
    rf, full = irfft_and_threshold(sel, plan, params.n_elements, gate=gate)
    return SimusResult(rf, full)


def simus(scatterers, rc, delays, params, medium, *, fs=None, tx_apodization=None, tx_n_wavelengths=1.0,
          db_thresh=-60.0, full_frequency_directivity=False, element_splitting=None, frequency_step=1.0):
    """simus.py:498-567."""
    plan = simus_precompute(scatterers, rc, delays, params, medium, fs=fs, tx_n_wavelengths=tx_n_wavelengths,
                            db_thresh=db_thresh, element_splitting=element_splitting,
                            frequency_step=frequency_step)
    return simus_compute(scatterers, rc, delays, plan, params, medium, tx_apodization=tx_apodization,
                         full_frequency_directivity=full_frequency_directivity)


def simus_multi_transmit(scatterers, rc, delays_list, params, medium, *, fs=None, tx_apodization=None):
    """Many firings on one phantom with ONE shared plan taken from the firing whose delay span
    is largest, as the reference's multi-transmit helper does
    (tests/_picmus_phantom_shared.py:319-367).  Returns (plan, [SimusResult per firing])."""
    spans = [float(np.ptp(np.nan_to_num(np.asarray(d, dtype=np.float64)))) for d in delays_list]
    ip = int(np.argmax(spans))
    plan = simus_precompute(scatterers, rc, delays_list[ip], params, medium, fs=fs)
    return plan, [simus_compute(scatterers, rc, d, plan, params, medium, tx_apodization=tx_apodization)
                  for d in delays_list]


# --------------------------------------------------------------------------------------
# pfield.py, _pfield_strategies.py
# --------------------------------------------------------------------------------------


class PfieldPlan(NamedTuple):
    """Fields of pfield.py:58-82."""

    selected_freqs: np.ndarray
    pulse_spectrum: np.ndarray
    probe_spectrum: np.ndarray
    n_sub: int
    seg_length: float
    correction_factor: float


def pfield_precompute(positions, delays, params, medium, *, tx_n_wavelengths=1.0, db_thresh=-60.0,
                      element_splitting=None, frequency_step=1.0):
    """One-way frequency plan; pfield.py:223-298."""
    c = medium.speed_of_sound
    positions = np.asarray(positions, dtype=np.float64)
    if positions.size == 0:
        raise ValueError("Grid has no points")
    delays = np.asarray(delays, dtype=np.float64)
    dclean = np.where(np.isnan(delays), np.asarray(0.0), delays)
    n_sub = _auto_n_sub(params, c, element_splitting)
    seg = params.element_width / n_sub
    epos, theta_e, _ = element_positions(params.n_elements, params.pitch, params.radius)
    if theta_e is None:
        theta_e = np.zeros(params.n_elements)
    offs = subelement_centroids(params.element_width, n_sub, theta_e)
    dist, _, _ = distances_and_angles(positions, offs, epos, theta_e, c, params.freq_center)
    df = 1.0 / (float(np.max(dist)) / c + float(np.max(dclean)))
    df = float(frequency_step) * df
    fp = select_frequencies(params.freq_center, params.bandwidth, tx_n_wavelengths, db_thresh, df)
    df = fp.freq_step
    corr = 1.0 if tx_n_wavelengths == float("inf") else df
    corr = corr * params.element_width
    return PfieldPlan(fp.selected_freqs, fp.pulse_spectrum, fp.probe_spectrum, n_sub, seg, corr)


def _prepare_frequency_sweep(positions, dclean, apod, plan, params, medium, full_frequency_directivity):
    """pfield.py:102-184: delays/apodization and 1/n_sub absorbed, sources flattened."""
    epos, theta_e, apex = element_positions(params.n_elements, params.pitch, params.radius)
    if theta_e is None:
        theta_e = np.zeros(params.n_elements)
    c = medium.speed_of_sound
    offs = subelement_centroids(params.element_width, plan.n_sub, theta_e)
    x = positions[..., 0]
    z = positions[..., 1]
    is_out = z < 0
    if params.radius != inf:
        is_out = is_out | ((x**2 + (z + apex) ** 2) <= params.radius**2)
    dist, sin_t, theta = distances_and_angles(positions, offs, epos, theta_e, c, params.freq_center)
    ob = obliquity_factor(theta, params.baffle)
    f0 = plan.selected_freqs[0]
    nf = plan.selected_freqs.shape[0]
    fstep = (plan.selected_freqs[1] - plan.selected_freqs[0]) if nf > 1 else np.asarray(0.0)
    init, step = init_exponentials(f0, c, medium.attenuation, dist, ob, fstep)
    if not full_frequency_directivity:
        kc = 2.0 * pi * params.freq_center / c
        init = init * np.sinc(np.asarray(kc * plan.seg_length / 2.0) * sin_t / pi)
    da0 = np.exp(np.asarray(1j * 2.0 * pi) * f0 * dclean) * apod
    dstep = np.exp(np.asarray(1j * 2.0 * pi) * fstep * dclean)
    init = init * da0[:, None]
    step = step * dstep[:, None]
    init = init / plan.n_sub

    def flat(a):
        return np.reshape(a, (*a.shape[:-2], a.shape[-2] * a.shape[-1]))

    wn = np.asarray(2.0 * pi) * plan.selected_freqs / c
    return flat(init), flat(step), is_out, wn, flat(sin_t)


def _pfield_sweep(init, step, is_out, wn, pulse, probe, seg, sin_t, ffd):
    """_pfield_strategies.py:21-50 (step body) and :53-88 (loop driver)."""
    spectra = pulse * probe
    nf = int(wn.shape[0])
    phase = init
    rp = np.zeros(phase.shape[:-1])
    zero = np.asarray(0.0)
    for k in range(nf):
        if ffd:
            w = phase * np.sinc(wn[k] * seg / 2.0 * sin_t / pi)
        else:
            w = phase
        pk = spectra[k] * np.sum(w, axis=-1)
        phase = phase * step
        rpk = np.real(pk * np.conj(pk))
        rp = rp + np.where(is_out, zero, rpk)
    return rp


def pfield_compute(positions, delays, plan, params, medium, *, tx_apodization=None,
                   full_frequency_directivity=False):
    """pfield.py:301-378 on the Python-loop driver: sqrt(accumulated |P|^2 * correction)."""
    positions = np.asarray(positions, dtype=np.float64)
    dclean, apod = _clean(delays, tx_apodization, params.n_elements)
    init, step, is_out, wn, sin_t = _prepare_frequency_sweep(positions, dclean, apod, plan, params, medium,
                                                             full_frequency_directivity)
    acc = _pfield_sweep(init, step, is_out, wn, plan.pulse_spectrum, plan.probe_spectrum, plan.seg_length, sin_t,
                        full_frequency_directivity)
    return np.sqrt(acc * plan.correction_factor)


def pfield(positions, delays, params, medium, *, tx_apodization=None, tx_n_wavelengths=1.0, db_thresh=-60.0,
           full_frequency_directivity=False, element_splitting=None, frequency_step=1.0):
    """pfield.py:381-475."""
    plan = pfield_precompute(positions, delays, params, medium, tx_n_wavelengths=tx_n_wavelengths,
                             db_thresh=db_thresh, element_splitting=element_splitting,
                             frequency_step=frequency_step)
    return pfield_compute(positions, delays, plan, params, medium, tx_apodization=tx_apodization,
                          full_frequency_directivity=full_frequency_directivity)


def tx_field(positions, delays, plan, params, medium, *, tx_apodization=None, full_frequency_directivity=False):
    """Complex transmit field p_k(x) = spectra[k] * sum_src(init * step^k) at every point and
    selected frequency, shape (n_points, F).  It is the quantity inside
    _pfield_strategies.py:48 before |.|^2 (identical to p_k of _simus_strategies.py:64-66)."""
    positions = np.asarray(positions, dtype=np.float64).reshape(-1, 2)
    dclean, apod = _clean(delays, tx_apodization, params.n_elements)
    init, step, is_out, wn, sin_t = _prepare_frequency_sweep(positions, dclean, apod, plan, params, medium,
                                                             full_frequency_directivity)
    spectra = plan.pulse_spectrum * plan.probe_spectrum
    nf = int(wn.shape[0])
    out = np.zeros((positions.shape[0], nf), dtype=np.complex128)
    phase = init
    for k in range(nf):
        w = phase * np.sinc(wn[k] * plan.seg_length / 2.0 * sin_t / pi) if full_frequency_directivity else phase
        out[:, k] = np.where(is_out, 0.0, spectra[k] * np.sum(w, axis=-1))
        phase = phase * step
    return out


# --------------------------------------------------------------------------------------
# tx_delay.py
# --------------------------------------------------------------------------------------


def focused(element_pos, focus, *, speed_of_sound, radius=inf, apex_offset=0.0):
    """tx_delay.py:31-113."""
    element_pos = np.asarray(element_pos, dtype=np.float64)
    focus = np.asarray(focus, dtype=np.float64)
    d = np.sqrt(np.sum((element_pos - focus) ** 2, axis=-1))
    if radius == inf:
        sgn = np.sign(focus[-1])
    else:
        sgn = np.sign(focus[0] ** 2 + (focus[-1] + apex_offset) ** 2 - radius**2)
    sgn = np.where(sgn == 0, -1, sgn)
    delays = -d * sgn / speed_of_sound
    return delays - np.min(delays)


def plane_wave(element_pos, tilt_rad, *, speed_of_sound, radius=inf, apex_offset=0.0):
    """tx_delay.py:116-189."""
    from math import cos, sin, sqrt

    if abs(tilt_rad) >= pi / 2:
        raise ValueError("Tilt angles must satisfy |tilt_rad| < pi/2")
    element_pos = np.asarray(element_pos, dtype=np.float64)
    xe = element_pos[:, 0]
    ze = element_pos[:, 1]
    if radius == inf:
        delays = xe * sin(tilt_rad) / speed_of_sound
    else:
        xn = radius * sin(tilt_rad)
        zn = radius * cos(tilt_rad) - apex_offset
        num = np.abs(ze + xn / (zn + apex_offset) * xe - xn**2 / (zn + apex_offset) - zn)
        den = sqrt(1 + xn**2 / (zn + apex_offset) ** 2)
        delays = -(num / den) / speed_of_sound
    return delays - np.min(delays)


def diverging_wave(element_pos, tilt_rad, width_rad, *, aperture_length, speed_of_sound):
    """tx_delay.py:192-276."""
    from math import fmod, tan

    if width_rad <= 0 or width_rad >= pi:
        raise ValueError("Width angles must satisfy 0 < width_rad < pi")
    tn = fmod(-tilt_rad + pi / 2, 2 * pi) - pi / 2
    sc = 1.0
    if abs(tn) > pi / 2:
        tn = pi - tn
        sc = -1.0
    den = tan(tn - width_rad / 2) - tan(tn + width_rad / 2)
    z0 = sc * aperture_length / den
    x0 = sc * z0 * tan(width_rad / 2 - tn) + aperture_length / 2
    return focused(element_pos, np.asarray([x0, z0]), speed_of_sound=speed_of_sound)


# --------------------------------------------------------------------------------------
# transmit field at (x, z, f, theta) samples, for the surrogate (closed form, FP64)
# --------------------------------------------------------------------------------------


def tx_field_samples(samples, params, medium, tx_n_wavelengths=1.0, n_sub=None):
    """Complex transmit pressure of a plane wave at samples (n, 4) = (x, z, f, theta):
    pulse(f) probe(f) * sum_{e,u} exp(i 2 pi f tau_e) G(x, z, e, u, f) / n_sub, where G is the
    closed form of _init_exponentials (_pfield_math.py:202-247) at frequency f with the
    centre-frequency directivity (pfield.py:148-152) and tau_e the plane-wave delays
    (tx_delay.py:116-189).  Equals the pressure inside _pfield_strategies.py:48 for
    f on a plan's grid."""
    samples = np.asarray(samples, dtype=np.float64).reshape(-1, 4)
    c = medium.speed_of_sound
    if n_sub is None:
        n_sub = _auto_n_sub(params, c, None)
    epos, theta_e, _ = element_positions(params.n_elements, params.pitch, params.radius)
    theta_e = np.zeros(params.n_elements) if theta_e is None else theta_e
    offs = subelement_centroids(params.element_width, n_sub, theta_e)
    seg = params.element_width / n_sub
    out = np.zeros(samples.shape[0], dtype=np.complex128)
    kc = 2.0 * pi * params.freq_center / c
    for i, (x, z, f, th) in enumerate(samples):
        dist, sin_t, theta = distances_and_angles(np.array([x, z]), offs, epos, theta_e, c, params.freq_center)
        ob = obliquity_factor(theta, params.baffle)
        init, _ = init_exponentials(f, c, medium.attenuation, dist, ob, 0.0)
        init = init * np.sinc(kc * seg / 2.0 * sin_t / pi)
        tau = plane_wave(epos, th, speed_of_sound=c)
        w = 2.0 * pi * f
        spec = pulse_spectrum(np.array([w]), params.freq_center, tx_n_wavelengths)[0] * \
            probe_spectrum(np.array([w]), params.freq_center, params.bandwidth)[0]
        p = spec * np.sum(init * np.exp(1j * 2.0 * pi * f * tau)[:, None]) / n_sub
        out[i] = 0.0 if z < 0 else p
    return out
