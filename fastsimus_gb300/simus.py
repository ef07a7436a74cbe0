"""Public simus API, drop-in for the reference's ``fast_simus.simus`` module (simus.py:107-567).

Same names, arguments and return types (``SimusResult(rf, spectrum)``); the frequency sweep
runs in libfsgb300.so on the GPU.  Inputs may be NumPy arrays (copied to the current CUDA
device) or torch tensors; results are torch tensors on that device with the reference's
dtypes: ``rf`` float64 (n_samples, E) and ``spectrum`` complex128 (n_freq_full, E).  The
values are computed in FP32 with double-float phases (relative L2 ~1e-6 against the FP64
path) and widened on the device; ``BatchedSimus`` keeps float32 / complex64.

``SimusStrategy`` keeps the reference's values and adds ``GB300``; ``None`` and ``CUDA`` select
the GB300 kernels.  The CPU strategies (PYTHON, SCAN) and Apple's METAL are not part of this
package and raise ``NotImplementedError`` -- there is no CPU fallback.
"""

from __future__ import annotations

from enum import StrEnum
from typing import NamedTuple

import torch

from fastsimus_gb300 import _device, _native
from fastsimus_gb300.params import MediumParams, TransducerParams
from fastsimus_gb300.plan import SimusPlan, simus_precompute

_DEFAULT_MEDIUM = MediumParams()


class SimusStrategy(StrEnum):
    """Sweep strategy (simus.py:107-120) plus GB300."""

    PYTHON = "python"
    SCAN = "scan"
    METAL = "metal"
    CUDA = "cuda"
    GB300 = "gb300"


class SimusResult(NamedTuple):
    """rf: (n_samples, n_elements) float64; spectrum: (n_freq_full, n_elements) complex128 (the
    batched API returns float32 / complex64 with a trailing firing axis)."""

    rf: torch.Tensor
    spectrum: torch.Tensor


def _check_strategy(strategy):
    if strategy is None:
        return SimusStrategy.GB300
    s = SimusStrategy(strategy)
    if s in (SimusStrategy.GB300, SimusStrategy.CUDA):
        return SimusStrategy.GB300
    raise NotImplementedError(f"strategy {s.value!r} is a CPU/Apple backend of the reference; fastsimus_gb300 "
                              "implements only the GB300 CUDA sweep (strategy=None or 'gb300')")


def _flatten(scatterers, rc, device):
    sc = _device.to_dev_f64(scatterers, device)
    n = sc.shape[0] if sc.ndim >= 2 else 1
    sc = sc.reshape(-1, 2) if sc.ndim != 2 else sc
    r = _device.to_dev_f64(rc, device).reshape(-1)
    if r.shape[0] != sc.shape[0]:
        raise ValueError(f"rc has {r.shape[0]} entries for {sc.shape[0]} scatterers")
    del n
    return sc.contiguous(), r.contiguous()


def _delays_apod(delays, tx_apodization, n_elements, device):
    d = _device.to_dev_f64(delays, device).reshape(-1)
    if d.shape[0] != n_elements:
        raise ValueError(f"delays has {d.shape[0]} entries for {n_elements} elements")
    a = None
    if tx_apodization is not None:
        a = _device.to_dev_f64(tx_apodization, device).reshape(-1)
        if a.shape[0] != n_elements:
            raise ValueError(f"tx_apodization has {a.shape[0]} entries for {n_elements} elements")
    return d, a


def _launch_simus(scat, rc, d, a, plan: SimusPlan, params: TransducerParams, medium: MediumParams,
                  ffd: bool, layout: int, device) -> torch.Tensor:
    lib = _native.load()
    tabs = _device.plan_tables(plan, device)
    probe = _native.make_probe(params, plan.n_sub)
    med = _native.make_medium(medium)
    fplan = tabs.fsg_plan(plan)
    n_scat = int(scat.shape[0])
    ws_bytes = lib.fsg_simus_workspace_size(probe, fplan, n_scat)
    if ws_bytes == 0:
        _native.check(_native.FSG_EINVAL)
    ws = _device.workspace(ws_bytes, device)
    rows = plan.n_freq_full if layout == _native.FSG_OUT_FULL_CORRECTED else tabs.n_freq
    out = torch.empty((rows, params.n_elements), dtype=torch.complex64, device=device)
    with torch.cuda.device(device), _device.timed("fsg_simus", device):
        st = lib.fsg_simus(probe, med, fplan, scat.data_ptr() if n_scat else None,
                           rc.data_ptr() if n_scat else None, n_scat, d.data_ptr(),
                           a.data_ptr() if a is not None else None, int(bool(ffd)), layout, out.data_ptr(),
                           ws.data_ptr(), ws.numel(), _device.stream_handle(device))
    _native.check(st)
    return out


def simus_gb300(scatterers, rc, params: TransducerParams, plan: SimusPlan, medium: MediumParams, delays_clean,
                tx_apodization, *, full_frequency_directivity: bool = False) -> torch.Tensor:
    """Backend hook with the reference's ``simus_cuda`` signature (kernels/cuda_simus.py:232-321):
    returns the selected-band spectrum (n_freq, n_elements) complex64 before ``correction_factor``."""
    device = _device.pick_device(scatterers, rc, delays_clean)
    scat, r = _flatten(scatterers, rc, device)
    d, a = _delays_apod(delays_clean, tx_apodization, params.n_elements, device)
    return _launch_simus(scat, r, d, a, plan, params, medium, full_frequency_directivity,
                         _native.FSG_OUT_SELECTED_RAW, device)


def irfft_and_threshold(full_spectrum: torch.Tensor, plan: SimusPlan, *, k_first: int = 0, k_count: int | None = None,
                        gate: bool = True) -> torch.Tensor:
    """rf = irfft(conj(S), n_fft, axis 0)[:(n_fft+1)//2] times the smooth -100 dB gate with each
    frame's own peak (simus.py:336-367), by ``fsg_irfft_gate``.  ``full_spectrum`` is one frame
    (n_freq_full, E) or a batch (B, n_freq_full, E) of complex64 on the GPU; only rows
    [k_first, k_first + k_count) are read, the others must be zero."""
    spec = full_spectrum if full_spectrum.dtype == torch.complex64 else full_spectrum.to(torch.complex64)
    spec = spec.contiguous()
    batched = spec.dim() == 3
    frames = spec if batched else spec.unsqueeze(0)
    nb, n_full, E = frames.shape
    if k_count is None:
        k_count = n_full - k_first
    n_fft = int(plan.n_fft)
    device = spec.device
    lib = _native.load()
    rf = torch.empty((nb, (n_fft + 1) // 2, E), dtype=torch.float32, device=device)
    ws = _device.workspace(lib.fsg_rf_workspace_size(n_fft, nb), device)
    _native.check(lib.fsg_irfft_gate(spec.data_ptr(), nb, n_full * E, n_full, E, n_fft, int(k_first), int(k_count),
                                     1 if gate else 0, rf.data_ptr(), ws.data_ptr(), ws.numel(),
                                     _device.stream_handle(device)))
    return rf if batched else rf[0]


def simus_compute(scatterers, rc, delays, plan: SimusPlan, params: TransducerParams,
                  medium: MediumParams = _DEFAULT_MEDIUM, *, tx_apodization=None,
                  full_frequency_directivity: bool = False, strategy: SimusStrategy | None = None) -> SimusResult:
    """RF signals for a precomputed plan (simus.py:392-495).  NaN delays switch their element
    off (apodization 0, delay 0), as in the reference."""
    _check_strategy(strategy)
    device = _device.pick_device(scatterers, rc, delays)
    scat, r = _flatten(scatterers, rc, device)
    d, a = _delays_apod(delays, tx_apodization, params.n_elements, device)
    full = _launch_simus(scat, r, d, a, plan, params, medium, full_frequency_directivity,
                         _native.FSG_OUT_FULL_CORRECTED, device)
    rf = irfft_and_threshold(full, plan, k_first=int(plan.freq_idx_start), k_count=int(plan.selected_freqs.shape[0]))
    return SimusResult(rf=rf.to(torch.float64), spectrum=full.to(torch.complex128))


def simus(scatterers, rc, delays, params: TransducerParams, medium: MediumParams = _DEFAULT_MEDIUM, *,
          fs: float | None = None, tx_apodization=None, tx_n_wavelengths: float = 1.0, db_thresh: float = -60.0,
          full_frequency_directivity: bool = False, element_splitting: int | None = None,
          frequency_step: float = 1.0, strategy: SimusStrategy | None = None) -> SimusResult:
    """Simulate per-element RF signals (simus.py:498-567): ``simus_precompute`` then
    ``simus_compute``."""
    _check_strategy(strategy)
    plan = simus_precompute(scatterers, rc, delays, params, medium, fs=fs, tx_n_wavelengths=tx_n_wavelengths,
                            db_thresh=db_thresh, element_splitting=element_splitting,
                            frequency_step=frequency_step)
    return simus_compute(scatterers, rc, delays, plan, params, medium, tx_apodization=tx_apodization,
                         full_frequency_directivity=full_frequency_directivity, strategy=strategy)
