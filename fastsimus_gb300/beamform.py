"""Beamforming of simulated RF on the GPU: I/Q demodulation and delay-and-sum.

The reference's validation tests image simus RF with PyMUST
(``tests/_picmus_phantom_shared.py:407-460``), per firing::

    iq = pymust.rf2iq(rf, fs, fc)
    M = pymust.dasmtx(1j * np.array(iq.shape), x_grid, z_grid, param)   # param.TXdelay = firing
    image += (M @ iq.flatten(order="F")).reshape(x_grid.shape, order="F")

This module provides those steps with the same call shapes -- ``rf2iq`` and ``dasmtx`` (a torch
sparse CSR matrix on the GPU) -- and ``das``, which applies the delay-and-sum of every firing
in one kernel without forming the matrices.  The arithmetic is MUST's (restated in
``fsg_das.cu``); PyMUST itself is not a dependency.

I/Q arrays are returned as ``(..., n_samples, n_channels)`` views of channel-major storage
(the Fortran-order columns of each frame are contiguous), the layout ``das`` reads directly.
"""

from __future__ import annotations

import ctypes
import math
from dataclasses import dataclass

import numpy as np
import torch

from fastsimus_gb300 import _device, _native

RF2IQ_ORDER = 5  # MUST's rf2iq low-pass: 5th-order Butterworth


@dataclass
class DasParam:
    """The fields of a PyMUST ``Param`` that ``rf2iq``/``dasmtx`` read.  ``fnumber=None`` selects
    the f-number from the element directivity (``default_fnumber``)."""

    fc: float
    pitch: float
    Nelements: int
    width: float
    radius: float = math.inf
    c: float = 1540.0
    fs: float | None = None
    TXdelay: object = None
    fnumber: float | None = None
    t0: float = 0.0

    @classmethod
    def from_params(cls, params, medium=None, *, fs: float | None = None, tx_delay=None, fnumber=None) -> "DasParam":
        """From this package's ``TransducerParams`` (+ ``MediumParams``)."""
        c = float(medium.speed_of_sound) if medium is not None else 1540.0
        return cls(fc=float(params.freq_center), pitch=float(params.pitch), Nelements=int(params.n_elements),
                   width=float(params.element_width), radius=float(params.radius), c=c,
                   fs=4.0 * float(params.freq_center) if fs is None else float(fs), TXdelay=tx_delay,
                   fnumber=fnumber)


def default_fnumber(element_width: float, fc: float, c: float) -> float:
    """Receive f-number ``1 / (2 tan(alpha))``, alpha the angle at which the soft-baffle element
    directivity ``sinc(w sin(alpha) / lambda) cos(alpha)`` at fc falls to ``1 / sqrt(2)``."""
    lam = c / fc

    def directivity(a):
        u = element_width / lam * math.sin(a)
        return (1.0 if u == 0 else math.sin(math.pi * u) / (math.pi * u)) * math.cos(a)

    lo, hi = 0.0, math.pi / 2.0
    for _ in range(80):
        mid = 0.5 * (lo + hi)
        if directivity(mid) > 1.0 / math.sqrt(2.0):
            lo = mid
        else:
            hi = mid
    return 1.0 / (2.0 * math.tan(0.5 * (lo + hi)))


def _lowpass(fs: float, fc: float, bandwidth: float | None):
    """rf2iq's low-pass as second-order sections (b0, b1, b2, 1, a1, a2) and their steady-state
    initial conditions for a unit input."""
    import scipy.signal

    wn = min(2.0 * fc / fs, 0.5) if bandwidth is None else bandwidth / fs
    sos = scipy.signal.butter(RF2IQ_ORDER, wn, output="sos")
    return np.ascontiguousarray(sos, np.float64), np.ascontiguousarray(scipy.signal.sosfilt_zi(sos), np.float64)


def rf2iq(rf, fs: float, fc: float, B: float | None = None, tau: float = 0.0) -> torch.Tensor:
    """I/Q components of RF signals (MUST ``rf2iq``): down-mixing by ``exp(-2 pi i fc t)``,
    ``t = n / fs + tau``, then a zero-phase 5th-order Butterworth low-pass (cut-off
    ``min(2 fc / fs, 0.5)`` of Nyquist, or ``B / fs`` for a bandwidth B in Hz), times 2.  The
    filter is applied as in ``scipy.signal.filtfilt`` (odd padding of 18 samples, steady-state
    initial conditions), run on the GPU as cascaded second-order sections in FP32.

    ``rf``: ``(n_samples, n_channels)`` or ``(n_frames, n_samples, n_channels)``, NumPy or
    torch; returns complex64 of the same shape on the GPU."""
    device = _device.pick_device(rf)
    x = rf if isinstance(rf, torch.Tensor) else torch.as_tensor(np.asarray(rf))
    x = x.to(device=device, dtype=torch.float32)
    if x.dim() not in (2, 3):
        raise ValueError(f"rf must be (n_samples, n_channels) or (n_frames, n_samples, n_channels), got {tuple(x.shape)}")
    frames = x.unsqueeze(0) if x.dim() == 2 else x
    frames = frames.contiguous()
    nf, ns, nc = frames.shape
    pad = 3 * (RF2IQ_ORDER + 1)
    if ns <= pad:
        raise ValueError(f"rf2iq needs more than {pad} samples per channel, got {ns}")
    sos, zi = _lowpass(float(fs), float(fc), B)
    out = torch.empty((nf, nc, ns), dtype=torch.complex64, device=device)
    lib = _native.load()
    dp = ctypes.POINTER(ctypes.c_double)
    _native.check(lib.fsg_rf2iq(frames.data_ptr(), nf, ns, nc, float(fs), float(fc), float(tau), sos.shape[0],
                                sos.ctypes.data_as(dp), zi.ctypes.data_as(dp), pad, out.data_ptr(),
                                _device.stream_handle(device)))
    iq = out.transpose(1, 2)
    return iq if x.dim() == 3 else iq[0]


def _das_call(param, method: str, iq: bool):
    methods = {"linear": _native.FSG_DAS_LINEAR, "nearest": _native.FSG_DAS_NEAREST}
    if method not in methods:
        raise ValueError(f"unknown interpolation method {method!r} (linear, nearest)")
    if param.fs is None:
        raise ValueError("param.fs (sampling frequency) is required")
    c = float(getattr(param, "c", 1540.0))
    fn = getattr(param, "fnumber", None)
    fn = default_fnumber(float(param.width), float(param.fc), c) if fn is None else float(fn)
    radius = float(getattr(param, "radius", math.inf))
    probe = _native.FsgProbe(n_elements=int(param.Nelements), n_sub=1, pitch=float(param.pitch),
                             element_width=float(param.width), radius=radius if math.isfinite(radius) else math.inf,
                             freq_center=float(param.fc), baffle=0, reserved0=0, baffle_impedance=0.0)
    p = _native.FsgDasParams(speed_of_sound=c, fs=float(param.fs), fc=float(param.fc),
                             t0=float(getattr(param, "t0", 0.0) or 0.0), fnumber=fn, method=methods[method],
                             iq=1 if iq else 0)
    return probe, p


def _pixels(x, z, device):
    xa, za = np.asarray(x, dtype=np.float64), np.asarray(z, dtype=np.float64)
    if xa.shape != za.shape:
        raise ValueError(f"x and z must have the same shape, got {xa.shape} and {za.shape}")
    # rows follow the Fortran order of the grid, as pymust.dasmtx's do
    pix = np.stack([xa.reshape(-1, order="F"), za.reshape(-1, order="F")], axis=1)
    return torch.as_tensor(np.ascontiguousarray(pix), device=device), xa.shape


def _from_fortran(flat: torch.Tensor, shape) -> torch.Tensor:
    if len(shape) <= 1:
        return flat.reshape(shape)
    return flat.reshape(tuple(reversed(shape))).permute(*reversed(range(len(shape))))


def dasmtx(sig, x, z, param, method: str = "linear") -> torch.Tensor:
    """Delay-and-sum matrix of one firing (MUST ``dasmtx``), delays from ``param.TXdelay``.

    ``sig`` is the signal or its shape: ``1j * np.array((n_samples, n_channels))`` for I/Q
    signals (as the reference's tests pass it), a real shape for RF, or an array.  Returns a
    complex64 sparse CSR tensor of ``x.size`` rows (pixels in Fortran order of the grid) and
    ``n_samples * n_channels`` columns (the Fortran-order flattening of the signal)."""
    if isinstance(sig, torch.Tensor):
        iq = bool(torch.is_complex(sig))
        ns, nc = int(sig.shape[-2]), int(sig.shape[-1])
    else:
        s = np.asarray(sig)
        if s.shape == (2,) and s.dtype.kind in "fc":
            iq = bool(np.iscomplexobj(s))
            ns, nc = (int(round(abs(v))) for v in s)
        else:
            iq = bool(np.iscomplexobj(s))
            ns, nc = int(s.shape[-2]), int(s.shape[-1])
    if nc != int(param.Nelements):
        raise ValueError(f"signal has {nc} channels but param.Nelements = {param.Nelements}")
    if param.TXdelay is None:
        raise ValueError("param.TXdelay is required")
    device = _device.require_cuda()
    probe, p = _das_call(param, method, iq)
    pix, shape = _pixels(x, z, device)
    txd = _device.to_dev_f64(param.TXdelay, device, (nc,))
    per = int(_native.load().fsg_dasmtx_nnz_per_row(p.method, nc))
    n = pix.shape[0]
    crow = torch.empty(n + 1, dtype=torch.int32, device=device)
    col = torch.empty(max(n * per, 1), dtype=torch.int32, device=device)
    val = torch.empty(max(n * per, 1), dtype=torch.complex64, device=device)
    _native.check(_native.load().fsg_dasmtx(ctypes.byref(probe), ctypes.byref(p), ns, txd.data_ptr(), pix.data_ptr(),
                                            n, crow.data_ptr(), col.data_ptr(), val.data_ptr(),
                                            _device.stream_handle(device)))
    return torch.sparse_csr_tensor(crow, col[:n * per], val[:n * per], size=(n, ns * nc))


def das(iq, x, z, delays, param, method: str = "linear") -> torch.Tensor:
    """Compounded delay-and-sum image: the sum over firings of ``dasmtx(iq_f, x, z, param with
    TXdelay = delays[f]) @ iq_f.flatten(order="F")``, computed in one kernel without the
    matrices.  ``iq``: ``(n_samples, n_channels)`` or ``(n_frames, n_samples, n_channels)``
    (complex I/Q or real RF); ``delays``: ``(n_channels,)`` or ``(n_frames, n_channels)``.
    Returns complex64 of x's shape."""
    device = _device.pick_device(iq)
    t = iq if isinstance(iq, torch.Tensor) else torch.as_tensor(np.asarray(iq))
    t = t.to(device)
    is_iq = torch.is_complex(t)
    t = t.to(torch.complex64)
    frames = t.unsqueeze(0) if t.dim() == 2 else t
    nf, ns, nc = frames.shape
    if nc != int(param.Nelements):
        raise ValueError(f"signal has {nc} channels but param.Nelements = {param.Nelements}")
    cm = frames.transpose(1, 2).contiguous()  # channel-major; no copy for rf2iq output
    d = np.asarray(delays.cpu() if isinstance(delays, torch.Tensor) else delays, dtype=np.float64)
    d = d.reshape(1, nc) if d.ndim == 1 else d
    if d.shape != (nf, nc):
        raise ValueError(f"delays must be ({nf}, {nc}), got {d.shape}")
    txd = torch.as_tensor(np.ascontiguousarray(d), device=device)
    probe, p = _das_call(param, method, is_iq)
    pix, shape = _pixels(x, z, device)
    out = torch.empty(pix.shape[0], dtype=torch.complex64, device=device)
    _native.check(_native.load().fsg_das(ctypes.byref(probe), ctypes.byref(p), cm.data_ptr(), nf, ns, txd.data_ptr(),
                                         pix.data_ptr(), pix.shape[0], out.data_ptr(),
                                         _device.stream_handle(device)))
    return _from_fortran(out, shape)
