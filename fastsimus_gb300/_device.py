"""Device plumbing: tensors in HBM, plan tables on the device, workspaces, streams.

PyTorch is used only for device memory and streams; all arithmetic of the path (sweeps,
reductions, the spectrum-to-RF epilogue) runs in libfsgb300.so.
"""

from __future__ import annotations

import numpy as np
import torch

from fastsimus_gb300 import _native


def require_cuda() -> torch.device:
    if not torch.cuda.is_available():
        raise RuntimeError("fastsimus_gb300 runs only on a CUDA GPU (sm_103a); no CUDA device is visible and there "
                           "is no CPU fallback")
    _native.load()
    return torch.device("cuda", torch.cuda.current_device())


def pick_device(*arrays) -> torch.device:
    for a in arrays:
        if isinstance(a, torch.Tensor) and a.is_cuda:
            return a.device
    return require_cuda()


def to_dev_f64(a, device: torch.device, shape=None) -> torch.Tensor:
    """Contiguous float64 tensor on `device` (copies host arrays in).  A pinned host tensor is
    copied asynchronously on the current stream, so the caller must leave it unchanged until the
    stream has passed the call; other host inputs are copied synchronously."""
    if isinstance(a, torch.Tensor):
        t = a.to(device=device, dtype=torch.float64, non_blocking=(not a.is_cuda) and a.is_pinned())
    else:
        t = torch.as_tensor(np.asarray(a, dtype=np.float64), device=device)
    if shape is not None:
        t = t.reshape(shape)
    return t.contiguous()


class PlanTables:
    """Device copies of a plan's pulse (complex128 interleaved) and probe spectra."""

    def __init__(self, plan, device: torch.device):
        ps = np.ascontiguousarray(np.asarray(plan.pulse_spectrum, dtype=np.complex128))
        self.pulse = torch.as_tensor(ps.view(np.float64), device=device)
        self.probe = torch.as_tensor(np.ascontiguousarray(np.asarray(plan.probe_spectrum, dtype=np.float64)),
                                     device=device)
        f = np.asarray(plan.selected_freqs, dtype=np.float64)
        self.n_freq = int(f.shape[0])
        self.freq_start = float(f[0])
        self.freq_step = float(f[1] - f[0]) if f.shape[0] > 1 else 0.0

    def fsg_plan(self, plan) -> _native.FsgFreqPlan:
        return _native.FsgFreqPlan(
            n_freq=self.n_freq,
            n_freq_full=int(getattr(plan, "n_freq_full", 0)),
            freq_idx_start=int(getattr(plan, "freq_idx_start", 0)),
            reserved0=0,
            freq_start=self.freq_start,
            freq_step=self.freq_step,
            seg_length=float(plan.seg_length),
            correction_factor=float(plan.correction_factor),
            pulse_spectrum=self.pulse.data_ptr(),
            probe_spectrum=self.probe.data_ptr(),
        )


_plan_cache: dict = {}


def plan_tables(plan, device: torch.device) -> PlanTables:
    """Per-(plan, device) cache of the device spectra; holds the plan alive while cached."""
    key = (id(plan), str(device))
    hit = _plan_cache.get(key)
    if hit is not None and hit[0] is plan:
        return hit[1]
    if len(_plan_cache) > 32:
        _plan_cache.clear()
    tabs = PlanTables(plan, device)
    _plan_cache[key] = (plan, tabs)
    return tabs


def workspace(nbytes: int, device: torch.device) -> torch.Tensor:
    return torch.empty(max(int(nbytes), 256), dtype=torch.uint8, device=device)


def stream_handle(device: torch.device) -> int:
    return torch.cuda.current_stream(device).cuda_stream


class LaunchTimer:
    """Records CUDA events around each native call on the launching stream (set by a caller
    that wants per-call device times; off by default)."""

    def __init__(self):
        self.events: dict[str, list] = {}

    def elapsed_ms(self, name: str) -> list[float]:
        return [a.elapsed_time(b) for a, b in self.events.get(name, [])]


_timer: LaunchTimer | None = None


def set_timer(timer: LaunchTimer | None):
    global _timer
    _timer = timer


class timed:
    def __init__(self, name: str, device: torch.device):
        self.name = name
        self.device = device
        self.start = None

    def __enter__(self):
        if _timer is not None:
            self.start = torch.cuda.Event(enable_timing=True)
            self.start.record(torch.cuda.current_stream(self.device))
        return self

    def __exit__(self, *exc):
        if _timer is not None and self.start is not None:
            end = torch.cuda.Event(enable_timing=True)
            end.record(torch.cuda.current_stream(self.device))
            _timer.events.setdefault(self.name, []).append((self.start, end))
        return False
