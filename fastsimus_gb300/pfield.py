"""Public pfield API, drop-in for the reference's ``fast_simus.pfield`` module (pfield.py:41-475).

Returns the RMS pressure field as a float64 torch tensor (the reference's dtype; computed in
FP32 with double-float phases) of shape ``positions.shape[:-1]`` on the current CUDA device.  ``PfieldStrategy`` keeps the reference's values and adds ``GB300``;
``None`` selects it.  VECTORIZED/SCAN (CPU) and METAL (Apple) raise ``NotImplementedError``.
"""

from __future__ import annotations

from enum import StrEnum

import torch

from fastsimus_gb300 import _device, _native
from fastsimus_gb300.params import MediumParams, TransducerParams
from fastsimus_gb300.plan import PfieldPlan, pfield_precompute

_DEFAULT_MEDIUM = MediumParams()


class PfieldStrategy(StrEnum):
    """Sweep strategy (pfield.py:41-55) plus GB300."""

    VECTORIZED = "vectorized"
    SCAN = "scan"
    METAL = "metal"
    GB300 = "gb300"


def _check_strategy(strategy):
    if strategy is None or PfieldStrategy(strategy) == PfieldStrategy.GB300:
        return PfieldStrategy.GB300
    raise NotImplementedError(f"strategy {PfieldStrategy(strategy).value!r} is a CPU/Apple backend of the reference; "
                              "fastsimus_gb300 implements only the GB300 CUDA sweep")


def pfield_compute(positions, delays, plan: PfieldPlan, params: TransducerParams,
                   medium: MediumParams = _DEFAULT_MEDIUM, *, tx_apodization=None,
                   full_frequency_directivity: bool = False, strategy: PfieldStrategy | None = None) -> torch.Tensor:
    """RMS pressure field for a precomputed plan (pfield.py:301-378)."""
    _check_strategy(strategy)
    device = _device.pick_device(positions, delays, tx_apodization)
    pos = _device.to_dev_f64(positions, device)
    grid_shape = tuple(pos.shape[:-1])
    pts = pos.reshape(-1, 2).contiguous()
    n = int(pts.shape[0])
    if n == 0:
        raise ValueError("Grid has no points")
    d = _device.to_dev_f64(delays, device).reshape(-1)
    if d.shape[0] != params.n_elements:
        raise ValueError(f"delays has {d.shape[0]} entries for {params.n_elements} elements")
    a = None
    if tx_apodization is not None:
        a = _device.to_dev_f64(tx_apodization, device).reshape(-1)
    lib = _native.load()
    tabs = _device.plan_tables(plan, device)
    probe = _native.make_probe(params, plan.n_sub)
    med = _native.make_medium(medium)
    fplan = tabs.fsg_plan(plan)
    ws_bytes = lib.fsg_pfield_workspace_size(probe, fplan, n)
    if ws_bytes == 0:
        _native.check(_native.FSG_EINVAL)
    ws = _device.workspace(ws_bytes, device)
    out = torch.empty(n, dtype=torch.float32, device=device)
    with torch.cuda.device(device), _device.timed("fsg_pfield", device):
        st = lib.fsg_pfield(probe, med, fplan, pts.data_ptr(), n, d.data_ptr(),
                            a.data_ptr() if a is not None else None, int(bool(full_frequency_directivity)),
                            out.data_ptr(), ws.data_ptr(), ws.numel(), _device.stream_handle(device))
    _native.check(st)
    return out.reshape(grid_shape).to(torch.float64)


def pfield(positions, delays, params: TransducerParams, medium: MediumParams = _DEFAULT_MEDIUM, *,
           tx_apodization=None, tx_n_wavelengths: float = 1.0, db_thresh: float = -60.0,
           full_frequency_directivity: bool = False, element_splitting: int | None = None,
           frequency_step: float = 1.0, strategy: PfieldStrategy | None = None) -> torch.Tensor:
    """RMS acoustic pressure field of the array (pfield.py:381-475)."""
    _check_strategy(strategy)
    plan = pfield_precompute(positions, delays, params, medium, tx_n_wavelengths=tx_n_wavelengths,
                             db_thresh=db_thresh, element_splitting=element_splitting,
                             frequency_step=frequency_step)
    return pfield_compute(positions, delays, plan, params, medium, tx_apodization=tx_apodization,
                          full_frequency_directivity=full_frequency_directivity, strategy=strategy)
