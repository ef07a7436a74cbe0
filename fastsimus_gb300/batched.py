"""Many transmits x many phantoms in one persistent launch (libfsgb300 ``fsg_simus_batched``).

The reference simulates a multi-transmit acquisition with a caller loop: one plan per phantom,
computed with ``simus_precompute`` on the firing whose delay span is largest, then one
``simus_compute`` per firing with that plan (``tests/_picmus_phantom_shared.py:319-367``), and
RF stacked as (samples, channels, firings).  ``simus_batched`` keeps exactly that plan rule
and output layout, but computes every (phantom, firing) in a single launch: each Green's term
is generated once and contracted with all firings.

``BatchedSimus`` keeps inputs, plans, workspace and outputs resident for repeated runs,
captures the whole batch (set-up, persistent sweep, reduction, irfft + gate epilogue) in a
CUDA graph, and picks tile shapes with ``autotune``.
"""

from __future__ import annotations

import json
import os
import time
from dataclasses import dataclass
from pathlib import Path

import numpy as np
import torch

from fastsimus_gb300 import _device, _native
from fastsimus_gb300.params import MediumParams, TransducerParams
from fastsimus_gb300.plan import SimusPlan, simus_precompute
from fastsimus_gb300.simus import SimusResult

_DEFAULT_MEDIUM = MediumParams()


@dataclass(frozen=True)
class BatchTuning:
    """Tile shapes of the batched sweep: frequencies per work item (1 or 2; probes of more
    than 64 elements always use 1), scatterers per work item, persistent CTAs per SM, and for
    the FP32 kernel the scatterers per tile (32, 64, 128) and the FP32x2-packed register tile.
    ``FP32_SHAPES`` lists the compiled (freqs_per_item, elements tile, tile_scatterers,
    packed, ctas_per_sm) combinations."""

    freqs_per_item: int = 2
    chunk_scatterers: int = 32768
    ctas_per_sm: int = 1
    tile_scatterers: int = 64
    packed: int = 0
    threads_per_cta: int = 256

    @staticmethod
    def default(backend: str) -> "BatchTuning":
        return BatchTuning(7, 16384, 1) if backend == "tc" else BatchTuning()

    def to_c(self) -> _native.FsgBatchTuning:
        return _native.FsgBatchTuning(self.freqs_per_item, self.chunk_scatterers, self.ctas_per_sm,
                                      self.tile_scatterers, self.packed, self.threads_per_cta)


# (freqs_per_item, elements tile, tile_scatterers, packed, ctas_per_sm, threads_per_cta) compiled
# into batched_kernel
FP32_SHAPES = ((2, 64, 64, 0, 1, 256), (2, 64, 32, 0, 1, 256), (1, 64, 64, 0, 1, 256), (1, 64, 32, 0, 1, 256),
               (1, 64, 128, 0, 1, 256), (1, 64, 64, 1, 1, 256), (1, 64, 32, 1, 1, 256), (1, 64, 32, 0, 2, 256),
               (1, 128, 64, 0, 1, 256), (1, 128, 32, 0, 1, 256), (2, 64, 64, 0, 1, 512), (1, 64, 64, 0, 1, 512),
               (1, 64, 128, 0, 1, 512), (1, 128, 64, 0, 1, 512))


def fp32_search_space(n_elements: int, total_scatterers: int) -> list[BatchTuning]:
    """The FP32 autotuner's candidates: every compiled tile shape for the probe's element tile,
    each with two chunk sizes bracketing the batch (items enough to fill the SMs)."""
    eb = 64 if n_elements <= 64 else 128
    chunks = sorted({c for c in (8192, 16384, 32768, 65536) if c < 2 * max(total_scatterers, 64)} or {8192})
    chunks = [chunks[0], chunks[-1]] if len(chunks) > 1 else chunks
    return [BatchTuning(fb, c, cps, bt, pk, nth) for fb, e, bt, pk, cps, nth in FP32_SHAPES if e == eb
            for c in chunks]


def shared_plan(scatterers, rc, delays_list, params: TransducerParams, medium: MediumParams, **plan_kw) -> SimusPlan:
    """The reference's multi-firing plan rule: precompute on the firing with the largest delay
    span (tests/_picmus_phantom_shared.py:329-347)."""
    spans = [float(np.ptp(np.nan_to_num(np.asarray(d, dtype=np.float64)))) for d in delays_list]
    return simus_precompute(scatterers, rc, delays_list[int(np.argmax(spans))], params, medium, **plan_kw)


class BatchedSimus:
    """A resident batch: phantoms (scatterers, rc), one delay law per firing, shared plans."""

    def __init__(self, phantoms, delays, params: TransducerParams, medium: MediumParams = _DEFAULT_MEDIUM, *,
                 plans: list[SimusPlan] | None = None, tx_apodization=None, tuning: BatchTuning | None = None,
                 fs: float | None = None, device: torch.device | None = None, backend: str = "fp32",
                 full_frequency_directivity: bool = False):
        if backend not in ("fp32", "tc"):
            raise ValueError("backend must be 'fp32' (CUDA cores) or 'tc' (tcgen05 BF16 hi/lo tensor cores)")
        if full_frequency_directivity and backend == "tc":
            raise NotImplementedError("full_frequency_directivity is implemented by the fp32 batched backend "
                                      "(and fsg_simus); the tensor-core backend uses the centre-frequency "
                                      "directivity")
        self.backend = backend
        self.ffd = bool(full_frequency_directivity)
        self.device = device or _device.require_cuda()
        self.lib = _native.load()
        self.params, self.medium = params, medium
        d = np.asarray(delays, dtype=np.float64)
        if d.ndim != 2 or d.shape[1] != params.n_elements:
            raise ValueError(f"delays must be (n_tx, {params.n_elements}), got {d.shape}")
        self.n_tx = d.shape[0]
        self.phantoms = []
        for scat, rc in phantoms:
            s = _device.to_dev_f64(scat, self.device).reshape(-1, 2).contiguous()
            r = _device.to_dev_f64(rc, self.device).reshape(-1).contiguous()
            if r.shape[0] != s.shape[0]:
                raise ValueError("rc and scatterers differ in length")
            self.phantoms.append((s, r))
        if plans is None:
            plans = [shared_plan(s.cpu().numpy(), r.cpu().numpy(), list(d), params, medium, fs=fs)
                     for s, r in self.phantoms]
        self.plans = plans
        self.delays = torch.as_tensor(d, device=self.device).contiguous()
        self.apod = None
        if tx_apodization is not None:
            a = np.broadcast_to(np.asarray(tx_apodization, dtype=np.float64), d.shape)
            self.apod = torch.as_tensor(np.array(a, dtype=np.float64, order="C", copy=True),
                                        device=self.device).contiguous()
        self.tabs = [_device.plan_tables(p, self.device) for p in plans]
        self.outs = [torch.empty((self.n_tx, p.n_freq_full, params.n_elements), dtype=torch.complex64,
                                 device=self.device) for p in plans]
        self.probe = _native.make_probe(params, plans[0].n_sub)
        if any(p.n_sub != plans[0].n_sub for p in plans):
            raise ValueError("all phantoms of a batch must share n_sub")
        self.med = _native.make_medium(medium)
        self.graph = None
        self.set_tuning(tuning or BatchTuning.default(backend))

    # -- native call -------------------------------------------------------------------------
    def _fsg_phantoms(self):
        arr = (_native.FsgPhantom * len(self.phantoms))()
        for i, ((s, r), p, t, o) in enumerate(zip(self.phantoms, self.plans, self.tabs, self.outs)):
            arr[i].scat_xz = s.data_ptr()
            arr[i].rc = r.data_ptr()
            arr[i].n_scat = int(s.shape[0])
            arr[i].plan = t.fsg_plan(p)
            arr[i].out = o.data_ptr()
        return arr

    def set_tuning(self, tuning: BatchTuning):
        self.tuning = tuning
        self._ph = self._fsg_phantoms()
        if self.backend == "tc":
            nbytes = self.lib.fsg_simus_batched_tc_workspace_size(self.probe, self._ph, len(self.phantoms), self.n_tx,
                                                                  tuning.to_c())
        else:
            nbytes = self.lib.fsg_simus_batched_workspace_size(self.probe, self._ph, len(self.phantoms), self.n_tx,
                                                               int(self.ffd), tuning.to_c())
        if nbytes == 0:
            raise ValueError("fsg_simus_batched_workspace_size rejected the batch")
        self.ws = _device.workspace(nbytes, self.device)
        self.graph = None

    def launch_sweep(self):
        """Enqueue the batched sweep on the current stream (outputs: corrected spectra)."""
        apod = self.apod.data_ptr() if self.apod is not None else None
        with torch.cuda.device(self.device), _device.timed("fsg_simus_batched", self.device):
            if self.backend == "tc":
                st = self.lib.fsg_simus_batched_tc(self.probe, self.med, self._ph, len(self.phantoms),
                                                   self.delays.data_ptr(), apod, self.n_tx, self.tuning.to_c(),
                                                   self.ws.data_ptr(), self.ws.numel(),
                                                   _device.stream_handle(self.device))
            else:
                st = self.lib.fsg_simus_batched(self.probe, self.med, self._ph, len(self.phantoms),
                                                self.delays.data_ptr(), apod, self.n_tx, int(self.ffd),
                                                self.tuning.to_c(), self.ws.data_ptr(), self.ws.numel(),
                                                _device.stream_handle(self.device))
        _native.check(st)

    def device_status(self) -> int:
        """Synchronise and return the device-side status of the last tensor-core sweep
        (0 = ok, 3 = a bounded wait gave up); always 0 for the FP32 backend."""
        if self.backend != "tc":
            return 0
        import ctypes

        out = ctypes.c_int32(-1)
        _native.check(self.lib.fsg_simus_batched_tc_status(self.ws.data_ptr(), self.probe, self._ph,
                                                            len(self.phantoms), self.n_tx, self.tuning.to_c(),
                                                            ctypes.byref(out), _device.stream_handle(self.device)))
        return int(out.value)

    def _finish(self):
        """RF of every firing: ``fsg_irfft_gate`` over each phantom's (n_tx, n_freq_full, E)
        spectra, each firing gated with its own peak.  Buffers persist across calls, so a CUDA
        graph that captured this keeps writing into ``self.rfs``."""
        lib = _native.load()
        if getattr(self, "_rf_bufs", None) is None:
            E = self.params.n_elements
            self._rf_bufs = [torch.empty((self.n_tx, (p.n_fft + 1) // 2, E), dtype=torch.float32, device=self.device)
                             for p in self.plans]
            self._rf_ws = [_device.workspace(lib.fsg_rf_workspace_size(int(p.n_fft), self.n_tx), self.device)
                           for p in self.plans]
        stream = _device.stream_handle(self.device)
        for plan, out, rf, ws in zip(self.plans, self.outs, self._rf_bufs, self._rf_ws):
            n_full, E = out.shape[1], out.shape[2]
            _native.check(lib.fsg_irfft_gate(out.data_ptr(), self.n_tx, n_full * E, n_full, E, int(plan.n_fft),
                                             int(plan.freq_idx_start), int(plan.selected_freqs.shape[0]), 1,
                                             rf.data_ptr(), ws.data_ptr(), ws.numel(), stream))
        self.rfs = self._rf_bufs

    def run(self) -> list[SimusResult]:
        """One pass (eager launches).  Returns, per phantom, rf (n_samples, E, n_tx) and
        spectrum (n_freq_full, E, n_tx) -- the reference helper's (samples, channels, firings)."""
        self.launch_sweep()
        self._finish()
        return self.results()

    def results(self) -> list[SimusResult]:
        return [SimusResult(rf=rf.permute(1, 2, 0), spectrum=o.permute(1, 2, 0)) for rf, o in zip(self.rfs, self.outs)]

    # -- CUDA graph ----------------------------------------------------------------------------
    def capture(self):
        """Record the whole batch in a CUDA graph (after one eager warm-up pass)."""
        self.run()
        torch.cuda.synchronize(self.device)
        g = torch.cuda.CUDAGraph()
        s = torch.cuda.Stream(self.device)
        s.wait_stream(torch.cuda.current_stream(self.device))
        with torch.cuda.stream(s):
            self.run()  # warm the capture stream (kernel attributes, lazy module loading)
        torch.cuda.current_stream(self.device).wait_stream(s)
        torch.cuda.synchronize(self.device)
        with torch.cuda.graph(g):
            self.launch_sweep()
            self._finish()
        self.graph = g
        return g

    def replay(self) -> list[SimusResult]:
        if self.graph is None:
            self.capture()
        self.graph.replay()
        return self.results()

    # -- autotuner -----------------------------------------------------------------------------
    def autotune(self, candidates: list[BatchTuning] | None = None, reps: int = 1, cache: bool = True) -> BatchTuning:
        """Time each candidate tiling on this batch with CUDA events and keep the fastest.
        Results are cached by (E, n_sub, n_tx, n_phantoms, log2 total scatterers, F bucket) in
        memory and in ``$FASTSIMUS_GB300_CACHE`` (default ``~/.cache/fastsimus_gb300``)."""
        key = self._tune_key()
        table = _load_cache() if cache else {}
        if cache and key in table:
            best = BatchTuning(**table[key])
            self.set_tuning(best)
            return best
        if candidates is None and self.backend == "tc":
            # band frequencies per item that fit TMEM: 7 up to 32 firings, 3 up to 64, 2 beyond
            top = 7 if self.n_tx <= 32 else (3 if self.n_tx <= 64 else 2)
            candidates = [BatchTuning(fb, c, 1) for fb in range(max(1, top - 2), top + 1) for c in (8192, 16384)]
        if candidates is None:
            total = sum(int(s.shape[0]) for s, _ in self.phantoms)
            candidates = fp32_search_space(self.params.n_elements, total)
        timings = []
        for cand in candidates:
            self.set_tuning(cand)
            self.launch_sweep()  # warm-up
            torch.cuda.synchronize(self.device)
            st, en = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            st.record()
            for _ in range(reps):
                self.launch_sweep()
            en.record()
            torch.cuda.synchronize(self.device)
            timings.append((st.elapsed_time(en) / reps, cand))
        best = min(timings, key=lambda x: x[0])[1]
        self.tune_log = [(t, c.__dict__) for t, c in timings]
        self.set_tuning(best)
        if cache:
            table[key] = best.__dict__
            _save_cache(table)
        return best

    def _tune_key(self) -> str:
        total = sum(int(s.shape[0]) for s, _ in self.phantoms)
        fbar = int(np.mean([p.selected_freqs.shape[0] for p in self.plans]))
        return (f"{self.backend}{'-ffd' if self.ffd else ''}-E{self.params.n_elements}-U{self.plans[0].n_sub}"
                f"-T{self.n_tx}-P{len(self.phantoms)}"
                f"-S{int(np.log2(max(total, 1)))}-F{fbar // 64}")


def _cache_path() -> Path:
    root = Path(os.environ.get("FASTSIMUS_GB300_CACHE", Path.home() / ".cache" / "fastsimus_gb300"))
    return root / "autotune.json"


_mem_cache: dict = {}


def _load_cache() -> dict:
    if _mem_cache:
        return _mem_cache
    try:
        _mem_cache.update(json.loads(_cache_path().read_text()))
    except Exception:
        pass
    return _mem_cache


def _save_cache(table: dict):
    _mem_cache.update(table)
    try:
        p = _cache_path()
        p.parent.mkdir(parents=True, exist_ok=True)
        tmp = p.with_suffix(f".{os.getpid()}.{time.time_ns()}.tmp")
        tmp.write_text(json.dumps(_mem_cache, indent=1, sort_keys=True))
        os.replace(tmp, p)
    except OSError:
        pass


def simus_batched(phantoms, delays, params: TransducerParams, medium: MediumParams = _DEFAULT_MEDIUM, *,
                  plans: list[SimusPlan] | None = None, tx_apodization=None, fs: float | None = None,
                  tuning: BatchTuning | None = None, backend: str = "fp32",
                  full_frequency_directivity: bool = False) -> list[SimusResult]:
    """RF of every (phantom, firing): ``phantoms`` is a list of (scatterers (S, 2), rc (S,)),
    ``delays`` is (n_tx, n_elements).  Returns per phantom rf (n_samples, E, n_tx) float32 and
    spectrum (n_freq_full, E, n_tx) complex64, on the GPU."""
    return BatchedSimus(phantoms, delays, params, medium, plans=plans, tx_apodization=tx_apodization,
                        tuning=tuning, fs=fs, backend=backend,
                        full_frequency_directivity=full_frequency_directivity).run()
