"""Learned transmit-field surrogate with the exact transmit kernel as error check and fallback.

The network maps (x, z, f, theta) -- a point, a frequency and a plane-wave steering angle --
to the complex transmit pressure of the array (the pressure inside the pfield step body,
_pfield_strategies.py:48, before |.|^2).  Architecture: 64 random Fourier features of the
normalised inputs, 4 hidden layers of width 256 with SiLU, a linear head; BF16 weights, FP32
accumulation.

The field oscillates at the wavelength in space and at 1/delay in frequency, and beside the
plane wave of the firing it carries the waves that start at the two ends of the aperture and,
at the pitch of these arrays (about one wavelength), the first grating lobes.  The head
therefore predicts the complex amplitudes a_j of five analytic carriers c_j -- the ideal plane
wave, the two edge waves and the grating lobes m = -1, +1, whose phases are computed exactly
(FP64) from the geometry -- and the field is  p = scale * sum_j a_j c_j.  What is left to learn
is a set of slowly varying amplitudes.

Training runs entirely in libfsgb300's tcgen05 kernels (fsg_mlp_train_*): a step gathers its
rows on the device, runs forward and backward on the tensor cores, reduces the weight
gradients on the tensor cores and applies Adam, in three launches with no host
synchronisation; the step counter, learning-rate schedule and loss history are device state,
so many steps are replayed from one CUDA graph.  Inference is the fused tcgen05 forward pass
(fsg_mlp_tc_forward) followed by fsg_surrogate_combine.  PyTorch only holds the buffers.

In simus the network supplies the transmit field at every (scatterer, frequency, firing) inside
its domain; the exact kernel ``fsg_txfield`` checks each (tile of scatterers, firing) on a few
of its scatterers and recomputes the pairs whose relative L2 error exceeds the tolerance.
Queries outside the network's domain (points outside the box, steering angles beyond it,
frequencies outside its band) are computed exactly.  ``simus_with_surrogate`` returns the
timings that show what the network gains (or loses) against the exact path.
"""

from __future__ import annotations

import ctypes
import math
import time
from dataclasses import dataclass

import numpy as np
import torch

from fastsimus_gb300 import _device, _native
from fastsimus_gb300.params import MediumParams, TransducerParams

HIDDEN = 256
DEPTH = 4
N_FOURIER = 64
TILE_ROWS = 128
AUX = 12  # floats per training row: five complex carriers and the complex target


@dataclass
class Box:
    """Domain of the surrogate: x, z ranges (m), band (Hz), max |steering angle| (rad)."""

    x: tuple
    z: tuple
    f: tuple
    max_angle: float


def _check(st):
    _native.check(st)


def mlp_flops_per_sample(n_out: int) -> float:
    """Forward multiply-adds x 2 of one query: 128 -> 256 -> 256 -> 256 -> 256 -> n_out."""
    return 2.0 * (2 * N_FOURIER * HIDDEN + (DEPTH - 1) * HIDDEN * HIDDEN + HIDDEN * n_out)


class TxFieldSurrogate:
    def __init__(self, params: TransducerParams, medium: MediumParams, box: Box, *, n_carriers: int = 5,
                 sigma: float = 0.5, seed: int = 0, device: torch.device | None = None,
                 tx_n_wavelengths: float = 1.0):
        if not params.is_linear:
            raise NotImplementedError("the transmit-field surrogate supports linear arrays")
        if n_carriers not in (1, 2, 3, 4, 5):
            raise ValueError("n_carriers must be in 1..5")
        self.params, self.medium, self.box = params, medium, box
        self.device = device or _device.require_cuda()
        self.lib = _native.load()
        self.tx_n_wavelengths = tx_n_wavelengths
        self.n_out = 2 * n_carriers
        dev = self.device
        g = torch.Generator().manual_seed(seed)
        self.bmat = (torch.randn(N_FOURIER, 4, generator=g) * sigma).to(dev).contiguous()
        # PyTorch's nn.Linear initialisation: U(-1/sqrt(fan_in), 1/sqrt(fan_in)) for weights and biases
        shapes = [(HIDDEN, 2 * N_FOURIER)] + [(HIDDEN, HIDDEN)] * (DEPTH - 1) + [(self.n_out, HIDDEN)]
        self.W, self.b = [], []
        for fan_out, fan_in in shapes:
            bound = 1.0 / math.sqrt(fan_in)
            self.W.append(((torch.rand(fan_out, fan_in, generator=g) * 2 - 1) * bound).to(dev).contiguous())
            self.b.append(((torch.rand(fan_out, generator=g) * 2 - 1) * bound).to(dev).contiguous())
        self.mW = [torch.zeros_like(w) for w in self.W]
        self.vW = [torch.zeros_like(w) for w in self.W]
        self.mb = [torch.zeros_like(b) for b in self.b]
        self.vb = [torch.zeros_like(b) for b in self.b]
        self.packed_fwd = [torch.empty(self.lib.fsg_mlp_tc_packed_bytes(w.shape[1]), dtype=torch.uint8, device=dev)
                           for w in self.W[:DEPTH]]
        self.packed_bwd = [None] + [torch.empty(HIDDEN * HIDDEN * 2, dtype=torch.uint8, device=dev)
                                    for _ in range(DEPTH - 1)]
        self.packed_head = torch.zeros(24576, dtype=torch.uint8, device=dev)  # W_head, BF16 hi/lo + MN-major hi
        self.step_counter = torch.zeros(1, dtype=torch.int32, device=dev)
        self.status = torch.zeros(1, dtype=torch.int32, device=dev)
        self.scale = 1.0
        self.probe = _native.make_probe(params, self._n_sub())
        self.med = _native.make_medium(medium)
        self.ws = _device.workspace(params.n_elements * self._n_sub() * 16 + params.n_elements * 8 + 1024, dev)
        self.domain = _native.FsgSurrogateDomain(
            x_lo=box.x[0], x_hi=box.x[1], z_lo=box.z[0], z_hi=box.z[1], f_lo=box.f[0], f_hi=box.f[1],
            max_angle=box.max_angle, pitch=float(params.pitch), speed_of_sound=float(medium.speed_of_sound),
            n_elements=int(params.n_elements), n_carriers=n_carriers)
        self._pack()

    def _n_sub(self):
        lam_min = self.medium.speed_of_sound / (self.params.freq_center * (1.0 + self.params.bandwidth / 2.0))
        return math.ceil(self.params.element_width / lam_min)

    def _stream(self):
        return _device.stream_handle(self.device)

    # -- exact field, inputs, domain ------------------------------------------------------------
    def exact(self, samples: torch.Tensor) -> torch.Tensor:
        """Exact complex transmit pressure at samples (n, 4) float64 [x, z, f, theta]."""
        s = samples.to(device=self.device, dtype=torch.float64).contiguous()
        out = torch.empty(s.shape[0], dtype=torch.complex64, device=self.device)
        _check(self.lib.fsg_txfield(self.probe, self.med, self.tx_n_wavelengths, self.params.bandwidth, s.data_ptr(),
                                    s.shape[0], out.data_ptr(), self.ws.data_ptr(), self.ws.numel(), self._stream()))
        return out

    def inputs(self, samples: torch.Tensor, field: torch.Tensor | None = None, with_aux: bool = True):
        """Normalised inputs u (n, 4) float32 and, with_aux, the carriers and the scaled target
        (n, 12) float32, by fsg_surrogate_inputs."""
        s = samples.to(device=self.device, dtype=torch.float64).contiguous()
        n = s.shape[0]
        u = torch.empty(n, 4, dtype=torch.float32, device=self.device)
        aux = torch.empty(n, AUX, dtype=torch.float32, device=self.device) if with_aux else None
        _check(self.lib.fsg_surrogate_inputs(self.domain, s.data_ptr(), n,
                                             field.data_ptr() if field is not None else None, 1.0 / self.scale,
                                             u.data_ptr(), aux.data_ptr() if aux is not None else None,
                                             self._stream()))
        return u, aux

    def sample_domain(self, n: int, seed: int) -> torch.Tensor:
        g = torch.Generator(device="cpu").manual_seed(seed)
        b = self.box
        r = torch.rand(n, 4, generator=g, dtype=torch.float64)
        lo = torch.tensor([b.x[0], b.z[0], b.f[0], -b.max_angle], dtype=torch.float64)
        hi = torch.tensor([b.x[1], b.z[1], b.f[1], b.max_angle], dtype=torch.float64)
        return (lo + r * (hi - lo)).to(self.device)

    def in_domain(self, samples: torch.Tensor) -> torch.Tensor:
        b = self.box
        x, z, f, th = samples.unbind(-1)
        return ((x >= b.x[0]) & (x <= b.x[1]) & (z >= b.z[0]) & (z <= b.z[1]) & (f >= b.f[0]) & (f <= b.f[1])
                & (th.abs() <= b.max_angle))

    # -- network weights ------------------------------------------------------------------------
    def _pack(self):
        """The packed BF16 copies of the hidden layers from the FP32 weights (fsg_mlp_train_init
        also clears the training counters)."""
        t = self._train_struct(n_tiles=1, n_split=1, n_data=1, u=self.bmat, aux=self.bmat)
        _check(self.lib.fsg_mlp_train_init(ctypes.byref(t), self._stream()))

    def _weights_struct(self):
        w = _native.FsgMlpWeights()
        for layer in range(DEPTH):
            w.packed[layer] = self.packed_fwd[layer].data_ptr()
            w.bias[layer] = self.b[layer].data_ptr()
        w.w_head = self.W[DEPTH].data_ptr()
        w.b_head = self.b[DEPTH].data_ptr()
        w.bmat = self.bmat.data_ptr()
        w.n_out = self.n_out
        return w

    def _train_struct(self, *, n_tiles, n_split, n_data, u, aux, seed=0, total_steps=1, warmup=0, lr=1e-3,
                      lr_min=0.0, loss_hist=None):
        need = self.lib.fsg_mlp_train_workspace_size(n_tiles, n_split)
        if getattr(self, "_train_ws", None) is None or self._train_ws.numel() < need:
            self._train_ws = _device.workspace(need, self.device)
        t = _native.FsgMlpTrain()
        t.u, t.aux, t.n_data, t.seed = u.data_ptr(), aux.data_ptr(), int(n_data), int(seed)
        t.bmat = self.bmat.data_ptr()
        for layer in range(DEPTH):
            t.w[layer] = self.W[layer].data_ptr()
            t.m_w[layer] = self.mW[layer].data_ptr()
            t.v_w[layer] = self.vW[layer].data_ptr()
            t.packed_fwd[layer] = self.packed_fwd[layer].data_ptr()
            t.packed_bwd[layer] = self.packed_bwd[layer].data_ptr() if self.packed_bwd[layer] is not None else None
            t.b[layer] = self.b[layer].data_ptr()
            t.m_b[layer] = self.mb[layer].data_ptr()
            t.v_b[layer] = self.vb[layer].data_ptr()
        t.w_head, t.m_w_head, t.v_w_head = (self.W[DEPTH].data_ptr(), self.mW[DEPTH].data_ptr(),
                                            self.vW[DEPTH].data_ptr())
        t.b_head, t.m_b_head, t.v_b_head = (self.b[DEPTH].data_ptr(), self.mb[DEPTH].data_ptr(),
                                            self.vb[DEPTH].data_ptr())
        t.packed_head = self.packed_head.data_ptr()
        t.n_out, t.n_tiles, t.n_split = self.n_out, int(n_tiles), int(n_split)
        t.total_steps, t.warmup_steps = int(total_steps), int(warmup)
        t.lr, t.lr_min, t.beta1, t.beta2, t.eps = float(lr), float(lr_min), 0.9, 0.999, 1e-8
        t.step = self.step_counter.data_ptr()
        t.loss_hist = loss_hist.data_ptr() if loss_hist is not None else None
        t.loss_hist_len = int(loss_hist.numel()) if loss_hist is not None else 0
        t.status = self.status.data_ptr()
        t.workspace, t.workspace_bytes = self._train_ws.data_ptr(), self._train_ws.numel()
        return t

    def oracle_params(self):
        """FP64 copies of the parameters as the kernels multiply them: hidden-layer weights
        rounded to BF16 (their packed copies), the head and the biases in FP32."""
        W = [w.to(torch.bfloat16).double().cpu().numpy() for w in self.W[:DEPTH]]
        W.append(self.W[DEPTH].double().cpu().numpy())
        return self.bmat.double().cpu().numpy(), W, [b.double().cpu().numpy() for b in self.b]

    # -- training --------------------------------------------------------------------------------
    def make_dataset(self, n: int, seed: int, scale: float | None = None):
        """n exact samples over the box: (samples float64, u, aux); sets ``scale`` (the RMS of the
        field) unless given."""
        s = self.sample_domain(n, seed)
        p = self.exact(s)
        if scale is None:
            self.scale = float(torch.sqrt((p.abs().double() ** 2).mean()))
        u, aux = self.inputs(s, p)
        return s, u, aux, p

    def gradients(self, u: torch.Tensor, aux: torch.Tensor, n_tiles: int = 2, n_split: int = 3, seed: int = 0):
        """One training step's gradients (no update): (list of weight gradients, list of bias
        gradients, sampled rows), in the layout of self.W / self.b."""
        t = self._train_struct(n_tiles=n_tiles, n_split=n_split, n_data=u.shape[0], u=u, aux=aux, seed=seed)
        n_par = self.lib.fsg_mlp_train_n_params(self.n_out)
        g = torch.empty(n_par, dtype=torch.float32, device=self.device)
        rows = torch.empty(n_tiles * TILE_ROWS, dtype=torch.int32, device=self.device)
        _check(self.lib.fsg_mlp_train_init(ctypes.byref(t), self._stream()))
        _check(self.lib.fsg_mlp_train_gradients(ctypes.byref(t), g.data_ptr(), rows.data_ptr(), self._stream()))
        torch.cuda.synchronize(self.device)
        self._check_status()
        sizes = [w.numel() for w in self.W[:DEPTH]] + [b.numel() for b in self.b[:DEPTH]] + [
            self.W[DEPTH].numel(), self.b[DEPTH].numel()]
        parts = list(torch.split(g, sizes))
        gW = [parts[i].view_as(self.W[i]) for i in range(DEPTH)] + [parts[2 * DEPTH].view_as(self.W[DEPTH])]
        gb = [parts[DEPTH + i] for i in range(DEPTH)] + [parts[2 * DEPTH + 1]]
        return gW, gb, rows.long()

    def _check_status(self):
        st = int(self.status.item())
        if st != 0:
            raise _native.FsgError(st, "a bounded wait in the surrogate kernels gave up")

    def train(self, n_train: int = 2_000_000, steps: int = 30_000, n_tiles: int | None = None, n_split: int = 15,
              lr: float = 3e-3, lr_min: float = 0.0, warmup_frac: float = 0.05, n_val: int = 65536, seed: int = 0,
              block: int = 1000, evals: int = 5, log=None) -> dict:
        """Train on n_train exact samples for `steps` steps of 128 n_tiles rows (default: one
        tile per SM).  Steps run in CUDA-graph replays of `block` steps; the validation error is
        measured `evals` times.  Returns the history and the training throughput."""
        dev = self.device
        if n_tiles is None:
            n_tiles = torch.cuda.get_device_properties(dev).multi_processor_count
        t0 = time.perf_counter()
        s, u, aux, _ = self.make_dataset(n_train, seed)
        sv = self.sample_domain(n_val, seed + 1)
        yv = self.exact(sv)
        torch.cuda.synchronize(dev)
        t_data = time.perf_counter() - t0
        block = max(1, min(block, steps))
        steps = (steps // block) * block
        hist_loss = torch.zeros(steps, dtype=torch.float32, device=dev)
        t = self._train_struct(n_tiles=n_tiles, n_split=n_split, n_data=n_train, u=u, aux=aux, seed=seed,
                               total_steps=steps, warmup=int(warmup_frac * steps), lr=lr, lr_min=lr_min,
                               loss_hist=hist_loss)
        self._tstruct = t  # the captured graph reads it by pointer
        self.step_counter.zero_()
        self.status.zero_()
        _check(self.lib.fsg_mlp_train_init(ctypes.byref(t), self._stream()))
        # one gradient pass (no update) loads the three kernels before the capture
        g_tmp = torch.empty(self.lib.fsg_mlp_train_n_params(self.n_out), dtype=torch.float32, device=dev)
        r_tmp = torch.empty(n_tiles * TILE_ROWS, dtype=torch.int32, device=dev)
        _check(self.lib.fsg_mlp_train_gradients(ctypes.byref(t), g_tmp.data_ptr(), r_tmp.data_ptr(), self._stream()))
        torch.cuda.synchronize(dev)
        del g_tmp, r_tmp
        graph = torch.cuda.CUDAGraph()
        side = torch.cuda.Stream(dev)
        side.wait_stream(torch.cuda.current_stream(dev))
        with torch.cuda.stream(side):
            # the capture records `block` steps; the step counter lives on the device
            with torch.cuda.graph(graph, stream=side):
                _check(self.lib.fsg_mlp_train_steps(ctypes.byref(t), block, side.cuda_stream))
        torch.cuda.current_stream(dev).wait_stream(side)
        torch.cuda.synchronize(dev)
        hist, train_ms = [], 0.0
        eval_at = {max(1, round((i + 1) * (steps // block) / max(1, evals))) for i in range(evals)}
        for bi in range(steps // block):
            ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            ev0.record()
            graph.replay()
            ev1.record()
            torch.cuda.synchronize(dev)
            train_ms += ev0.elapsed_time(ev1)
            if (bi + 1) in eval_at:
                self._check_status()
                val = self.relative_error(sv, yv)
                lo = (bi + 1 - 1) * block
                rec = {"step": (bi + 1) * block, "train_loss": float(hist_loss[lo:(bi + 1) * block].mean()),
                       "val_rel_l2": val}
                hist.append(rec)
                if log:
                    log(rec)
        self._check_status()
        samples = steps * n_tiles * TILE_ROWS
        flops = 3.0 * mlp_flops_per_sample(self.n_out) * samples
        return {"history": hist, "train_s": train_ms * 1e-3, "data_s": t_data, "steps": steps,
                "batch": n_tiles * TILE_ROWS, "samples": n_train, "scale": self.scale,
                "val_rel_l2": hist[-1]["val_rel_l2"] if hist else None,
                "ms_per_step": train_ms / steps, "samples_per_s": samples / (train_ms * 1e-3),
                "algorithmic_tflops": flops / (train_ms * 1e-3) / 1e12,
                "loss_curve": hist_loss[:: max(1, steps // 200)].cpu().tolist()}

    # -- inference ---------------------------------------------------------------------------------
    def forward_tc(self, u: torch.Tensor) -> torch.Tensor:
        """The network's outputs (n x n_out) by the fused tcgen05 kernel."""
        w = self._weights_struct()
        u = u.contiguous()
        out = torch.empty(u.shape[0], self.n_out, device=self.device)
        if u.shape[0]:
            _check(self.lib.fsg_mlp_tc_forward(ctypes.byref(w), u.data_ptr(), u.shape[0], out.data_ptr(),
                                               self.status.data_ptr(), self._stream()))
        return out

    def tc_status(self) -> int:
        return int(self.status.item())

    @torch.no_grad()
    def predict(self, samples: torch.Tensor, chunk: int = 1 << 21) -> torch.Tensor:
        """Complex transmit pressure at samples (n, 4) [x, z, f, theta] from the network."""
        s = samples.to(device=self.device, dtype=torch.float64).contiguous()
        out = torch.empty(s.shape[0], dtype=torch.complex64, device=self.device)
        for i in range(0, s.shape[0], chunk):
            si = s[i:i + chunk]
            u, _ = self.inputs(si, with_aux=False)
            net = self.forward_tc(u)
            _check(self.lib.fsg_surrogate_combine(self.domain, si.data_ptr(), si.shape[0], net.data_ptr(), self.scale,
                                                  out[i:i + chunk].data_ptr(), self._stream()))
        return out

    def relative_error(self, samples: torch.Tensor, exact: torch.Tensor) -> float:
        pred = self.predict(samples)
        return float(torch.linalg.vector_norm(pred - exact) / torch.linalg.vector_norm(exact))


def simus_with_surrogate(sur: TxFieldSurrogate, scat: np.ndarray, rc: np.ndarray, angles_rad, plan, *,
                         tol: float = 1e-3, tile: int = 64, checks_per_tile: int = 4, exact_reference=True) -> dict:
    """Simus of one phantom for every firing with the transmit field from the network where the
    query lies in its domain, and from the exact kernel elsewhere.  Every (tile of scatterers,
    firing) that used the network is checked by the exact kernel on `checks_per_tile` of its
    scatterers over all frequencies and recomputed exactly where the relative L2 error exceeds
    `tol`.  The receive contraction with that transmit field is the batched receive kernel.
    Returns RF, timings, the fraction of (tile, firing) units that fell back, the share of
    transmit-field queries the network answered, and (exact_reference) the exact batched sweep's
    RF and time for comparison."""
    from fastsimus_gb300.batched import BatchedSimus, BatchTuning
    from fastsimus_gb300.plan import element_positions
    from fastsimus_gb300.tx_delay import plane_wave

    dev = sur.device
    p, m = sur.params, sur.medium
    S = scat.shape[0]
    F = plan.selected_freqs.shape[0]
    T = len(angles_rad)
    f = torch.as_tensor(plan.selected_freqs, dtype=torch.float64, device=dev)
    th = torch.as_tensor(np.asarray(angles_rad, dtype=np.float64), device=dev)
    sc = torch.as_tensor(scat, dtype=torch.float64, device=dev)
    epos, _, _ = element_positions(p.n_elements, p.pitch, p.radius)
    delays = np.stack([plane_wave(epos, float(a), speed_of_sound=m.speed_of_sound) for a in angles_rad])
    n_tiles = (S + tile - 1) // tile
    b = sur.box
    f_in = (f >= b.f[0]) & (f <= b.f[1])
    t_in = th.abs() <= b.max_angle
    pt_in = (sc[:, 0] >= b.x[0]) & (sc[:, 0] <= b.x[1]) & (sc[:, 1] >= b.z[0]) & (sc[:, 1] <= b.z[1])
    pad = torch.ones(n_tiles * tile, dtype=torch.bool, device=dev)
    pad[:S] = pt_in
    tile_in = pad.view(n_tiles, tile).all(dim=1)
    use_net = tile_in[:, None] & t_in[None, :]  # (tile, firing) units the network may answer

    def queries(rows: torch.Tensor, fsel: torch.Tensor, tsel: torch.Tensor) -> torch.Tensor:
        q = torch.empty(rows.shape[0], fsel.shape[0], tsel.shape[0], 4, dtype=torch.float64, device=dev)
        q[..., 0] = sc[rows, 0][:, None, None]
        q[..., 1] = sc[rows, 1][:, None, None]
        q[..., 2] = fsel[None, :, None]
        q[..., 3] = tsel[None, None, :]
        return q.reshape(-1, 4)

    torch.cuda.synchronize(dev)
    t0 = time.perf_counter()
    tx = torch.empty(S, F, T, dtype=torch.complex64, device=dev)
    # network: in-domain tiles x in-band frequencies x in-range firings; everything else exact
    net_rows = torch.nonzero(tile_in.repeat_interleave(tile)[:S]).flatten()
    fi, ti_ = torch.nonzero(f_in).flatten(), torch.nonzero(t_in).flatten()
    n_net = int(net_rows.numel() * fi.numel() * ti_.numel())
    step = max(1, (1 << 22) // max(1, fi.numel() * ti_.numel()))
    for i in range(0, net_rows.numel(), step):
        rows = net_rows[i:i + step]
        val = sur.predict(queries(rows, f[fi], th[ti_])).view(rows.shape[0], fi.numel(), ti_.numel())
        tx[rows[:, None, None], fi[None, :, None], ti_[None, None, :]] = val
    torch.cuda.synchronize(dev)
    t_net = time.perf_counter() - t0
    t0 = time.perf_counter()
    # exact: every query the network does not answer
    mask = torch.zeros(S, F, T, dtype=torch.bool, device=dev)
    mask[net_rows[:, None, None], fi[None, :, None], ti_[None, None, :]] = True
    ex_idx = torch.nonzero(~mask.view(-1)).flatten()
    for i in range(0, ex_idx.numel(), 1 << 22):
        idx = ex_idx[i:i + (1 << 22)]
        s_i, rem = idx // (F * T), idx % (F * T)
        q = torch.stack([sc[s_i, 0], sc[s_i, 1], f[rem // T], th[rem % T]], -1)
        tx.view(-1)[idx] = sur.exact(q)
    torch.cuda.synchronize(dev)
    t_exact_part = time.perf_counter() - t0
    # check every network-answered (tile, firing) on a few members; recompute failing units exactly
    t0 = time.perf_counter()
    units = torch.nonzero(use_net)
    errs = torch.zeros(0, device=dev)
    failed_units = units[:0]
    if units.numel():
        n_u = units.shape[0]
        lo = units[:, 0] * tile
        last = torch.clamp(lo + tile, max=S) - 1
        frac = torch.linspace(0.0, 1.0, checks_per_tile, dtype=torch.float64, device=dev)
        jrows = (lo[:, None] + ((last - lo)[:, None].double() * frac[None, :]).round().long())  # (units, checks)
        q = torch.empty(n_u, checks_per_tile, F, 4, dtype=torch.float64, device=dev)
        q[..., 0] = sc[jrows, 0][..., None]
        q[..., 1] = sc[jrows, 1][..., None]
        q[..., 2] = f[None, None, :]
        q[..., 3] = th[units[:, 1]][:, None, None]
        ex = sur.exact(q.view(-1, 4)).view(n_u, checks_per_tile, F)
        got = tx[jrows, :, units[:, 1][:, None]]  # (units, checks, F)
        errs = torch.linalg.vector_norm((got - ex).reshape(n_u, -1), dim=1) / \
            torch.linalg.vector_norm(ex.reshape(n_u, -1), dim=1)
        failed_units = units[errs > tol]
    n_fail_queries = 0
    for ti, tf in failed_units.tolist():
        lo_, hi_ = ti * tile, min(S, (ti + 1) * tile)
        rows = torch.arange(lo_, hi_, device=dev)
        tx[lo_:hi_, :, tf] = sur.exact(queries(rows, f, th[tf:tf + 1])).view(-1, F)
        n_fail_queries += (hi_ - lo_) * int(fi.numel())
    failed = int(failed_units.shape[0])
    errs = errs.cpu().numpy()
    torch.cuda.synchronize(dev)
    t_check = time.perf_counter() - t0
    # receive contraction with that transmit field
    bs = BatchedSimus([(scat, rc)], delays, p, m, plans=[plan], backend="fp32", tuning=BatchTuning(2, 32768, 1))
    t0 = time.perf_counter()
    _check(sur.lib.fsg_simus_batched_rx(bs.probe, bs.med, bs._ph, bs.delays.data_ptr(), T, tx.data_ptr(),
                                        bs.tuning.to_c(), bs.ws.data_ptr(), bs.ws.numel(), _device.stream_handle(dev)))
    bs._finish()
    torch.cuda.synchronize(dev)
    t_rx = time.perf_counter() - t0
    n_units = n_tiles * T
    fallback_units = n_units - int(use_net.sum()) + failed
    res = {"rf": bs.rfs[0].clone(), "t_network_s": t_net, "t_exact_outside_domain_s": t_exact_part,
           "t_check_fallback_s": t_check, "t_rx_s": t_rx,
           "t_surrogate_total_s": t_net + t_exact_part + t_check + t_rx, "units": n_units,
           "units_in_domain": int(use_net.sum()), "units_failed_check": failed,
           "fallback_fraction": fallback_units / max(1, n_units),
           "network_query_share": (n_net - n_fail_queries) / max(1, S * F * T),
           "unit_rel_err_median": float(np.median(errs)) if errs.size else None,
           "unit_rel_err_max": float(np.max(errs)) if errs.size else None, "queries": S * F * T}
    if exact_reference:
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        bs.run()
        torch.cuda.synchronize(dev)
        res["t_exact_s"] = time.perf_counter() - t0
        res["rf_exact"] = bs.rfs[0].clone()
        d = (res["rf"] - res["rf_exact"]).double()
        res["rf_rel_l2_vs_exact"] = float(torch.linalg.vector_norm(d) / torch.linalg.vector_norm(res["rf_exact"].double()))
        res["gain"] = res["t_exact_s"] / res["t_surrogate_total_s"]
    return res


def cfg5_box(params: TransducerParams) -> Box:
    """The whole training domain of the learned-surrogate configuration: the imaging box
    x in [-10, 10] mm, z in [5, 30] mm, the band fc (1 +- B / 2), steering up to 16 degrees."""
    fc, bw = params.freq_center, params.bandwidth
    return Box(x=(-10e-3, 10e-3), z=(5e-3, 30e-3), f=(fc * (1 - bw / 2), fc * (1 + bw / 2)),
               max_angle=16.0 * math.pi / 180.0)




def main(argv=None):
    """Train the surrogate of the 64-element probe over its training box and print the report:
    ``python -m fastsimus_gb300.surrogate [--steps N] [--n-train M] [--block B] [--seed S]``."""
    import argparse
    import json

    from fastsimus_gb300 import workloads as W

    ap = argparse.ArgumentParser(description=main.__doc__)
    ap.add_argument("--steps", type=int, default=60_000)
    ap.add_argument("--n-train", type=int, default=2_000_000)
    ap.add_argument("--block", type=int, default=1000, help="steps per CUDA-graph replay")
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--predict", type=int, default=0, help="then time inference on this many queries")
    a = ap.parse_args(argv)
    p, m = W.cfg1_probe(), W.cfg1_medium()
    sur = TxFieldSurrogate(p, m, cfg5_box(p), seed=a.seed)
    rep = sur.train(n_train=a.n_train, steps=a.steps, block=a.block, seed=a.seed, evals=1)
    out = {k: v for k, v in rep.items() if k != "loss_curve"}
    if a.predict:
        q = sur.sample_domain(a.predict, seed=a.seed + 9)
        sur.predict(q)
        torch.cuda.synchronize(sur.device)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        sur.predict(q)
        e1.record()
        torch.cuda.synchronize(sur.device)
        out["predict_ns_per_query"] = e0.elapsed_time(e1) * 1e6 / a.predict
    print(json.dumps(out))


if __name__ == "__main__":
    main()
