"""Learned transmit-field surrogate with the exact transmit kernel as judge and fallback.

The network maps (x, z, f, theta) -- a point, a frequency and a plane-wave steering angle --
to the complex transmit pressure of the array (the pressure inside the pfield step body,
_pfield_strategies.py:48, before |.|^2).  Architecture: 64 random Fourier features of the
normalised inputs, 4 hidden layers of width 256 with SiLU, a linear (Re, Im) head; BF16
weights, FP32 accumulation.  Training, inference and the gradients all run in libfsgb300's own
kernels (``fsg_mlp_gemm`` with fused bias/SiLU epilogues, ``fsg_mlp_features``,
``fsg_mlp_colsum``, ``fsg_mlp_adam``); PyTorch only holds the buffers.

The raw field oscillates at the wavelength in space and at 1/delay in frequency, so the
network learns the envelope  p * exp(-i phi_c),  phi_c = 2 pi f / c (x sin theta + z cos theta
- min_e x_e sin theta), the phase of the ideal plane wave; ``predict`` multiplies it back.

In simus the network supplies the transmit field at every (scatterer, frequency, firing); the
exact kernel ``fsg_txfield`` judges each tile of scatterers on a few of its members and any tile
whose relative L2 error exceeds the tolerance is recomputed exactly.  ``simus_with_surrogate``
returns the timings that show what the network gains (or loses) against the exact path.
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
from fastsimus_gb300.plan import element_positions

HIDDEN = 256
DEPTH = 4
N_FOURIER = 64


@dataclass
class Box:
    """Domain of the surrogate: x, z ranges (m), band (Hz), max steering angle (rad)."""

    x: tuple
    z: tuple
    f: tuple
    max_angle: float


def _check(st):
    _native.check(st)


class TxFieldSurrogate:
    def __init__(self, params: TransducerParams, medium: MediumParams, box: Box, *, sigma=(6.0, 6.0, 3.0, 3.0),
                 seed: int = 0, device: torch.device | None = None, tx_n_wavelengths: float = 1.0):
        if not params.is_linear:
            raise NotImplementedError("the transmit-field surrogate supports linear arrays")
        self.params, self.medium, self.box = params, medium, box
        self.device = device or _device.require_cuda()
        self.lib = _native.load()
        self.tx_n_wavelengths = tx_n_wavelengths
        g = torch.Generator().manual_seed(seed)
        sig = torch.tensor(sigma, dtype=torch.float32)
        self.bmat = (torch.randn(N_FOURIER, 4, generator=g) * sig).to(self.device).contiguous()
        shapes = [(HIDDEN, 2 * N_FOURIER)] + [(HIDDEN, HIDDEN)] * (DEPTH - 1) + [(2, HIDDEN)]
        self.W, self.b = [], []
        for fan_out, fan_in in shapes:
            w = torch.randn(fan_out, fan_in, generator=g) * math.sqrt(2.0 / fan_in)
            self.W.append(w.to(self.device).contiguous())
            self.b.append(torch.zeros(fan_out, device=self.device))
        self.Wb = [w.to(torch.bfloat16).contiguous() for w in self.W]
        self.m = [torch.zeros_like(p) for p in self.W + self.b]
        self.v = [torch.zeros_like(p) for p in self.W + self.b]
        self.step = 0
        self.scale = 1.0
        epos, _, _ = element_positions(params.n_elements, params.pitch, params.radius)
        self.elem_x = torch.as_tensor(epos[:, 0], dtype=torch.float64, device=self.device)
        self.probe = _native.make_probe(params, self._n_sub())
        self.med = _native.make_medium(medium)
        self.ws = _device.workspace(params.n_elements * self._n_sub() * 16 + params.n_elements * 8 + 1024,
                                    self.device)

    def _n_sub(self):
        lam_min = self.medium.speed_of_sound / (self.params.freq_center * (1.0 + self.params.bandwidth / 2.0))
        return math.ceil(self.params.element_width / lam_min)

    def _stream(self):
        return _device.stream_handle(self.device)

    # -- exact field, carrier, normalisation -------------------------------------------------
    def exact(self, samples: torch.Tensor) -> torch.Tensor:
        """Exact complex transmit pressure at samples (n, 4) float64 [x, z, f, theta]."""
        s = samples.to(device=self.device, dtype=torch.float64).contiguous()
        out = torch.empty(s.shape[0], dtype=torch.complex64, device=self.device)
        _check(self.lib.fsg_txfield(self.probe, self.med, self.tx_n_wavelengths, self.params.bandwidth, s.data_ptr(),
                                    s.shape[0], out.data_ptr(), self.ws.data_ptr(), self.ws.numel(), self._stream()))
        return out

    def carrier(self, samples: torch.Tensor) -> torch.Tensor:
        x, z, f, th = samples.unbind(-1)
        st = torch.sin(th)
        xmin = torch.minimum(self.elem_x.min() * st, self.elem_x.max() * st)
        cyc = f / self.medium.speed_of_sound * (x * st + z * torch.cos(th) - xmin)
        cyc = cyc - torch.round(cyc)
        ph = (2 * math.pi) * cyc
        return torch.polar(torch.ones_like(ph), ph).to(torch.complex64)

    def normalise(self, samples: torch.Tensor) -> torch.Tensor:
        b = self.box
        x, z, f, th = samples.unbind(-1)
        u = torch.stack([(2 * x - (b.x[0] + b.x[1])) / (b.x[1] - b.x[0]),
                         (2 * z - (b.z[0] + b.z[1])) / (b.z[1] - b.z[0]),
                         (2 * f - (b.f[0] + b.f[1])) / (b.f[1] - b.f[0]),
                         th / b.max_angle], dim=-1)
        return u.to(torch.float32).contiguous()

    def sample_domain(self, n: int, seed: int) -> torch.Tensor:
        g = torch.Generator(device="cpu").manual_seed(seed)
        b = self.box
        r = torch.rand(n, 4, generator=g, dtype=torch.float64)
        lo = torch.tensor([b.x[0], b.z[0], b.f[0], -b.max_angle], dtype=torch.float64)
        hi = torch.tensor([b.x[1], b.z[1], b.f[1], b.max_angle], dtype=torch.float64)
        return (lo + r * (hi - lo)).to(self.device)

    # -- network ------------------------------------------------------------------------------
    def _gemm(self, A, a_sm, a_sk, B, b_sk, b_sn, b_bf16, bias, Zs, C, C2, ldc, M, N, K, epi, acc=0):
        _check(self.lib.fsg_mlp_gemm(A.data_ptr(), a_sm, a_sk, B.data_ptr(), b_sk, b_sn, b_bf16,
                                     bias.data_ptr() if bias is not None else None,
                                     Zs.data_ptr() if Zs is not None else None, C.data_ptr(),
                                     C2.data_ptr() if C2 is not None else None, ldc, M, N, K, epi, acc,
                                     self._stream()))

    def forward(self, u: torch.Tensor, keep: bool = False):
        n = u.shape[0]
        feat = torch.empty(n, 2 * N_FOURIER, device=self.device)
        _check(self.lib.fsg_mlp_features(u.data_ptr(), self.bmat.data_ptr(), feat.data_ptr(), n, self._stream()))
        acts, zs = [feat], []
        x, k = feat, 2 * N_FOURIER
        for layer in range(DEPTH):
            z = torch.empty(n, HIDDEN, device=self.device)
            a = torch.empty(n, HIDDEN, device=self.device)
            self._gemm(x, k, 1, self.Wb[layer], 1, k, 1, self.b[layer], None, z, a, HIDDEN, n, HIDDEN, k, 1)
            zs.append(z)
            acts.append(a)
            x, k = a, HIDDEN
            if not keep:
                acts[-2] = None
        out = torch.empty(n, 2, device=self.device)
        self._gemm(x, HIDDEN, 1, self.Wb[DEPTH], 1, HIDDEN, 1, self.b[DEPTH], None, out, None, 2, n, 2, HIDDEN, 0)
        return out, (acts, zs)

    # -- tensor-core inference ------------------------------------------------------------------
    def _tc_weights(self):
        """Packed BF16 hidden-layer weights for ``fsg_mlp_tc_forward``; re-packed after every
        optimiser step."""
        if getattr(self, "_tc_step", None) != self.step:
            lib, stream = self.lib, self._stream()
            self._tc_packed = []
            for layer in range(DEPTH):
                k = self.Wb[layer].shape[1]
                buf = torch.empty(lib.fsg_mlp_tc_packed_bytes(k) // 2, dtype=torch.bfloat16, device=self.device)
                _check(lib.fsg_mlp_tc_pack(self.Wb[layer].data_ptr(), HIDDEN, k, buf.data_ptr(), stream))
                self._tc_packed.append(buf)
            self._tc_head = self.Wb[DEPTH].float().contiguous()  # the head multiplies the same BF16 values
            w = _native.FsgMlpWeights()
            for layer in range(DEPTH):
                w.packed[layer] = self._tc_packed[layer].data_ptr()
                w.bias[layer] = self.b[layer].data_ptr()
            w.w_head = self._tc_head.data_ptr()
            w.b_head = self.b[DEPTH].data_ptr()
            w.bmat = self.bmat.data_ptr()
            self._tc_struct = w
            self._tc_status = torch.zeros(1, dtype=torch.int32, device=self.device)
            self._tc_step = self.step
        return self._tc_struct

    def forward_tc(self, u: torch.Tensor) -> torch.Tensor:
        """The network's output (n x 2) by the fused tcgen05 kernel (inference only)."""
        w = self._tc_weights()
        u = u.contiguous()
        out = torch.empty(u.shape[0], 2, device=self.device)
        _check(self.lib.fsg_mlp_tc_forward(ctypes.byref(w), u.data_ptr(), u.shape[0], out.data_ptr(),
                                           self._tc_status.data_ptr(), self._stream()))
        return out

    def tc_status(self) -> int:
        return int(self._tc_status.item()) if hasattr(self, "_tc_status") else 0

    def backward(self, cache, dout: torch.Tensor):
        acts, zs = cache
        n = dout.shape[0]
        gW = [None] * (DEPTH + 1)
        gb = [None] * (DEPTH + 1)
        # head
        gW[DEPTH] = torch.empty(2, HIDDEN, device=self.device)
        self._gemm(dout, 1, 2, acts[DEPTH], HIDDEN, 1, 0, None, None, gW[DEPTH], None, HIDDEN, 2, HIDDEN, n, 0)
        gb[DEPTH] = torch.empty(2, device=self.device)
        _check(self.lib.fsg_mlp_colsum(dout.data_ptr(), n, 2, gb[DEPTH].data_ptr(), 0, self._stream()))
        dz = torch.empty(n, HIDDEN, device=self.device)
        self._gemm(dout, 2, 1, self.Wb[DEPTH], HIDDEN, 1, 1, None, zs[DEPTH - 1], dz, None, HIDDEN, n, HIDDEN, 2, 2)
        for layer in range(DEPTH - 1, -1, -1):
            a_prev = acts[layer]
            k = a_prev.shape[1]
            gW[layer] = torch.empty(HIDDEN, k, device=self.device)
            self._gemm(dz, 1, HIDDEN, a_prev, k, 1, 0, None, None, gW[layer], None, k, HIDDEN, k, n, 0)
            gb[layer] = torch.empty(HIDDEN, device=self.device)
            _check(self.lib.fsg_mlp_colsum(dz.data_ptr(), n, HIDDEN, gb[layer].data_ptr(), 0, self._stream()))
            if layer > 0:
                dz_prev = torch.empty(n, HIDDEN, device=self.device)
                self._gemm(dz, HIDDEN, 1, self.Wb[layer], HIDDEN, 1, 1, None, zs[layer - 1], dz_prev, None, HIDDEN,
                           n, HIDDEN, HIDDEN, 2)
                dz = dz_prev
        return gW, gb

    def loss_and_grads(self, u: torch.Tensor, y: torch.Tensor):
        out, cache = self.forward(u, keep=True)
        diff = out - y
        loss = float((diff * diff).sum()) / (2 * u.shape[0])
        gW, gb = self.backward(cache, (diff / u.shape[0]).contiguous())
        return loss, gW, gb

    def adam(self, gW, gb, lr: float, b1=0.9, b2=0.999, eps=1e-8):
        self.step += 1
        params = self.W + self.b
        grads = gW + gb
        for i, (p, g) in enumerate(zip(params, grads)):
            wb = self.Wb[i] if i < len(self.W) else None
            _check(self.lib.fsg_mlp_adam(p.data_ptr(), wb.data_ptr() if wb is not None else None, g.data_ptr(),
                                         self.m[i].data_ptr(), self.v[i].data_ptr(), p.numel(), lr, b1, b2, eps,
                                         self.step, 1.0, self._stream()))

    # -- training / inference -----------------------------------------------------------------
    def make_dataset(self, n: int, seed: int):
        s = self.sample_domain(n, seed)
        p = self.exact(s)
        env = p * torch.conj(self.carrier(s))
        return s, env

    def train(self, n_train: int = 2_000_000, epochs: int = 20, batch: int = 4096, lr: float = 2e-3,
              n_val: int = 65536, seed: int = 0, log=None) -> dict:
        t0 = time.perf_counter()
        s, env = self.make_dataset(n_train, seed)
        sv, envv = self.make_dataset(n_val, seed + 1)
        self.scale = float(torch.sqrt((env.abs() ** 2).mean()))
        u = self.normalise(s)
        y = (torch.view_as_real(env) / self.scale).to(torch.float32).contiguous()
        t_data = time.perf_counter() - t0
        steps_per_epoch = n_train // batch
        total = epochs * steps_per_epoch
        hist = []
        torch.cuda.synchronize(self.device)
        t1 = time.perf_counter()
        g = torch.Generator(device=self.device).manual_seed(seed)
        it = 0
        for ep in range(epochs):
            perm = torch.randperm(n_train, device=self.device, generator=g)
            ep_loss = 0.0
            for b in range(steps_per_epoch):
                idx = perm[b * batch:(b + 1) * batch]
                rate = lr * 0.5 * (1.0 + math.cos(math.pi * it / total))
                loss, gW, gb = self.loss_and_grads(u[idx].contiguous(), y[idx].contiguous())
                self.adam(gW, gb, rate)
                ep_loss += loss
                it += 1
            val = self.relative_error(sv, envv * self.carrier(sv))
            hist.append({"epoch": ep, "train_mse": ep_loss / steps_per_epoch, "val_rel_l2": val})
            if log:
                log(hist[-1])
        torch.cuda.synchronize(self.device)
        return {"history": hist, "train_s": time.perf_counter() - t1, "data_s": t_data, "steps": it,
                "samples": n_train, "scale": self.scale}

    @torch.no_grad()
    def predict(self, samples: torch.Tensor, chunk: int = 1 << 20, backend: str = "tc") -> torch.Tensor:
        """Complex transmit pressure at samples (n, 4) [x, z, f, theta].  ``backend="tc"`` runs
        the fused tensor-core forward pass, ``"simt"`` the training kernels' forward pass."""
        out = torch.empty(samples.shape[0], dtype=torch.complex64, device=self.device)
        for i in range(0, samples.shape[0], chunk):
            s = samples[i:i + chunk]
            u = self.normalise(s)
            o = self.forward_tc(u) if backend == "tc" else self.forward(u)[0]
            out[i:i + chunk] = torch.view_as_complex(o.contiguous()) * self.scale * self.carrier(s)
        return out

    def relative_error(self, samples: torch.Tensor, exact: torch.Tensor) -> float:
        pred = self.predict(samples)
        return float(torch.linalg.vector_norm(pred - exact) / torch.linalg.vector_norm(exact))


def simus_with_surrogate(sur: TxFieldSurrogate, scat: np.ndarray, rc: np.ndarray, angles_rad, plan, *,
                         tol: float = 1e-3, tile: int = 64, judges_per_tile: int = 4, exact_reference=True) -> dict:
    """Simus of one phantom for every firing with the transmit field from the network, each
    scatterer tile judged by the exact kernel on `judges_per_tile` of its scatterers and
    recomputed exactly where the relative L2 error exceeds `tol`.  Returns RF, timings and the
    fallback fraction, plus the exact batched sweep's RF and time for comparison."""
    from fastsimus_gb300.batched import BatchedSimus, BatchTuning
    from fastsimus_gb300.tx_delay import plane_wave

    dev = sur.device
    p, m = sur.params, sur.medium
    S = scat.shape[0]
    F = plan.selected_freqs.shape[0]
    T = len(angles_rad)
    f = torch.as_tensor(plan.selected_freqs, dtype=torch.float64, device=dev)
    th = torch.as_tensor(np.asarray(angles_rad, dtype=np.float64), device=dev)
    sc = torch.as_tensor(scat, dtype=torch.float64, device=dev)
    epos, _, apex = element_positions(p.n_elements, p.pitch, p.radius)
    delays = np.stack([plane_wave(epos, float(a), speed_of_sound=m.speed_of_sound) for a in angles_rad])

    def queries(rows: torch.Tensor) -> torch.Tensor:  # (len(rows) * F * T, 4) in [s][f][t] order
        n = rows.shape[0]
        q = torch.empty(n, F, T, 4, dtype=torch.float64, device=dev)
        q[..., 0] = sc[rows, 0][:, None, None]
        q[..., 1] = sc[rows, 1][:, None, None]
        q[..., 2] = f[None, :, None]
        q[..., 3] = th[None, None, :]
        return q.reshape(-1, 4)

    torch.cuda.synchronize(dev)
    t0 = time.perf_counter()
    tx = torch.empty(S * F * T, dtype=torch.complex64, device=dev)
    step = max(1, (1 << 22) // (F * T))
    for i in range(0, S, step):
        rows = torch.arange(i, min(S, i + step), device=dev)
        tx[i * F * T:(i + rows.shape[0]) * F * T] = sur.predict(queries(rows))
    torch.cuda.synchronize(dev)
    t_net = time.perf_counter() - t0
    # judge every tile on a few members; recompute failing tiles exactly
    t0 = time.perf_counter()
    n_tiles = (S + tile - 1) // tile
    failed = []
    errs = []
    txv = tx.view(S, F, T)
    for ti in range(n_tiles):
        lo, hi = ti * tile, min(S, (ti + 1) * tile)
        judges = torch.linspace(lo, hi - 1, min(judges_per_tile, hi - lo), device=dev).round().long()
        ex = sur.exact(queries(judges)).view(-1, F, T)
        err = float(torch.linalg.vector_norm(txv[judges] - ex) / torch.linalg.vector_norm(ex))
        errs.append(err)
        if err > tol:
            failed.append(ti)
            rows = torch.arange(lo, hi, device=dev)
            txv[lo:hi] = sur.exact(queries(rows)).view(-1, F, T)
    torch.cuda.synchronize(dev)
    t_judge = time.perf_counter() - t0
    # receive contraction with the (network or exact) transmit field
    b = BatchedSimus([(scat, rc)], delays, p, m, plans=[plan], backend="fp32", tuning=BatchTuning(2, 32768, 1))
    lib = sur.lib
    t0 = time.perf_counter()
    _check(lib.fsg_simus_batched_rx(b.probe, b.med, b._ph, b.delays.data_ptr(), T, tx.data_ptr(),
                                    b.tuning.to_c(), b.ws.data_ptr(), b.ws.numel(), _device.stream_handle(dev)))
    b._finish()
    torch.cuda.synchronize(dev)
    t_rx = time.perf_counter() - t0
    res = {"rf": b.rfs[0].clone(), "t_network_s": t_net, "t_judge_fallback_s": t_judge, "t_rx_s": t_rx,
           "t_surrogate_total_s": t_net + t_judge + t_rx, "tiles": n_tiles, "tiles_fallback": len(failed),
           "fallback_fraction": len(failed) / max(1, n_tiles), "tile_rel_err_median": float(np.median(errs)),
           "queries": S * F * T}
    if exact_reference:
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        b.run()
        torch.cuda.synchronize(dev)
        res["t_exact_s"] = time.perf_counter() - t0
        res["rf_exact"] = b.rfs[0].clone()
        d = (res["rf"] - res["rf_exact"]).double()
        res["rf_rel_l2_vs_exact"] = float(torch.linalg.vector_norm(d) / torch.linalg.vector_norm(res["rf_exact"].double()))
        res["gain"] = res["t_exact_s"] / res["t_surrogate_total_s"]
    return res


def cfg5_box(params: TransducerParams) -> Box:
    fc, bw = params.freq_center, params.bandwidth
    return Box(x=(-10e-3, 10e-3), z=(5e-3, 30e-3), f=(fc * (1 - bw / 2), fc * (1 + bw / 2)),
               max_angle=16.0 * math.pi / 180.0)

