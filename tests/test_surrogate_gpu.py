"""Transmit-field surrogate: the exact field kernel against the FP64 oracle, the network's
hand-written forward/backward kernels against an FP64 gradient oracle, training, and the
simus experiment with exact fallback (which reports the measured gain, positive or not)."""

import math

import numpy as np
import pytest

import oracle.fastsimus_fp64 as O
import oracle.mlp_fp64 as M
from tests import _golden as G
from tests._gpu import np64, require_gpu, torch

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _gpu():
    require_gpu()


def _surrogate(seed=0):
    from fastsimus_gb300 import workloads as W
    from fastsimus_gb300.surrogate import TxFieldSurrogate, cfg5_box

    p, m = W.cfg1_probe(), W.cfg1_medium()
    return TxFieldSurrogate(p, m, cfg5_box(p), seed=seed)


def test_exact_txfield_matches_oracle():
    from fastsimus_gb300 import workloads as W

    sur = _surrogate()
    s = sur.sample_domain(300, seed=3)
    got = np64(sur.exact(s))
    ref = O.tx_field_samples(s.cpu().numpy(), W.cfg1_probe(), W.cfg1_medium())
    err = G.rel_l2(got, ref)
    print(f"txfield relL2 {err:.3e}")
    assert err < 1e-5


def test_txfield_equals_pfield_pressure_on_plan_grid():
    """At a plan frequency and 0 degrees the sample field equals the pfield pressure p_k."""
    from fastsimus_gb300 import workloads as W
    from fastsimus_gb300.plan import pfield_precompute

    p, m = W.cfg1_probe(), W.cfg1_medium()
    sur = _surrogate()
    pts = np.array([[0.0, 0.012], [0.004, 0.02], [-0.006, 0.028]])
    plan = pfield_precompute(pts, np.zeros(64), p, m)
    ref = O.tx_field(pts, np.zeros(64), plan, p, m)  # (points, F)
    k = [0, plan.selected_freqs.shape[0] // 2]
    samples = np.array([[x, z, plan.selected_freqs[0] + kk * (plan.selected_freqs[1] - plan.selected_freqs[0]), 0.0]
                        for kk in k for x, z in pts])
    got = np64(sur.exact(torch.as_tensor(samples))).reshape(len(k), len(pts)).T
    assert G.rel_l2(got, ref[:, k]) < 1e-5


def test_network_gradients_match_fp64_oracle():
    sur = _surrogate(seed=4)
    n = 96
    s = sur.sample_domain(n, seed=5)
    u = sur.normalise(s)
    y = torch.randn(n, 2, device=sur.device, generator=torch.Generator(device=sur.device).manual_seed(1))
    loss, gW, gb = sur.loss_and_grads(u, y)
    Wd = [w.to(torch.bfloat16).double().cpu().numpy() for w in sur.W]  # kernels read BF16 weights
    bd = [b.double().cpu().numpy() for b in sur.b]
    l2, rW, rb = M.loss_and_grads(u.double().cpu().numpy(), y.double().cpu().numpy(),
                                  sur.bmat.double().cpu().numpy(), Wd, bd)
    assert abs(loss - l2) / l2 < 1e-4
    for a, r in zip(gW + gb, rW + rb):
        assert G.rel_l2(a.double().cpu().numpy(), r) < 1e-4


def test_tc_forward_matches_training_forward():
    """The fused tcgen05 inference kernel (BF16 weights, hi + lo BF16 activations, FP32
    accumulation in TMEM) against the training kernels' FP32-activation forward pass."""
    sur = _surrogate(seed=6)
    for n in (1000, 128, 1):  # ragged last tile, exactly one tile, a single query
        s = sur.sample_domain(n, seed=9 + n)
        u = sur.normalise(s)
        ref, _ = sur.forward(u)
        got = sur.forward_tc(u)
        torch.cuda.synchronize()
        assert sur.tc_status() == 0
        err = G.rel_l2(got.double().cpu().numpy(), ref.double().cpu().numpy())
        print(f"tc forward n={n}: relL2 vs training forward {err:.2e}")
        assert err < 1e-4
    # after an optimiser step the packed weights follow the new values
    y = torch.zeros(256, 2, device=sur.device)
    u = sur.normalise(sur.sample_domain(256, seed=3))
    _, gW, gb = sur.loss_and_grads(u, y)
    sur.adam(gW, gb, 1e-2)
    ref, _ = sur.forward(u)
    got = sur.forward_tc(u)
    assert G.rel_l2(got.double().cpu().numpy(), ref.double().cpu().numpy()) < 1e-4


def test_training_reduces_error():
    sur = _surrogate(seed=1)
    rep = sur.train(n_train=40960, epochs=4, batch=2048, lr=3e-3, n_val=4096)
    h = rep["history"]
    assert h[-1]["train_mse"] < h[0]["train_mse"]
    assert h[-1]["val_rel_l2"] < 1.0


def test_simus_with_surrogate_fallback_is_exact():
    """With the 1e-3 tolerance every tile the network cannot meet is recomputed by the exact
    kernel; the RF then matches the exact batched sweep at FP32 level.  The timing fields are
    the honest gain measurement."""
    from fastsimus_gb300 import workloads as W
    from fastsimus_gb300.batched import shared_plan
    from fastsimus_gb300.surrogate import simus_with_surrogate

    p, m = W.cfg1_probe(), W.cfg1_medium()
    sur = _surrogate(seed=2)
    sur.train(n_train=20480, epochs=2, batch=2048, n_val=2048)
    s, r = W.cfg1_scatterers(192, seed=8)
    angles = np.deg2rad([-10.0, 0.0, 10.0])
    delays = W.plane_wave_delays(p, m, np.rad2deg(angles))
    plan = shared_plan(s, r, list(delays), p, m)
    res = simus_with_surrogate(sur, s, r, angles, plan, tol=1e-3)
    print({k: v for k, v in res.items() if not k.startswith("rf")})
    if res["fallback_fraction"] == 1.0:
        assert res["rf_rel_l2_vs_exact"] < 1e-5
    loose = simus_with_surrogate(sur, s, r, angles, plan, tol=math.inf)
    assert loose["fallback_fraction"] == 0.0
    assert np.isfinite(loose["rf_rel_l2_vs_exact"])
