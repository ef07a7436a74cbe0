"""Tensor-core (tcgen05, BF16 hi/lo three-product) path: the GEMM tile primitive, then the full
multi-transmit sweep against the FP64 oracle and the plain FP32 kernel.  Target relative L2
<= 1e-3 versus FP64; max phase error is reported."""

import ctypes

import numpy as np
import pytest

import oracle.fastsimus_fp64 as O
from tests import _golden as G
from tests._gpu import np64, require_gpu, torch

pytestmark = pytest.mark.gpu

TC_TOL = 1e-3


@pytest.fixture(scope="module", autouse=True)
def _gpu():
    require_gpu()


@pytest.mark.parametrize("a_mn,b_mn", [(0, 0), (1, 1), (0, 1), (1, 0)])
def test_tc_tile_gemm(a_mn, b_mn):
    from fastsimus_gb300 import _native

    lib = _native.load()
    rng = np.random.default_rng(3 + 2 * a_mn + b_mn)
    a = rng.standard_normal((128, 64)).astype(np.float32)
    b = rng.standard_normal((64, 64)).astype(np.float32)
    dev = torch.device("cuda", torch.cuda.current_device())
    ta, tb = torch.as_tensor(a, device=dev), torch.as_tensor(b, device=dev)
    td = torch.full((128, 64), float("nan"), dtype=torch.float32, device=dev)
    st = torch.zeros(1, dtype=torch.int32, device=dev)
    _native.check(lib.fsg_tc_selftest(ta.data_ptr(), tb.data_ptr(), td.data_ptr(), a_mn, b_mn, st.data_ptr(),
                                      torch.cuda.current_stream(dev).cuda_stream))
    torch.cuda.synchronize()
    assert int(st.item()) == 0
    d = td.cpu().numpy().astype(np.float64)
    ref = a.astype(np.float64) @ b.astype(np.float64).T
    err = G.rel_l2(d, ref)
    print(f"tile a_mn={a_mn} b_mn={b_mn}: relL2 {err:.3e}")
    assert err < 1e-4


def test_tc_sweep_vs_oracle_small():
    from fastsimus_gb300 import workloads as W
    from fastsimus_gb300.batched import BatchedSimus, BatchTuning

    p, m = W.cfg1_probe(), W.cfg1_medium()
    rng = np.random.default_rng(21)
    phantoms = [(W.uniform_box(rng, 150, (-10e-3, 10e-3), (5e-3, 30e-3)), rng.standard_normal(150)),
                (W.uniform_box(rng, 90, (-5e-3, 5e-3), (8e-3, 20e-3)), rng.standard_normal(90))]
    delays = W.plane_wave_delays(p, m, [-12.0, -4.0, 0.0, 6.0, 12.0])
    b = BatchedSimus(phantoms, delays, p, m, backend="tc", tuning=BatchTuning(6, 64, 1))
    res = b.run()
    assert b.device_status() == 0
    worst = 0.0
    for (s, r), plan, out in zip(phantoms, b.plans, res):
        rf = np64(out.rf)
        spec = np64(out.spectrum)
        for t in range(delays.shape[0]):
            ref = O.simus_compute(s, r, delays[t], plan, p, m)
            err = G.rel_l2(rf[:, :, t], ref.rf)
            i0 = plan.freq_idx_start
            sel = slice(i0, i0 + plan.selected_freqs.shape[0])
            ph = G.max_phase_err(spec[sel, :, t], ref.spectrum[sel])
            worst = max(worst, err)
            assert err < TC_TOL, (t, err, ph)
    print(f"tc vs oracle worst relL2 {worst:.3e}")


def test_tc_vs_plain_at_scale_and_graph():
    import fastsimus_gb300 as F
    from fastsimus_gb300 import workloads as W
    from fastsimus_gb300.batched import BatchedSimus

    p, m = W.cfg1_probe(), W.cfg1_medium()
    s, r = W.cfg4_scatterers(20_000, seed=7)
    delays = W.plane_wave_delays(p, m, np.linspace(-12.0, 12.0, 31))
    b = BatchedSimus([(s, r)], delays, p, m, backend="tc")
    spec = np64(b.run()[0].spectrum)
    assert b.device_status() == 0
    for t in (0, 15, 30):
        ref = np64(F.simus_compute(s, r, delays[t], b.plans[0], p, m).spectrum)
        err = G.rel_l2(spec[:, :, t], ref)
        print(f"tc vs plain firing {t}: relL2 {err:.3e}")
        assert err < TC_TOL
    b.capture()
    rep = np64(b.replay()[0].spectrum)
    np.testing.assert_array_equal(rep, spec)


@pytest.mark.parametrize("n_tx", [40, 75])
def test_tc_more_than_32_transmits_vs_plain(n_tx):
    """40 and 75 firings: accumulators of 2 and 3 column chunks of 32 transmits (N = 128 and
    192), with 3 and 1 band frequencies per item."""
    import fastsimus_gb300 as F
    from fastsimus_gb300 import workloads as W
    from fastsimus_gb300.batched import BatchedSimus

    p, m = W.cfg1_probe(), W.cfg1_medium()
    rng = np.random.default_rng(n_tx)
    phantoms = [(W.uniform_box(rng, 700, (-10e-3, 10e-3), (5e-3, 30e-3)), rng.standard_normal(700)),
                (W.uniform_box(rng, 130, (-6e-3, 6e-3), (6e-3, 20e-3)), rng.standard_normal(130))]
    delays = W.plane_wave_delays(p, m, np.linspace(-16.0, 16.0, n_tx))
    b = BatchedSimus(phantoms, delays, p, m, backend="tc")
    res = b.run()
    assert b.device_status() == 0
    for (s, r), plan, out in zip(phantoms, b.plans, res):
        spec = np64(out.spectrum)
        for t in (0, n_tx // 3, n_tx // 2 + 1, n_tx - 1):
            ref = np64(F.simus_compute(s, r, delays[t], plan, p, m).spectrum)
            err = G.rel_l2(spec[:, :, t], ref)
            assert err < TC_TOL, (t, err)


def test_tc_rejects_too_many_transmits():
    from fastsimus_gb300 import workloads as W
    from fastsimus_gb300.batched import BatchedSimus

    p, m = W.cfg1_probe(), W.cfg1_medium()
    s, r = W.cfg1_scatterers(100)
    with pytest.raises(NotImplementedError):
        BatchedSimus([(s, r)], W.plane_wave_delays(p, m, np.linspace(-10, 10, 97)), p, m, backend="tc").run()


@pytest.mark.parametrize("name", ["simus_small_rigid", "simus_small_impedance", "simus_small_nan_apod",
                                  "simus_p4_focused", "simus_cfg1_full"])
def test_tc_matches_reference_goldens(name):
    """Single-firing reference fixtures of up to 64 elements through the tensor-core sweep:
    rigid and impedance baffles, NaN delays with apodisation, a focused phased-array firing."""
    import fastsimus_gb300 as F
    from fastsimus_gb300.batched import BatchedSimus

    g = G.load(name)
    assert not g.ffd and g.params.n_elements <= 64
    plan = F.simus_precompute(g.scatterers, g.rc, g.delays, g.params, g.medium, fs=g.fs,
                              element_splitting=g.element_splitting)
    b = BatchedSimus([(g.scatterers, g.rc)], g.delays[None], g.params, g.medium, plans=[plan],
                     tx_apodization=g.apod, backend="tc")
    rf = np64(b.run()[0].rf)[:, :, 0]
    assert b.device_status() == 0
    err = G.rel_l2(rf, g.rf)
    print(f"tc {name}: relL2 {err:.3e}")
    assert err < TC_TOL


@pytest.mark.parametrize("baffle", ["soft", "rigid", 1.75])
def test_tc_convex_array_vs_oracle(baffle):
    """A 64-element convex array (the C5-2v's pitch, width and radius) with soft, rigid and
    impedance baffles, three firings and two phantoms, against the FP64 oracle; scatterers
    behind the array or inside its circle contribute nothing."""
    import dataclasses

    from fastsimus_gb300 import workloads as W
    from fastsimus_gb300.batched import BatchedSimus, BatchTuning

    c5 = G.load("simus_c5_convex").params
    p = dataclasses.replace(c5, n_elements=64, baffle=baffle)
    m = W.cfg1_medium()
    rng = np.random.default_rng(3)
    phantoms = [(W.uniform_box(rng, n, (-15e-3, 15e-3), (-4e-3, 45e-3)), rng.standard_normal(n)) for n in (140, 70)]
    delays = W.plane_wave_delays(p, m, [-10.0, 0.0, 8.0])
    b = BatchedSimus(phantoms, delays, p, m, backend="tc", tuning=BatchTuning(5, 64, 1))
    res = b.run()
    assert b.device_status() == 0
    for (s, r), plan, out in zip(phantoms, b.plans, res):
        rf = np64(out.rf)
        for t in range(delays.shape[0]):
            ref = O.simus_compute(s, r, delays[t], plan, p, m)
            err = G.rel_l2(rf[:, :, t], ref.rf)
            assert err < TC_TOL, (t, err)
