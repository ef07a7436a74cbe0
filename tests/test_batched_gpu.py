"""GPU parity of the batched multi-transmit / multi-phantom sweep (fsg_simus_batched)."""

import numpy as np
import pytest

import oracle.fastsimus_fp64 as O
from tests import _golden as G
from tests._gpu import np64, require_gpu, torch

pytestmark = pytest.mark.gpu

PLAIN_TOL = 1e-5


@pytest.fixture(scope="module", autouse=True)
def _gpu():
    require_gpu()


def test_batched_matches_reference_multi_firing_golden():
    from fastsimus_gb300.batched import BatchedSimus

    g = G.load("simus_multi3_cfg1")
    b = BatchedSimus([(g.scatterers, g.rc)], g.delays, g.params, g.medium)
    np.testing.assert_array_equal(b.plans[0].selected_freqs, g.plan_selected_freqs)
    rf = np64(b.run()[0].rf)
    assert rf.shape == g.rf.shape
    err = G.rel_l2(rf, g.rf)
    print(f"batched multi3 relL2 {err:.3e}")
    assert err < PLAIN_TOL


@pytest.mark.parametrize("fb", [1, 2])
def test_batched_many_phantoms_vs_oracle(fb):
    from fastsimus_gb300 import workloads as W
    from fastsimus_gb300.batched import BatchedSimus, BatchTuning

    p, m = W.cfg1_probe(), W.cfg1_medium()
    rng = np.random.default_rng(11)
    phantoms = []
    for n, box in ((150, ((-10e-3, 10e-3), (5e-3, 30e-3))), (70, ((-4e-3, 4e-3), (4e-3, 12e-3))),
                   (230, ((-8e-3, 6e-3), (10e-3, 35e-3)))):
        s = W.uniform_box(rng, n, *box)
        phantoms.append((s, rng.standard_normal(n)))
    delays = W.plane_wave_delays(p, m, [-10.0, -3.0, 0.0, 4.0, 12.0])
    delays[2, 5] = np.nan
    apod = np.hanning(64) + 0.2
    b = BatchedSimus(phantoms, delays, p, m, tx_apodization=apod, tuning=BatchTuning(fb, 64, 1))
    res = b.run()
    for (s, r), plan, out in zip(phantoms, b.plans, res):
        rf = np64(out.rf)
        for t in range(delays.shape[0]):
            ref = O.simus_compute(s, r, delays[t], plan, p, m, tx_apodization=apod)
            err = G.rel_l2(rf[:, :, t], ref.rf)
            assert err < PLAIN_TOL, (t, err)


def test_graph_replay_equals_eager_and_autotune():
    from fastsimus_gb300 import workloads as W
    from fastsimus_gb300.batched import BatchedSimus, BatchTuning

    p, m = W.cfg1_probe(), W.cfg1_medium()
    phantoms = [W.cfg1_scatterers(3000, seed=s) for s in (1, 2)]
    delays = W.plane_wave_delays(p, m, np.linspace(-16, 16, 9))
    b = BatchedSimus(phantoms, delays, p, m, tuning=BatchTuning(2, 1024, 1))
    eager = [np64(r.rf) for r in b.run()]
    b.capture()
    rep = [np64(r.rf) for r in b.replay()]
    for a, c in zip(eager, rep):
        np.testing.assert_array_equal(a, c)
    best = b.autotune(candidates=[BatchTuning(1, 1024, 1), BatchTuning(2, 2048, 1)], cache=False)
    assert best in (BatchTuning(1, 1024, 1), BatchTuning(2, 2048, 1))
    tuned = [np64(r.rf) for r in b.run()]
    for a, c in zip(eager, tuned):
        assert G.rel_l2(c, a) < PLAIN_TOL


def test_batched_consistent_with_plain_kernel_at_scale():
    """Cross-implementation property at 20k scatterers: every firing of the batched sweep
    equals the single-transmit plain kernel run with the same plan."""
    import fastsimus_gb300 as F
    from fastsimus_gb300 import workloads as W
    from fastsimus_gb300.batched import BatchedSimus

    p, m = W.cfg1_probe(), W.cfg1_medium()
    s, r = W.cfg4_scatterers(20_000, seed=5)
    delays = W.plane_wave_delays(p, m, [-12.0, 0.0, 12.0])
    b = BatchedSimus([(s, r)], delays, p, m)
    spec = np64(b.run()[0].spectrum)
    for t in range(3):
        ref = np64(F.simus_compute(s, r, delays[t], b.plans[0], p, m).spectrum)
        assert G.rel_l2(spec[:, :, t], ref) < PLAIN_TOL


def test_batched_rejects_unsupported_shapes():
    from fastsimus_gb300 import workloads as W
    from fastsimus_gb300.batched import BatchedSimus

    p, m = W.cfg1_probe(), W.cfg1_medium()
    s, r = W.cfg1_scatterers(100)
    with pytest.raises(NotImplementedError):  # 81 firings > 80
        BatchedSimus([(s, r)], np.zeros((81, 64)), p, m).run()


@pytest.mark.parametrize("n_elements", [128, 96])
def test_batched_128_element_tile_vs_oracle(n_elements):
    """Probes of 65-128 elements use the 128-element tile (one frequency per item): the
    config-2 L11 probe, and a 96-element array whose tile is a third padding."""
    import dataclasses

    from fastsimus_gb300 import workloads as W
    from fastsimus_gb300.batched import BatchedSimus

    p, m = W.cfg2_probe(), W.cfg2_medium()
    p = dataclasses.replace(p, n_elements=n_elements)
    rng = np.random.default_rng(5)
    phantoms = [(W.uniform_box(rng, n, (-8e-3, 8e-3), (6e-3, 30e-3)), rng.standard_normal(n)) for n in (120, 45)]
    delays = W.plane_wave_delays(p, m, [-8.0, 0.0, 6.0])
    b = BatchedSimus(phantoms, delays, p, m)
    res = b.run()
    for (sc, rc), plan, out in zip(phantoms, b.plans, res):
        rf = np64(out.rf)
        assert rf.shape[1] == n_elements
        for t in range(delays.shape[0]):
            ref = O.simus_compute(sc, rc, delays[t], plan, p, m)
            err = G.rel_l2(rf[:, :, t], ref.rf)
            assert err < PLAIN_TOL, (t, err)


def test_batched_phantom_without_scatterers_gives_zero():
    """A phantom with no scatterers next to a populated one: zero RF for it, unchanged RF
    for the other."""
    from fastsimus_gb300 import workloads as W
    from fastsimus_gb300.batched import BatchedSimus

    p, m = W.cfg1_probe(), W.cfg1_medium()
    s, r = W.cfg1_scatterers(500, seed=3)
    empty = (np.zeros((0, 2)), np.zeros(0))
    delays = W.plane_wave_delays(p, m, [-5.0, 5.0])
    both = BatchedSimus([(s, r), empty], delays, p, m).run()
    alone = BatchedSimus([(s, r)], delays, p, m).run()
    assert float(np.abs(np64(both[1].rf)).max()) == 0.0
    assert G.rel_l2(np64(both[0].rf), np64(alone[0].rf)) < 1e-6


def _single_firing_goldens():
    return [n for n in G.names("simus") if G.load(n).delays.ndim == 1]


@pytest.mark.parametrize("name", _single_firing_goldens())
def test_batched_matches_every_reference_golden(name):
    """Every single-firing reference fixture through the batched sweep: soft, rigid and
    impedance baffles, the C5-2v convex array, full-frequency directivity, three sub-elements,
    NaN delays with apodisation, focused and plane-wave firings, 16 to 128 elements."""
    import fastsimus_gb300 as F
    from fastsimus_gb300.batched import BatchedSimus

    g = G.load(name)
    plan = F.simus_precompute(g.scatterers, g.rc, g.delays, g.params, g.medium, fs=g.fs,
                              element_splitting=g.element_splitting)
    b = BatchedSimus([(g.scatterers, g.rc)], g.delays[None], g.params, g.medium, plans=[plan],
                     tx_apodization=g.apod, full_frequency_directivity=g.ffd)
    rf = np64(b.run()[0].rf)[:, :, 0]
    assert rf.shape == g.rf.shape
    err = G.rel_l2(rf, g.rf)
    print(f"batched {name}: relL2 {err:.3e}")
    assert err < PLAIN_TOL


@pytest.mark.parametrize("fb", [1, 2])
@pytest.mark.parametrize("probe", ["c5_convex", "rigid_ffd", "impedance_split2"])
def test_batched_probe_options_many_firings_vs_oracle(probe, fb):
    """Probe options with several firings and two phantoms against the FP64 oracle's
    simus_compute per firing: the C5-2v convex array with full-frequency directivity, a
    rigid baffle with full-frequency directivity, an impedance baffle with two sub-elements.
    fb = frequencies per work item (128-element probes always take one)."""
    import fastsimus_gb300 as F
    from fastsimus_gb300 import workloads as W
    from fastsimus_gb300.batched import BatchedSimus, BatchTuning
    from fastsimus_gb300.params import TransducerParams

    m = F.MediumParams(attenuation=0.4)
    split = None
    if probe == "c5_convex":
        p, ffd = G.load("simus_c5_convex").params, True
    elif probe == "rigid_ffd":
        p, ffd = TransducerParams(freq_center=5e6, pitch=3e-4, n_elements=40, width=2.6e-4, bandwidth=0.7,
                                  baffle="rigid"), True
    else:
        p, ffd, split = TransducerParams(freq_center=4e6, pitch=3e-4, n_elements=64, width=2.5e-4, bandwidth=0.6,
                                         baffle=1.75), False, 2
    rng = np.random.default_rng(7)
    top = 5e-3 if np.isinf(p.radius) else -5e-3
    phantoms = [(W.uniform_box(rng, n, (-12e-3, 12e-3), (top, 40e-3)), rng.standard_normal(n)) for n in (130, 60)]
    delays = W.plane_wave_delays(p, m, [-9.0, 0.0, 7.0])
    delays[1, 3] = np.nan
    plans = [F.simus_precompute(s, r, delays[0], p, m, element_splitting=split) for s, r in phantoms]
    b = BatchedSimus(phantoms, delays, p, m, plans=plans, full_frequency_directivity=ffd,
                     tuning=BatchTuning(fb, 64, 1))
    for (s, r), plan, out in zip(phantoms, plans, b.run()):
        rf = np64(out.rf)
        for t in range(delays.shape[0]):
            ref = O.simus_compute(s, r, delays[t], plan, p, m, full_frequency_directivity=ffd)
            err = G.rel_l2(rf[:, :, t], ref.rf)
            assert err < PLAIN_TOL, (t, err)


def test_batched_ffd_differs_from_centre_frequency_directivity():
    """The option is live: with full-frequency directivity the RF differs from the
    centre-frequency directivity by more than the tolerance."""
    from fastsimus_gb300 import workloads as W
    from fastsimus_gb300.batched import BatchedSimus

    g = G.load("simus_small_ffd")
    delays = W.plane_wave_delays(g.params, g.medium, [0.0, 10.0])
    a = np64(BatchedSimus([(g.scatterers, g.rc)], delays, g.params, g.medium).run()[0].rf)
    c = np64(BatchedSimus([(g.scatterers, g.rc)], delays, g.params, g.medium,
                          full_frequency_directivity=True).run()[0].rf)
    assert G.rel_l2(c, a) > 100 * PLAIN_TOL


def test_batched_ffd_wide_subelements_raise():
    import fastsimus_gb300 as F
    from fastsimus_gb300 import workloads as W
    from fastsimus_gb300.batched import BatchedSimus
    from fastsimus_gb300.params import TransducerParams

    g = G.load("simus_small_ffd")
    p = g.params
    wide = TransducerParams(freq_center=p.freq_center, pitch=4 * p.pitch, n_elements=p.n_elements,
                            width=3.5 * p.pitch, bandwidth=p.bandwidth)
    d = W.plane_wave_delays(wide, g.medium, [0.0])
    plan = F.simus_precompute(g.scatterers, g.rc, d[0], wide, g.medium, element_splitting=1)
    with pytest.raises(NotImplementedError):
        BatchedSimus([(g.scatterers, g.rc)], d, wide, g.medium, plans=[plan], full_frequency_directivity=True).run()
    with pytest.raises(NotImplementedError):
        BatchedSimus([(g.scatterers, g.rc)], d, p, g.medium, backend="tc", full_frequency_directivity=True)


def _fp32_shapes():
    from fastsimus_gb300.batched import FP32_SHAPES

    return FP32_SHAPES


@pytest.mark.parametrize("shape", _fp32_shapes(), ids=lambda s: "fb{}-e{}-bt{}-pk{}-cta{}-t{}".format(*s))
def test_batched_every_tile_shape_vs_oracle(shape):
    """Every compiled tile shape of the FP32 batched kernel (frequencies per item, element
    tile, scatterers per tile, packed FP32x2 register tile, CTAs per SM) against the FP64
    oracle, with a chunk that is not a multiple of the larger tiles' scatterer count and two
    phantoms of uneven sizes."""
    from fastsimus_gb300 import workloads as W
    from fastsimus_gb300.batched import BatchedSimus, BatchTuning

    fb, eb, bt, pk, cps, nth = shape
    p, m = (W.cfg1_probe(), W.cfg1_medium()) if eb == 64 else (W.cfg2_probe(), W.cfg2_medium())
    rng = np.random.default_rng(bt + 7 * fb + pk)
    phantoms = [(W.uniform_box(rng, n, (-8e-3, 8e-3), (5e-3, 25e-3)), rng.standard_normal(n)) for n in (190, 77)]
    delays = W.plane_wave_delays(p, m, [-7.0, 0.0, 9.0])
    apod = np.hanning(p.n_elements) + 0.3
    b = BatchedSimus(phantoms, delays, p, m, tx_apodization=apod, tuning=BatchTuning(fb, 96, cps, bt, pk, nth))
    for (s, r), plan, out in zip(phantoms, b.plans, b.run()):
        rf = np64(out.rf)
        for t in range(delays.shape[0]):
            ref = O.simus_compute(s, r, delays[t], plan, p, m, tx_apodization=apod)
            err = G.rel_l2(rf[:, :, t], ref.rf)
            assert err < PLAIN_TOL, (shape, t, err)


def test_batched_rejects_uncompiled_tile_shape():
    from fastsimus_gb300 import workloads as W
    from fastsimus_gb300.batched import BatchedSimus, BatchTuning

    p, m = W.cfg1_probe(), W.cfg1_medium()
    s, r = W.cfg1_scatterers(100)
    with pytest.raises(NotImplementedError):  # the packed register tile takes one frequency per item
        BatchedSimus([(s, r)], W.plane_wave_delays(p, m, [0.0]), p, m, tuning=BatchTuning(2, 8192, 1, 64, 1)).run()
