"""Pin the CPU oracle against golden vectors produced by the reference implementation itself."""

import numpy as np
import pytest

import oracle.fastsimus_fp64 as O
from tests import _golden as G

SIMUS = [n for n in G.names("simus_") if not n.startswith("simus_multi")]
PFIELD = G.names("pfield_")


def _plan_check(g, plan):
    np.testing.assert_array_equal(plan.selected_freqs, g.plan_selected_freqs)
    np.testing.assert_allclose(plan.pulse_spectrum, g.plan_pulse_spectrum, rtol=0, atol=1e-15)
    np.testing.assert_allclose(plan.probe_spectrum, g.plan_probe_spectrum, rtol=0, atol=1e-15)
    assert plan.n_sub == int(g.plan_n_sub)
    assert plan.seg_length == pytest.approx(float(g.plan_seg_length), rel=1e-15)
    assert plan.correction_factor == pytest.approx(float(g.plan_correction_factor), rel=1e-15)


@pytest.mark.parametrize("name", SIMUS)
def test_oracle_simus_matches_reference(name):
    g = G.load(name)
    plan = O.simus_precompute(g.scatterers, g.rc, g.delays, g.params, g.medium, fs=g.fs,
                              element_splitting=g.element_splitting)
    _plan_check(g, plan)
    assert (plan.n_freq_full, plan.freq_idx_start, plan.n_fft) == (
        int(g.plan_n_freq_full), int(g.plan_freq_idx_start), int(g.plan_n_fft))
    res = O.simus_compute(g.scatterers, g.rc, g.delays, plan, g.params, g.medium, tx_apodization=g.apod,
                          full_frequency_directivity=g.ffd)
    tol = 1e-11 if g.rf.dtype == np.float64 else 2e-7
    assert G.rel_l2(res.rf, g.rf) < tol
    if hasattr(g, "spectrum_selected"):
        i0 = plan.freq_idx_start
        sel = res.spectrum[i0: i0 + plan.selected_freqs.shape[0]]
        assert G.rel_l2(sel, g.spectrum_selected) < 2e-7


def test_oracle_multi_transmit_shared_plan():
    g = G.load("simus_multi3_cfg1")
    plan, results = O.simus_multi_transmit(g.scatterers, g.rc, list(g.delays), g.params, g.medium)
    np.testing.assert_array_equal(plan.selected_freqs, g.plan_selected_freqs)
    rf = np.stack([r.rf for r in results], axis=-1)
    assert G.rel_l2(rf, g.rf) < 2e-7


@pytest.mark.parametrize("name", PFIELD)
def test_oracle_pfield_matches_reference(name):
    g = G.load(name)
    plan = O.pfield_precompute(g.positions, g.delays, g.params, g.medium)
    _plan_check(g, plan)
    out = O.pfield_compute(g.positions, g.delays, plan, g.params, g.medium, tx_apodization=g.apod,
                           full_frequency_directivity=g.ffd)
    assert out.shape == g.prms.shape
    assert G.rel_l2(out, g.prms) < 1e-11


def test_oracle_plans_known_answers():
    """Plan scalars at benchmark sizes, including the reference's P4-2v ~812-frequency case
    (tests/test_simus.py:361-386 asserts 812 +- 20)."""
    from fastsimus_gb300 import workloads as W
    from fastsimus_gb300.params import P4_2v, MediumParams
    from fastsimus_gb300.plan import element_positions
    from fastsimus_gb300.tx_delay import focused

    known = np.load(G.GOLDEN / "plans_known.npz")
    p4 = P4_2v()
    ep4, _, _ = element_positions(64, p4.pitch, p4.radius)
    d4 = focused(ep4, np.array([0.0, 0.03]), speed_of_sound=1540.0)
    s4 = np.stack([np.zeros(6), np.linspace(1e-2, 8e-2, 6)], -1)
    pl = O.simus_precompute(s4, np.ones(6), d4, p4, MediumParams())
    row = known["p4_80mm"]
    assert pl.selected_freqs.shape[0] == int(row[0])
    assert abs(pl.selected_freqs.shape[0] - 812) < 20
    s1, r1 = W.cfg1_scatterers()
    pl1 = O.simus_precompute(s1, r1, np.zeros(64), W.cfg1_probe(), W.cfg1_medium())
    row = known["cfg1"]
    assert (pl1.selected_freqs.shape[0], pl1.n_freq_full, pl1.freq_idx_start, pl1.n_fft) == (
        int(row[0]), int(row[6]), int(row[7]), int(row[8]))


def _oracle_shard(args):
    import oracle.fastsimus_fp64 as O_

    s, r, d, plan, p, m = args
    return O_.simus_spectrum_selected(s, r, d, plan, p, m)


def test_oracle_on_full_frame_plan_matches_reference():
    """The oracle on the 200,000-scatterer frame's own plan (1,142 frequencies, k r up to
    ~2,600 rad) against the reference on a 4,096-scatterer subset; sharded over processes
    (the sweep is linear in the scatterers)."""
    import multiprocessing as mp
    import os

    from fastsimus_gb300 import workloads as W

    g = G.load("simus_cfg2_fullplan")
    s_full, r_full = W.cfg2_scatterers(200_000)
    plan = O.simus_precompute(s_full, r_full, g.delays, g.params, g.medium)
    _plan_check(g, plan)
    n = max(1, min(8, len(os.sched_getaffinity(0))))
    shards = np.array_split(np.arange(g.scatterers.shape[0]), n)
    # one BLAS thread per worker process (the spawned workers read the environment at start)
    saved = {v: os.environ.get(v) for v in ("OMP_NUM_THREADS", "OPENBLAS_NUM_THREADS", "MKL_NUM_THREADS")}
    os.environ.update({v: "1" for v in saved})
    try:
        with mp.get_context("spawn").Pool(n) as pool:
            parts = pool.map(_oracle_shard, [(g.scatterers[i], g.rc[i], g.delays, plan, g.params, g.medium)
                                             for i in shards])
    finally:
        for v, old in saved.items():
            if old is None:
                os.environ.pop(v, None)
            else:
                os.environ[v] = old
    sel = sum(parts) * plan.correction_factor
    assert G.rel_l2(sel, g.spectrum_selected) < 2e-7
    rf, _ = O.irfft_and_threshold(sel, plan, g.params.n_elements)
    assert G.rel_l2(rf, g.rf) < 2e-7

    gp = G.load("pfield_cfg2_fullplan")
    pplan = O.pfield_precompute(W.cfg2_grid(), gp.delays, gp.params, gp.medium)
    out = O.pfield_compute(gp.positions, gp.delays, pplan, gp.params, gp.medium)
    assert G.rel_l2(out, gp.prms) < 1e-11
