"""The product's host-side planning (fastsimus_gb300.plan / tx_delay / params) against the
reference's golden plans and the oracle -- CPU only."""

import math

import numpy as np
import pytest

import oracle.fastsimus_fp64 as O
from fastsimus_gb300 import plan as P
from fastsimus_gb300 import tx_delay as T
from fastsimus_gb300 import workloads as W
from fastsimus_gb300.params import BaffleType, MediumParams, TransducerParams, C5_2v, L11_5v, L12_3v, P4_2v
from tests import _golden as G


@pytest.mark.parametrize("name", [n for n in G.names("simus_") if not n.startswith("simus_multi")])
def test_simus_plan_matches_reference(name):
    g = G.load(name)
    pl = P.simus_precompute(g.scatterers, g.rc, g.delays, g.params, g.medium, fs=g.fs,
                            element_splitting=g.element_splitting)
    np.testing.assert_array_equal(pl.selected_freqs, g.plan_selected_freqs)
    np.testing.assert_allclose(pl.pulse_spectrum, g.plan_pulse_spectrum, rtol=0, atol=1e-15)
    np.testing.assert_allclose(pl.probe_spectrum, g.plan_probe_spectrum, rtol=0, atol=1e-15)
    assert (pl.n_sub, pl.n_freq_full, pl.freq_idx_start, pl.n_fft) == (
        int(g.plan_n_sub), int(g.plan_n_freq_full), int(g.plan_freq_idx_start), int(g.plan_n_fft))
    assert pl.correction_factor == pytest.approx(float(g.plan_correction_factor), rel=1e-14)


@pytest.mark.parametrize("name", G.names("pfield_"))
def test_pfield_plan_matches_reference(name):
    g = G.load(name)
    pl = P.pfield_precompute(g.positions, g.delays, g.params, g.medium)
    np.testing.assert_array_equal(pl.selected_freqs, g.plan_selected_freqs)
    assert pl.n_sub == int(g.plan_n_sub)
    assert pl.correction_factor == pytest.approx(float(g.plan_correction_factor), rel=1e-14)


def test_benchmark_plans_known():
    known = np.load(G.GOLDEN / "plans_known.npz")
    s2, r2 = W.cfg2_scatterers()
    pl = P.simus_precompute(s2, r2, np.zeros(128), W.cfg2_probe(), W.cfg2_medium())
    row = known["cfg2"]
    assert (pl.selected_freqs.shape[0], pl.n_freq_full, pl.freq_idx_start, pl.n_fft) == (
        int(row[0]), int(row[6]), int(row[7]), int(row[8]))
    pp = P.pfield_precompute(W.cfg2_grid(), np.zeros(128), W.cfg2_probe(), W.cfg2_medium())
    assert pp.selected_freqs.shape[0] == int(known["pfield_cfg2"][0])


def test_torch_inputs_plan_equal_numpy():
    torch = pytest.importorskip("torch")
    s, r = W.cfg1_scatterers(300)
    a = P.simus_precompute(s, r, np.zeros(64), W.cfg1_probe(), W.cfg1_medium())
    b = P.simus_precompute(torch.as_tensor(s), torch.as_tensor(r), torch.zeros(64, dtype=torch.float64),
                           W.cfg1_probe(), W.cfg1_medium())
    np.testing.assert_array_equal(a.selected_freqs, b.selected_freqs)
    assert a.n_fft == b.n_fft


@pytest.mark.parametrize("preset", [P4_2v, L11_5v, L12_3v, C5_2v])
def test_element_positions_match_oracle(preset):
    p = preset()
    a, ta, xa = P.element_positions(p.n_elements, p.pitch, p.radius)
    b, tb, xb = O.element_positions(p.n_elements, p.pitch, p.radius)
    np.testing.assert_array_equal(a, b)
    assert xa == xb


def test_tx_delays_match_oracle():
    p = C5_2v()
    ep, _, apex = P.element_positions(p.n_elements, p.pitch, p.radius)
    for tilt in (-0.3, 0.0, 0.2):
        np.testing.assert_allclose(T.plane_wave(ep, tilt, speed_of_sound=1540.0, radius=p.radius, apex_offset=apex),
                                   O.plane_wave(ep, tilt, speed_of_sound=1540.0, radius=p.radius, apex_offset=apex),
                                   rtol=0, atol=1e-18)
    pl = L11_5v()
    el, _, _ = P.element_positions(pl.n_elements, pl.pitch, pl.radius)
    for focus in ([0.0, 0.03], [0.005, -0.02], [0.0, 0.0]):
        np.testing.assert_allclose(T.focused(el, np.array(focus), speed_of_sound=1540.0),
                                   O.focused(el, np.array(focus), speed_of_sound=1540.0), rtol=0, atol=1e-18)
    np.testing.assert_allclose(
        T.diverging_wave(el, 0.1, 0.6, aperture_length=127 * pl.pitch, speed_of_sound=1540.0),
        O.diverging_wave(el, 0.1, 0.6, aperture_length=127 * pl.pitch, speed_of_sound=1540.0), rtol=0, atol=1e-18)
    with pytest.raises(ValueError):
        T.plane_wave(el, math.pi / 2, speed_of_sound=1540.0)
    with pytest.raises(ValueError):
        T.diverging_wave(el, 0.0, 0.0, aperture_length=0.03, speed_of_sound=1540.0)


def test_param_validation_matches_reference_rules():
    with pytest.raises(ValueError):
        TransducerParams(freq_center=5e6, pitch=3e-4, n_elements=8)  # neither width nor kerf
    with pytest.raises(ValueError):
        TransducerParams(freq_center=5e6, pitch=3e-4, n_elements=8, width=2e-4, kerf=1e-4)
    with pytest.raises(ValueError):
        TransducerParams(freq_center=5e6, pitch=3e-4, n_elements=8, width=4e-4)
    with pytest.raises(ValueError):
        TransducerParams(freq_center=5e6, pitch=3e-4, n_elements=8, kerf=3e-4)
    with pytest.raises(ValueError):
        TransducerParams(freq_center=5e6, pitch=3e-4, n_elements=8, width=2e-4, baffle=-1.0)
    with pytest.raises(ValueError):
        MediumParams(attenuation=-0.1)
    p = TransducerParams(freq_center=5e6, pitch=3e-4, n_elements=8, kerf=5e-5, baffle="RIGID")
    assert p.baffle is BaffleType.RIGID and p.element_width == pytest.approx(2.5e-4)
    with pytest.raises(ValueError):
        P.probe_spectrum(np.array([1.0]), 5e6, 2.0)


def test_shared_plan_rule_matches_oracle():
    from fastsimus_gb300.batched import shared_plan

    g = G.load("simus_multi3_cfg1")
    pl = shared_plan(g.scatterers, g.rc, list(g.delays), g.params, g.medium)
    plo, _ = O.simus_multi_transmit(g.scatterers, g.rc, list(g.delays[:1]), g.params, g.medium)
    np.testing.assert_array_equal(pl.selected_freqs, g.plan_selected_freqs)
    assert pl.n_fft == int(g.plan_n_fft)


@pytest.mark.parametrize("name", G.fullplan_names())
def test_full_frame_plans_match_reference(name):
    """The plans of the 200,000-scatterer frame and of the 256 x 512 grid, rebuilt here from
    the full inputs, equal the plans the reference used for the *_fullplan fixtures."""
    g = G.load(name)
    if g.kind == "simus":
        s, r = W.cfg2_scatterers(200_000)
        np.testing.assert_array_equal(s[g.subset_index], g.scatterers)
        pl = P.simus_precompute(s, r, g.delays, g.params, g.medium)
        assert (pl.n_sub, pl.n_freq_full, pl.freq_idx_start, pl.n_fft) == (
            int(g.plan_n_sub), int(g.plan_n_freq_full), int(g.plan_freq_idx_start), int(g.plan_n_fft))
        assert pl.selected_freqs.shape[0] == 1142
    else:
        grid = W.cfg2_grid()
        np.testing.assert_array_equal(grid[::8, ::8], g.positions)
        pl = P.pfield_precompute(grid, g.delays, g.params, g.medium)
        assert pl.selected_freqs.shape[0] == 274
    np.testing.assert_array_equal(pl.selected_freqs, g.plan_selected_freqs)
    np.testing.assert_allclose(pl.pulse_spectrum, g.plan_pulse_spectrum, rtol=0, atol=1e-15)
    np.testing.assert_allclose(pl.probe_spectrum, g.plan_probe_spectrum, rtol=0, atol=1e-15)
    assert pl.correction_factor == pytest.approx(float(g.plan_correction_factor), rel=1e-14)
