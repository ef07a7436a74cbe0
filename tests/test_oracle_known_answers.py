"""Known-answer tests of the reference (tests/test_pfield_math.py:100-330), restated against the
FP64 oracle so that the oracle is pinned by hand-computed values as well as by the golden
vectors."""

from math import cos, pi, sqrt

import numpy as np

import oracle.fastsimus_fp64 as O


def _single_element(points, c=1540.0, fc=5e6):
    theta_e = np.zeros(1)
    offs = O.subelement_centroids(1e-4, 1, theta_e)
    return O.distances_and_angles(np.asarray(points, dtype=np.float64), offs, np.zeros((1, 2)), theta_e, c, fc)


def test_distance_3_4_5():
    d, _, _ = _single_element([[3e-3, 4e-3]])
    assert abs(d[0, 0, 0] - 5e-3) <= 1e-6 * 5e-3


def test_distance_clipped_at_half_wavelength():
    c, fc = 1540.0, 5e6
    dmin = c / fc / 2.0
    d, _, _ = _single_element([[0.01 * dmin, 0.01 * dmin]], c, fc)
    assert d[0, 0, 0] >= dmin


def test_angle_directly_above_element_is_zero():
    _, _, theta = _single_element([[0.0, 10e-3]])
    assert abs(theta[0, 0, 0]) < 1e-6


def test_obliquity_rigid_soft_impedance_and_horizon():
    th = np.asarray([[0.3, -0.5]])
    assert np.allclose(O.obliquity_factor(th, "rigid"), 1.0, atol=1e-15)
    angles = np.asarray([[0.0, 0.3, 0.8]])
    assert np.allclose(O.obliquity_factor(angles, "soft")[0], [cos(a) for a in angles[0]], rtol=1e-12)
    assert np.allclose(O.obliquity_factor(angles, 1.75)[0], [cos(a) / (cos(a) + 1.75) for a in angles[0]], rtol=1e-12)
    horizon = np.asarray([[pi / 2, 0.7 * pi]])
    assert np.allclose(O.obliquity_factor(horizon, "soft"), 1e-16, atol=1e-20)
    assert np.allclose(O.obliquity_factor(horizon, "rigid"), 1e-16, atol=1e-20)


def test_init_exponentials_known_values():
    d = np.asarray([[0.01, 0.02]])
    ob = np.ones((1, 2))
    init, _ = O.init_exponentials(3e6, 1540.0, 0.0, d, ob, 1e5)
    assert np.allclose(np.abs(init)[0], 1.0 / np.sqrt([0.01, 0.02]), rtol=1e-6)
    # step magnitude exp(-alpha r), alpha in Np/m from dB/cm/MHz
    _, step = O.init_exponentials(3e6, 1540.0, 0.5, np.asarray([[0.02]]), np.ones((1, 1)), 1e5)
    alpha = 0.5 / O.NEPER_TO_DB * 1e5 / 1e6 * 1e2
    assert abs(abs(step[0, 0]) - np.exp(-alpha * 0.02)) <= 1e-10
    # the initial phase is k r wrapped to [0, 2 pi)
    init, _ = O.init_exponentials(5e6, 1540.0, 0.0, np.asarray([[0.05, 0.10]]), np.ones((1, 2)), 1e5)
    ph = np.angle(init)[0] % (2 * pi)
    assert np.all(ph >= 0) and np.all(ph < 2 * pi + 1e-10)


def test_step_body_two_sources_gives_four():
    """|spectrum * sum(phase)|^2 with two sources of 0.5 (1/n_sub absorbed) and spectrum 2 is 4."""
    init = np.asarray([[0.5 + 0j, 0.5 + 0j]])
    step = np.ones((1, 2), dtype=complex)
    rp = O._pfield_sweep(init, step, np.zeros(1, dtype=bool), np.asarray([1.0]), np.asarray([2.0 + 0j]),
                         np.asarray([1.0]), 1e-4, np.zeros((1, 2)), False)
    assert abs(rp[0] - 4.0) < 1e-12


def test_select_frequencies_properties():
    plan = O.select_frequencies(5e6, 0.65, 2.5, -40.0, 5e4)
    f = np.asarray(plan.selected_freqs)
    assert f.shape[0] > 0 and plan.freq_step > 0
    assert np.all(f >= 0) and np.all(f <= 2 * 5e6)
    assert plan.pulse_spectrum.shape[0] == f.shape[0] == plan.probe_spectrum.shape[0]
