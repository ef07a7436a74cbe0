"""GPU parity of the pfield kernel against the reference's golden RMS fields."""

import numpy as np
import pytest

import oracle.fastsimus_fp64 as O
from tests import _golden as G
from tests._gpu import np64, require_gpu

pytestmark = pytest.mark.gpu

CASES = G.names("pfield_")


@pytest.fixture(scope="module", autouse=True)
def _gpu():
    require_gpu()


@pytest.mark.parametrize("name", CASES)
def test_pfield_matches_reference_golden(name):
    import fastsimus_gb300 as F

    g = G.load(name)
    out = np64(F.pfield(g.positions, g.delays, g.params, g.medium, tx_apodization=g.apod,
                        full_frequency_directivity=g.ffd))
    assert out.shape == g.prms.shape
    err = G.rel_l2(out, g.prms)
    print(f"{name}: relL2 = {err:.3e}")
    assert err < 1e-5


def test_pfield_cfg2_probe_larger_grid_vs_oracle():
    import fastsimus_gb300 as F
    from fastsimus_gb300 import workloads as W

    p, m = W.cfg2_probe(), W.cfg2_medium()
    grid = W.cfg2_grid(40, 64)
    plan = F.pfield_precompute(grid, np.zeros(128), p, m)
    out = np64(F.pfield_compute(grid, np.zeros(128), plan, p, m))
    ref = O.pfield_compute(grid, np.zeros(128), plan, p, m)
    assert G.rel_l2(out, ref) < 1e-5


def test_empty_grid_raises():
    import fastsimus_gb300 as F
    from fastsimus_gb300 import workloads as W

    with pytest.raises(ValueError):
        F.pfield(np.zeros((0, 2)), np.zeros(128), W.cfg2_probe())


def test_pfield_full_grid_plan_matches_reference_golden():
    """The 256 x 512 grid's own plan (274 frequencies): the reference's RMS field on every 8th
    grid point, computed with the full grid's plan."""
    import fastsimus_gb300 as F
    from fastsimus_gb300 import workloads as W

    g = G.load("pfield_cfg2_fullplan")
    grid = W.cfg2_grid()
    np.testing.assert_array_equal(grid[::8, ::8], g.positions)
    plan = F.pfield_precompute(grid, g.delays, g.params, g.medium)
    np.testing.assert_array_equal(plan.selected_freqs, g.plan_selected_freqs)
    out = np64(F.pfield_compute(g.positions, g.delays, plan, g.params, g.medium))
    err = G.rel_l2(out, g.prms)
    print(f"pfield full-grid plan: relL2 {err:.3e}")
    assert err < 1e-5
