"""API invariants of the reference's simus tests (tests/test_simus.py:253-320, :392-427),
through this package's GPU path on the reference's P4-2v preset."""

import numpy as np
import pytest

from tests._gpu import np64, require_gpu

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _gpu():
    require_gpu()


def _case():
    import fastsimus_gb300 as F

    p = F.P4_2v()
    s = np.stack([np.zeros(3), np.linspace(1e-2, 5e-2, 3)], axis=-1)
    return F, p, s, np.ones(3), np.zeros(p.n_elements)


def test_result_type_and_shapes():
    F, p, s, r, d = _case()
    res = F.simus(s, r, d, p)
    assert isinstance(res, F.SimusResult)
    assert res.rf.dim() == 2 and res.rf.shape[1] == p.n_elements
    assert res.spectrum.dim() == 2 and res.spectrum.shape[1] == p.n_elements


def test_custom_sampling_frequency_gives_more_samples():
    F, p, s, r, d = _case()
    assert F.simus(s, r, d, p, fs=10 * p.freq_center).rf.shape[0] > F.simus(s, r, d, p).rf.shape[0]


def test_precompute_then_compute_is_bitwise_simus():
    F, p, s, r, d = _case()
    a = F.simus(s, r, d, p)
    plan = F.simus_precompute(s, r, d, p)
    b = F.simus_compute(s, r, d, plan, p)
    assert np.array_equal(np64(a.rf), np64(b.rf))
    assert np.array_equal(np64(a.spectrum), np64(b.spectrum))


def test_single_scatterer_nonzero_and_attenuation_lowers_power():
    F, p, s, r, d = _case()
    one = F.simus(np.array([[0.0, 3e-2]]), np.ones(1), d, p)
    assert float(np64(one.rf).__abs__().max()) > 0
    no = F.simus(s, r, d, p, medium=F.MediumParams(attenuation=0.0))
    yes = F.simus(s, r, d, p, medium=F.MediumParams(attenuation=0.5))
    assert float((np64(yes.rf) ** 2).sum()) < float((np64(no.rf) ** 2).sum())
