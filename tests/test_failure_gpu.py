"""Failure detection without a GPU fault: every device-side wait of the sweeps is bounded (poll
count and a 2 s global-timer limit).  A wait on an mbarrier phase that nothing completes must
give up, report FSG_ETIMEOUT through its status word, and leave the context usable."""

import time

import numpy as np
import pytest

from tests._gpu import require_gpu, torch

pytestmark = pytest.mark.gpu


def _selftest(arrive, tries):
    from fastsimus_gb300 import _device, _native

    lib = _native.load()
    st = torch.full((1,), -1, dtype=torch.int32, device="cuda")
    t0 = time.perf_counter()
    _native.check(lib.fsg_wait_selftest(arrive, tries, st.data_ptr(), _device.stream_handle(st.device)))
    torch.cuda.synchronize()
    return int(st.item()), time.perf_counter() - t0


def test_completed_phase_is_not_a_timeout():
    require_gpu()
    from fastsimus_gb300 import _native

    status, _ = _selftest(1, 1000)
    assert status == _native.FSG_OK


def test_wait_that_never_completes_times_out_and_context_survives():
    require_gpu()
    from fastsimus_gb300 import _native

    status, dt = _selftest(0, 4096)  # poll budget runs out
    assert status == _native.FSG_ETIMEOUT and dt < 5.0
    status, dt = _selftest(0, 2**31 - 1)  # the 2 s timer limit ends it
    assert status == _native.FSG_ETIMEOUT and 1.0 < dt < 10.0
    # the context is still usable: a simus call afterwards matches the oracle
    import fastsimus_gb300 as F
    import oracle.fastsimus_fp64 as O
    from fastsimus_gb300 import workloads as W

    p, m = W.cfg1_probe(), W.cfg1_medium()
    s, r = W.cfg1_scatterers(16, seed=3)
    d = np.zeros(p.n_elements)
    plan = F.simus_precompute(s, r, d, p, m)
    rf = F.simus_compute(s, r, d, plan, p, m).rf.double().cpu().numpy()
    ref = O.simus_compute(s, r, d, plan, p, m).rf
    assert np.linalg.norm(rf - ref) / np.linalg.norm(ref) < 1e-5


def test_bad_arguments_rejected():
    require_gpu()
    from fastsimus_gb300 import _native

    lib = _native.load()
    assert lib.fsg_wait_selftest(0, 0, None, None) == _native.FSG_EINVAL
