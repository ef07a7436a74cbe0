"""The no-allocation entry point fsg_simus_noalloc, called through the C ABI.

It exists for callers that cannot allocate device memory (for example a plugin whose host
application owns all device memory and passes only input and output buffers).  The test
allocates inputs and outputs itself -- the entry point allocates nothing -- and checks two
calls in a row against fsg_simus with a caller workspace, at the plain-kernel tolerance, on
a small frame and on the 200,000-scatterer frame, whose default workspace is larger than the
static scratch (the call then runs in more, smaller scatterer chunks).  A plan whose fixed part
does not fit is rejected before anything is launched.  This file is collected last so a failure
here never hides another test.
"""

import ctypes

import numpy as np
import pytest

from tests._gpu import require_gpu, torch

pytestmark = pytest.mark.gpu

PLAIN_TOL = 1e-5


def _rel(a, b):
    a = a.to(torch.complex128)
    b = b.to(torch.complex128)
    return float(torch.linalg.vector_norm(a - b) / torch.linalg.vector_norm(b))


def _frame(which):
    import fastsimus_gb300 as F
    from fastsimus_gb300 import workloads as W

    if which == "cfg1_2k":
        p, m = W.cfg1_probe(), W.cfg1_medium()
        s, r = W.cfg1_scatterers(2000, seed=4)
        delays = W.plane_wave_delays(p, m, [7.0])[0]
    else:  # the 200,000-scatterer, 128-element frame: its default workspace is far above 16 MiB
        p, m = W.cfg2_probe(), W.cfg2_medium()
        s, r = W.cfg2_scatterers(200_000)
        delays = np.zeros(p.n_elements)
    return p, m, s, r, delays, F.simus_precompute(s, r, delays, p, m)


@pytest.mark.parametrize("which", ["cfg1_2k", "cfg2_200k"])
def test_noalloc_matches_workspace_entry_point_twice(which):
    require_gpu()
    from fastsimus_gb300 import _device, _native

    lib = _native.load()
    dev = torch.device("cuda", torch.cuda.current_device())
    p, m, s, r, delays, plan = _frame(which)
    tabs = _device.plan_tables(plan, dev)
    probe, med, fplan = _native.make_probe(p, plan.n_sub), _native.make_medium(m), tabs.fsg_plan(plan)
    scat = torch.as_tensor(s, device=dev)
    rc = torch.as_tensor(r, device=dev)
    d = torch.as_tensor(delays, device=dev)
    stream = torch.cuda.current_stream(dev).cuda_stream
    shape = (plan.n_freq_full, p.n_elements)

    ws_bytes = lib.fsg_simus_workspace_size(probe, fplan, s.shape[0])
    if which == "cfg2_200k":  # the scratch holds fewer scatterers per chunk than the default workspace
        assert ws_bytes > lib.fsg_simus_noalloc_scratch_bytes()
    ws = torch.empty(ws_bytes, dtype=torch.uint8, device=dev)
    ref = torch.empty(shape, dtype=torch.complex64, device=dev)
    _native.check(lib.fsg_simus(probe, med, fplan, scat.data_ptr(), rc.data_ptr(), s.shape[0], d.data_ptr(), None,
                                0, _native.FSG_OUT_FULL_CORRECTED, ref.data_ptr(), ws.data_ptr(), ws.numel(), stream))
    del ws
    outs = []
    for _ in range(2):
        out = torch.full(shape, float("nan"), dtype=torch.complex64, device=dev)
        _native.check(lib.fsg_simus_noalloc(probe, med, fplan, scat.data_ptr(), rc.data_ptr(), s.shape[0],
                                            d.data_ptr(), None, 0, _native.FSG_OUT_FULL_CORRECTED, out.data_ptr(),
                                            stream))
        outs.append(out)
    torch.cuda.synchronize()
    for out in outs:
        assert bool(torch.isfinite(torch.view_as_real(out)).all())
        assert _rel(out, ref) < PLAIN_TOL


def test_noalloc_rejects_requests_beyond_its_scratch():
    require_gpu()
    from fastsimus_gb300 import _native

    lib = _native.load()
    dev = torch.device("cuda", torch.cuda.current_device())
    n_freq = 200_000
    pulse = torch.zeros(2 * n_freq, dtype=torch.float64, device=dev)
    probe_s = torch.zeros(n_freq, dtype=torch.float64, device=dev)
    probe = _native.FsgProbe(n_elements=256, n_sub=1, pitch=3e-4, element_width=2.5e-4, radius=float("inf"),
                             freq_center=5e6, baffle=0, reserved0=0, baffle_impedance=0.0)
    med = _native.FsgMedium(speed_of_sound=1540.0, attenuation=0.0)
    fplan = _native.FsgFreqPlan(n_freq=n_freq, n_freq_full=n_freq, freq_idx_start=0, reserved0=0, freq_start=1e6,
                                freq_step=10.0, seg_length=2.5e-4, correction_factor=1.0,
                                pulse_spectrum=pulse.data_ptr(), probe_spectrum=probe_s.data_ptr())
    scat = torch.zeros((10, 2), dtype=torch.float64, device=dev)
    rc = torch.zeros(10, dtype=torch.float64, device=dev)
    d = torch.zeros(256, dtype=torch.float64, device=dev)
    out = torch.empty(16, dtype=torch.complex64, device=dev)
    st = lib.fsg_simus_noalloc(probe, med, fplan, scat.data_ptr(), rc.data_ptr(), 10, d.data_ptr(), None, 0,
                               _native.FSG_OUT_SELECTED_RAW, out.data_ptr(), torch.cuda.current_stream(dev).cuda_stream)
    assert st == _native.FSG_EINVAL
    assert b"static scratch" in lib.fsg_last_error_string()
