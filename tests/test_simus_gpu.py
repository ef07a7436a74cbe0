"""GPU parity of the plain fused FP32 simus kernel (through the C ABI) against the reference's
golden vectors and the CPU oracle.  Tolerance: relative L2 <= 1e-5 on RF and on the
selected-band spectrum (the plain-kernel target); max phase error reported."""

import numpy as np
import pytest

import oracle.fastsimus_fp64 as O
from tests import _golden as G
from tests._gpu import np64, require_gpu, torch

pytestmark = pytest.mark.gpu

PLAIN_TOL = 1e-5
CASES = [n for n in G.names("simus_") if not n.startswith("simus_multi")]


@pytest.fixture(scope="module", autouse=True)
def _gpu():
    require_gpu()


@pytest.mark.parametrize("name", CASES)
def test_simus_rf_matches_reference_golden(name):
    import fastsimus_gb300 as F

    g = G.load(name)
    res = F.simus(g.scatterers, g.rc, g.delays, g.params, g.medium, fs=g.fs, tx_apodization=g.apod,
                  element_splitting=g.element_splitting, full_frequency_directivity=g.ffd)
    rf = np64(res.rf)
    assert rf.shape == g.rf.shape
    err = G.rel_l2(rf, g.rf)
    print(f"{name}: rf relL2 = {err:.3e}")
    assert err < PLAIN_TOL
    if hasattr(g, "spectrum_selected"):
        i0 = int(g.plan_freq_idx_start)
        sel = np64(res.spectrum)[i0: i0 + g.plan_selected_freqs.shape[0]]
        e2 = G.rel_l2(sel, g.spectrum_selected)
        ph = G.max_phase_err(sel, g.spectrum_selected)
        print(f"{name}: spectrum relL2 = {e2:.3e}, max phase err = {ph:.3e} rad")
        assert e2 < PLAIN_TOL


def test_hook_selected_raw_matches_oracle():
    """simus_gb300 (the simus_cuda-shaped hook) returns the pre-correction selected band."""
    import fastsimus_gb300 as F

    g = G.load("simus_small_nan_apod")
    plan = F.simus_precompute(g.scatterers, g.rc, g.delays, g.params, g.medium)
    d = np.where(np.isnan(g.delays), 0.0, g.delays)
    a = np.where(np.isnan(g.delays), 0.0, g.apod)
    out = np64(F.simus_gb300(g.scatterers, g.rc, g.params, plan, g.medium, d, a))
    ref = O.simus_spectrum_selected(g.scatterers, g.rc, d, plan, g.params, g.medium, tx_apodization=a)
    assert out.shape == ref.shape
    assert G.rel_l2(out, ref) < PLAIN_TOL


def test_multi_transmit_shared_plan_matches_reference():
    import fastsimus_gb300 as F

    g = G.load("simus_multi3_cfg1")
    plan = F.simus_precompute(g.scatterers, g.rc, g.delays[int(g.plan_source)], g.params, g.medium)
    rf = np.stack([np64(F.simus_compute(g.scatterers, g.rc, d, plan, g.params, g.medium).rf) for d in g.delays], -1)
    assert G.rel_l2(rf, g.rf) < PLAIN_TOL


def test_zero_scatterers_and_zero_rc_give_zero_rf():
    import fastsimus_gb300 as F
    from fastsimus_gb300 import workloads as W

    p, m = W.cfg1_probe(), W.cfg1_medium()
    s, r = W.cfg1_scatterers(50)
    plan = F.simus_precompute(s, r, np.zeros(64), p, m)
    res0 = F.simus_compute(np.zeros((0, 2)), np.zeros(0), np.zeros(64), plan, p, m)
    assert float(res0.rf.abs().max()) == 0.0
    res1 = F.simus_compute(s, np.zeros(50), np.zeros(64), plan, p, m)
    assert float(res1.rf.abs().max()) < 1e-10


def test_single_scatterer_and_out_of_field():
    import fastsimus_gb300 as F
    from fastsimus_gb300.params import P4_2v

    p = P4_2v()
    s = np.array([[0.0, 3e-2]])
    res = F.simus(s, np.ones(1), np.zeros(64), p)
    rf = np64(res.rf)
    ref = O.simus(s, np.ones(1), np.zeros(64), p, F.MediumParams())
    assert np.abs(rf).max() > 0
    assert G.rel_l2(rf, ref.rf) < PLAIN_TOL
    # a scatterer behind the array (z < 0) contributes nothing
    res2 = F.simus(np.array([[0.0, 3e-2], [0.0, -1e-2]]), np.ones(2), np.zeros(64), p)
    plan = F.simus_precompute(np.array([[0.0, 3e-2], [0.0, -1e-2]]), np.ones(2), np.zeros(64), p)
    res3 = F.simus_compute(s, np.ones(1), np.zeros(64), plan, p)
    assert G.rel_l2(np64(res2.spectrum), np64(res3.spectrum)) < 1e-6


def test_linearity_in_scatterers_at_scale():
    """Spectrum is linear in the scatterer set: S(A u B) = S(A) + S(B) (size-independent
    property used at full scale)."""
    import fastsimus_gb300 as F
    from fastsimus_gb300 import workloads as W

    p, m = W.cfg2_probe(), W.cfg2_medium()
    s, r = W.cfg2_scatterers(20_000, seed=3)
    plan = F.simus_precompute(s, r, np.zeros(128), p, m)
    full = np64(F.simus_compute(s, r, np.zeros(128), plan, p, m).spectrum)
    a = np64(F.simus_compute(s[:7000], r[:7000], np.zeros(128), plan, p, m).spectrum)
    b = np64(F.simus_compute(s[7000:], r[7000:], np.zeros(128), plan, p, m).spectrum)
    assert G.rel_l2(a + b, full) < 1e-5


def test_deterministic_bitwise():
    import fastsimus_gb300 as F
    from fastsimus_gb300 import workloads as W

    p, m = W.cfg1_probe(), W.cfg1_medium()
    s, r = W.cfg1_scatterers(3000, seed=9)
    plan = F.simus_precompute(s, r, np.zeros(64), p, m)
    x = F.simus_compute(s, r, np.zeros(64), plan, p, m).spectrum
    y = F.simus_compute(s, r, np.zeros(64), plan, p, m).spectrum
    assert torch.equal(x, y)


def test_ffd_wide_subelements_raise():
    """Full-frequency directivity is supported while k_max seg/2 <= pi (the automatic
    sub-element rule); forcing one sub-element across a multi-wavelength element is refused
    instead of silently losing accuracy."""
    import fastsimus_gb300 as F
    from fastsimus_gb300.params import TransducerParams

    g = G.load("simus_small_ffd")
    p = g.params
    wide = TransducerParams(freq_center=p.freq_center, pitch=4 * p.pitch, n_elements=p.n_elements,
                            width=3.5 * p.pitch, bandwidth=p.bandwidth, baffle=p.baffle)
    with pytest.raises(NotImplementedError):
        F.simus(g.scatterers, g.rc, g.delays, wide, g.medium, full_frequency_directivity=True, element_splitting=1)


def test_cpu_strategies_raise():
    import fastsimus_gb300 as F

    g = G.load("simus_small_rigid")
    with pytest.raises(NotImplementedError):
        F.simus(g.scatterers, g.rc, g.delays, g.params, g.medium, strategy="python")


def test_bad_arguments_raise_before_launch():
    import fastsimus_gb300 as F

    g = G.load("simus_small_rigid")
    with pytest.raises(ValueError):
        F.simus(g.scatterers, g.rc[:-1], g.delays, g.params, g.medium)
    with pytest.raises(ValueError):
        F.simus(g.scatterers, g.rc, g.delays[:-1], g.params, g.medium)


@pytest.mark.parametrize("n_elements,splitting,baffle", [(65, 2, "soft"), (33, 4, "rigid"), (96, 1, 1.5)])
def test_odd_arrays_and_sub_element_counts_vs_oracle(n_elements, splitting, baffle):
    """Element counts that are not powers of two (odd, 33, 96) and 1 / 2 / 4 sub-elements
    exercise every lanes-per-point width and the padded source slots of the kernels."""
    import fastsimus_gb300 as F
    from fastsimus_gb300.params import TransducerParams

    p = TransducerParams(freq_center=5e6, pitch=3e-4, n_elements=n_elements, width=2.7e-4, bandwidth=0.65,
                         baffle=baffle)
    m = F.MediumParams(attenuation=0.3)
    rng = np.random.default_rng(n_elements)
    s = np.stack([rng.uniform(-8e-3, 8e-3, 150), rng.uniform(4e-3, 25e-3, 150)], axis=-1)
    r = rng.standard_normal(150)
    d = np.zeros(n_elements)
    plan = F.simus_precompute(s, r, d, p, m, element_splitting=splitting)
    got = np64(F.simus_compute(s, r, d, plan, p, m).rf)
    ref = O.simus_compute(s, r, d, plan, p, m)
    err = G.rel_l2(got, ref.rf)
    print(f"E={n_elements} U={splitting} baffle={baffle}: relL2 {err:.2e}")
    assert err < PLAIN_TOL


def test_full_frame_plan_matches_reference_golden():
    """The 200,000-scatterer, 128-element frame's own plan: 1,142 frequencies, k r up to
    ~2,600 rad, 18 frequency bands.  The reference ran on a random 4,096-scatterer subset of
    the frame with the full frame's plan (linearity makes that a pin of the full-frame
    arithmetic).  Checked twice: with the default workspace (one scatterer chunk; 256 tiles x
    18 bands split unevenly over the SMs) and through the C ABI with a workspace sized for 512
    scatterers, so the call runs nine chunks, the last one partial, each split unevenly."""
    import fastsimus_gb300 as F
    from fastsimus_gb300 import _device, _native
    from fastsimus_gb300 import workloads as W

    g = G.load("simus_cfg2_fullplan")
    s_full, r_full = W.cfg2_scatterers(200_000)
    np.testing.assert_array_equal(s_full[g.subset_index], g.scatterers)
    plan = F.simus_precompute(s_full, r_full, g.delays, g.params, g.medium)
    np.testing.assert_array_equal(plan.selected_freqs, g.plan_selected_freqs)
    assert (plan.n_freq_full, plan.freq_idx_start, plan.n_fft) == (
        int(g.plan_n_freq_full), int(g.plan_freq_idx_start), int(g.plan_n_fft))
    i0, nf = plan.freq_idx_start, plan.selected_freqs.shape[0]
    res = F.simus_compute(g.scatterers, g.rc, g.delays, plan, g.params, g.medium)
    rf_err = G.rel_l2(np64(res.rf), g.rf)
    sel = np64(res.spectrum)[i0:i0 + nf]
    sp_err = G.rel_l2(sel, g.spectrum_selected)
    ph = G.max_phase_err(sel, g.spectrum_selected)
    print(f"full plan, default workspace: rf relL2 {rf_err:.3e}, spectrum relL2 {sp_err:.3e}, max phase {ph:.3e} rad")
    assert rf_err < PLAIN_TOL and sp_err < PLAIN_TOL

    lib = _native.load()
    dev = torch.device("cuda", torch.cuda.current_device())
    tabs = _device.plan_tables(plan, dev)
    probe, med, fplan = _native.make_probe(g.params, plan.n_sub), _native.make_medium(g.medium), tabs.fsg_plan(plan)
    scat = torch.as_tensor(g.scatterers, device=dev)
    rc = torch.as_tensor(g.rc, device=dev)
    d = torch.as_tensor(g.delays, device=dev)
    n = g.scatterers.shape[0]
    small = lib.fsg_simus_workspace_size(probe, fplan, 512)
    assert small < lib.fsg_simus_workspace_size(probe, fplan, n)
    ws = torch.empty(small, dtype=torch.uint8, device=dev)
    out = torch.full((nf, g.params.n_elements), float("nan"), dtype=torch.complex64, device=dev)
    _native.check(lib.fsg_simus(probe, med, fplan, scat.data_ptr(), rc.data_ptr(), n, d.data_ptr(), None, 0,
                                _native.FSG_OUT_SELECTED_RAW, out.data_ptr(), ws.data_ptr(), ws.numel(),
                                torch.cuda.current_stream(dev).cuda_stream))
    torch.cuda.synchronize()
    chunked = np64(out) * plan.correction_factor
    err_c = G.rel_l2(chunked, g.spectrum_selected)
    print(f"full plan, 512-scatterer workspace (chunked): spectrum relL2 {err_c:.3e}")
    assert err_c < PLAIN_TOL


@pytest.mark.parametrize("n_elements,splitting,ffd,baffle", [
    (256, 1, False, "soft"), (256, 2, True, "rigid"), (128, 1, False, 1.5), (128, 3, False, "soft"),
    (128, 4, True, "soft"), (64, 4, False, "rigid"), (64, 1, True, "soft"),
    (192, 2, False, "soft"), (48, 2, True, 1.5), (160, 3, False, "soft"),
    (64, 6, False, "soft"), (48, 8, True, "rigid"), (32, 5, False, 1.5)])
def test_sweep_kernel_shapes_vs_oracle(n_elements, splitting, ffd, baffle):
    """Every sweep kernel against the FP64 oracle: the warp-specialised stash kernel (64, 128
    and 256 elements, one to four sub-elements, with and without full-frequency directivity),
    the single-role stash kernel (192 and 48 elements; five to eight sub-elements on probes of
    up to 64 elements) and the re-generating band kernel (160 elements x 3 sub-elements, whose
    16-slot lanes the stash kernels cannot map)."""
    import fastsimus_gb300 as F
    from fastsimus_gb300.params import TransducerParams

    p = TransducerParams(freq_center=4e6, pitch=3e-4, n_elements=n_elements, width=2.7e-4, bandwidth=0.6,
                         baffle=baffle)
    m = F.MediumParams(attenuation=0.4)
    rng = np.random.default_rng(n_elements + splitting)
    n = 140
    s = np.stack([rng.uniform(-15e-3, 15e-3, n), rng.uniform(3e-3, 35e-3, n)], axis=-1)
    r = rng.standard_normal(n)
    d = np.linspace(0.0, 2e-6, n_elements)
    d[3] = np.nan
    apod = np.hanning(n_elements) + 0.1
    plan = F.simus_precompute(s, r, d, p, m, element_splitting=splitting)
    got = np64(F.simus_compute(s, r, d, plan, p, m, tx_apodization=apod, full_frequency_directivity=ffd).rf)
    ref = O.simus_compute(s, r, d, plan, p, m, tx_apodization=apod, full_frequency_directivity=ffd)
    err = G.rel_l2(got, ref.rf)
    print(f"E={n_elements} U={splitting} ffd={ffd} baffle={baffle}: relL2 {err:.2e}")
    assert err < PLAIN_TOL


def test_more_than_four_sub_elements_on_a_wide_probe_raise():
    """Five or more sub-elements are mapped for probes of up to 64 elements; a 128-element probe
    with six raises instead of running a kernel that cannot hold it."""
    import fastsimus_gb300 as F
    from fastsimus_gb300.params import TransducerParams

    p = TransducerParams(freq_center=4e6, pitch=3e-4, n_elements=128, width=2.7e-4, bandwidth=0.6)
    s = np.array([[0.0, 0.02]])
    with pytest.raises(NotImplementedError):
        F.simus(s, np.ones(1), np.zeros(128), p, element_splitting=6)
