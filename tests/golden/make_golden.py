"""Generate the golden fixtures in this directory by running the REFERENCE implementation.

Run in a container where the reference checkout is available (read-only is fine):

    python tests/golden/make_golden.py --reference-src /root/reference/src

It imports the reference's unmodified ``fast_simus`` package (its FP64 NumPy code path) with
the annotation/shim stand-ins under ``tests/golden/_refstubs`` in place of four small third-party
packages that are absent here (array_api_compat, array_api_extra, jaxtyping, beartype), and
writes one ``.npz`` per case: inputs, plan scalars and arrays, and the reference's outputs.
The inputs come from ``fastsimus_gb300.workloads`` (seeded) and are stored in the fixture, so
tests never regenerate them.  Large outputs are stored as float32/complex64 where a 1e-7
relative pin is enough; the full-size config-1 case keeps float64 RF.
"""

from __future__ import annotations

import argparse
import sys
from math import pi
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
REPO = HERE.parent.parent


def _load_reference(src: str):
    sys.path.insert(0, str(HERE / "_refstubs"))
    sys.path.insert(0, src)
    sys.path.insert(0, str(REPO))
    import fast_simus  # noqa: F401
    from fast_simus import _pfield_math, pfield, simus, transducer_presets, tx_delay  # noqa: F401

    return fast_simus


def _ref_params(fs_mod, p):
    """Convert a fastsimus_gb300 TransducerParams into the reference's pydantic model."""
    kw = dict(freq_center=p.freq_center, pitch=p.pitch, n_elements=p.n_elements, radius=p.radius,
              bandwidth=p.bandwidth, baffle=p.baffle if isinstance(p.baffle, float) else str(p.baffle),
              height=p.height, elev_focus=p.elev_focus)
    if p.width is not None:
        kw["width"] = p.width
    else:
        kw["kerf"] = p.kerf
    return fs_mod.TransducerParams(**kw)


def _plan_dict(plan, prefix="plan_"):
    out = {}
    for k, v in plan._asdict().items():
        out[prefix + k] = np.asarray(v)
    return out


def simus_case(fs_mod, name, params, medium, scat, rc, delays, *, apod=None, ffd=False, element_splitting=None,
               rf_dtype=np.float32, fs=None, store_spectrum=True):
    rp = _ref_params(fs_mod, params)
    rm = fs_mod.MediumParams(speed_of_sound=medium.speed_of_sound, attenuation=medium.attenuation)
    plan = fs_mod.simus_precompute(scat, rc, delays, rp, rm, element_splitting=element_splitting, fs=fs)
    res = fs_mod.simus_compute(scat, rc, delays, plan, rp, rm, tx_apodization=apod,
                               full_frequency_directivity=ffd, strategy=fs_mod.SimusStrategy.PYTHON)
    sel = res.spectrum[plan.freq_idx_start: plan.freq_idx_start + plan.selected_freqs.shape[0]]
    d = dict(kind="simus", scatterers=scat, rc=rc, delays=delays, ffd=ffd,
             apod=np.ones(params.n_elements) if apod is None else apod,
             element_splitting=-1 if element_splitting is None else element_splitting,
             fs=-1.0 if fs is None else fs,
             rf=res.rf.astype(rf_dtype), rf_peak=np.max(np.abs(res.rf)))
    if store_spectrum:
        d["spectrum_selected"] = sel.astype(np.complex64)
    d.update(_plan_dict(plan))
    _save(name, params, medium, d)
    return res


def pfield_case(fs_mod, name, params, medium, grid, delays, *, apod=None, ffd=False):
    rp = _ref_params(fs_mod, params)
    rm = fs_mod.MediumParams(speed_of_sound=medium.speed_of_sound, attenuation=medium.attenuation)
    plan = fs_mod.pfield_precompute(grid, delays, rp, rm)
    out = fs_mod.pfield_compute(grid, delays, plan, rp, rm, tx_apodization=apod, full_frequency_directivity=ffd,
                                strategy=fs_mod.PfieldStrategy.VECTORIZED)
    d = dict(kind="pfield", positions=grid, delays=delays, ffd=ffd,
             apod=np.ones(params.n_elements) if apod is None else apod, prms=np.asarray(out, dtype=np.float64))
    d.update(_plan_dict(plan))
    _save(name, params, medium, d)


def _save(name, params, medium, d):
    meta = dict(freq_center=params.freq_center, pitch=params.pitch, n_elements=params.n_elements,
                width=np.nan if params.width is None else params.width,
                kerf=np.nan if params.kerf is None else params.kerf, radius=params.radius,
                bandwidth=params.bandwidth,
                baffle=params.baffle if isinstance(params.baffle, float) else str(params.baffle),
                speed_of_sound=medium.speed_of_sound, attenuation=medium.attenuation)
    payload = {f"p_{k}": np.asarray(v) for k, v in meta.items()}
    payload.update({k: np.asarray(v) for k, v in d.items()})
    path = HERE / f"{name}.npz"
    np.savez_compressed(path, **payload)
    print(f"wrote {path.name}: {path.stat().st_size / 1024:.0f} KiB")


def cfg2_full_plan_cases(fs_mod):
    """The 200,000-scatterer, 128-element frame's own plan (1,142 frequencies, k r up to
    ~2,600 rad): the reference's simus on a random 4,096-scatterer subset of that frame,
    computed on the plan of the full frame (the sweep is linear in the scatterers, so a subset
    on the full plan is a valid pin of the full-frame arithmetic), and the reference's pfield
    on every 8th point of the 256 x 512 grid with the full grid's plan."""
    from fastsimus_gb300 import workloads as W

    p2, m2 = W.cfg2_probe(), W.cfg2_medium()
    rp = _ref_params(fs_mod, p2)
    rm = fs_mod.MediumParams(speed_of_sound=m2.speed_of_sound, attenuation=m2.attenuation)
    s_full, r_full = W.cfg2_scatterers(200_000)
    delays = np.zeros(p2.n_elements)
    plan = fs_mod.simus_precompute(s_full, r_full, delays, rp, rm)
    idx = np.sort(np.random.default_rng(11).choice(s_full.shape[0], 4096, replace=False))
    s, r = s_full[idx], r_full[idx]
    res = fs_mod.simus_compute(s, r, delays, plan, rp, rm, strategy=fs_mod.SimusStrategy.PYTHON)
    sel = res.spectrum[plan.freq_idx_start: plan.freq_idx_start + plan.selected_freqs.shape[0]]
    d = dict(kind="simus", scatterers=s, rc=r, delays=delays, ffd=False, apod=np.ones(p2.n_elements),
             element_splitting=-1, fs=-1.0, subset_of=200_000, subset_index=idx.astype(np.int32),
             rf=res.rf.astype(np.float32), rf_peak=np.max(np.abs(res.rf)),
             spectrum_selected=sel.astype(np.complex64))
    d.update(_plan_dict(plan))
    _save("simus_cfg2_fullplan", p2, m2, d)

    g_full = W.cfg2_grid()
    pplan = fs_mod.pfield_precompute(g_full, delays, rp, rm)
    g = np.ascontiguousarray(g_full[::8, ::8])
    out = fs_mod.pfield_compute(g, delays, pplan, rp, rm, strategy=fs_mod.PfieldStrategy.VECTORIZED)
    d = dict(kind="pfield", positions=g, delays=delays, ffd=False, apod=np.ones(p2.n_elements),
             prms=np.asarray(out, dtype=np.float64), grid_stride=8)
    d.update(_plan_dict(pplan))
    _save("pfield_cfg2_fullplan", p2, m2, d)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference-src", default="/root/reference/src")
    ap.add_argument("--only", choices=["all", "cfg2_fullplan"], default="all",
                    help="cfg2_fullplan: only the fixtures on the 200,000-scatterer frame's own plans")
    args = ap.parse_args()
    fs_mod = _load_reference(args.reference_src)
    if args.only == "cfg2_fullplan":
        cfg2_full_plan_cases(fs_mod)
        return

    from fastsimus_gb300 import workloads as W
    from fastsimus_gb300.params import C5_2v, L11_5v, P4_2v, MediumParams, TransducerParams
    from fastsimus_gb300.plan import element_positions
    from fastsimus_gb300.tx_delay import focused, plane_wave

    # 1. BASELINE config 1 at full size: the reference's own CPU case (float64 RF).
    p1, m1 = W.cfg1_probe(), W.cfg1_medium()
    scat, rc = W.cfg1_scatterers(2000, seed=0)
    simus_case(fs_mod, "simus_cfg1_full", p1, m1, scat, rc, np.zeros(64), rf_dtype=np.float64)

    # 2. config-2 probe (128 elements, attenuation), small box, disks zeroed.
    p2, m2 = W.cfg2_probe(), W.cfg2_medium()
    rng = np.random.default_rng(1)
    s2 = W.uniform_box(rng, 300, (-6e-3, 6e-3), (5e-3, 16e-3))
    r2 = rng.standard_normal(300)
    r2[(s2[:, 0] ** 2 + (s2[:, 1] - 10e-3) ** 2) <= (2e-3) ** 2] = 0.0
    simus_case(fs_mod, "simus_cfg2_small", p2, m2, s2, r2, np.zeros(128), store_spectrum=False)

    # 3. P4-2v focused at (0, 30 mm), 6 on-axis scatterers (the reference's PyMUST case).
    p4 = P4_2v()
    ep4, _, _ = element_positions(p4.n_elements, p4.pitch, p4.radius)
    d4 = focused(ep4, np.array([0.0, 0.03]), speed_of_sound=1540.0)
    s4 = np.stack([np.zeros(6), np.linspace(1e-2, 8e-2, 6)], -1)
    simus_case(fs_mod, "simus_p4_focused", p4, MediumParams(), s4, np.ones(6), d4)

    # 4. L11-5v plane wave at 5 degrees, 6 diagonal scatterers (the reference's second case).
    pl = L11_5v()
    epl, _, _ = element_positions(pl.n_elements, pl.pitch, pl.radius)
    dl = plane_wave(epl, 5.0 * pi / 180, speed_of_sound=1540.0)
    sl = np.stack([np.linspace(-1e-2, 1e-2, 6), np.linspace(0.5e-2, 3e-2, 6)], -1)
    simus_case(fs_mod, "simus_l11_plane5", pl, MediumParams(), sl, np.ones(6), dl, store_spectrum=False)

    # 5. Convex C5-2v, 0-degree wave, scatterers incl. one behind the arc (is_out).
    pc = C5_2v()
    epc, _, apex = element_positions(pc.n_elements, pc.pitch, pc.radius)
    dc = plane_wave(epc, 0.0, speed_of_sound=1540.0, radius=pc.radius, apex_offset=apex)
    rngc = np.random.default_rng(5)
    sc = W.uniform_box(rngc, 40, (-15e-3, 15e-3), (2e-3, 40e-3))
    sc = np.concatenate([sc, np.array([[0.0, -2e-3], [0.0, 1e-3]])], 0)
    simus_case(fs_mod, "simus_c5_convex", pc, MediumParams(attenuation=0.3), sc,
               np.random.default_rng(6).standard_normal(42), dc, store_spectrum=False)

    # 6. Small custom probe variants: rigid / impedance baffle, full-frequency directivity,
    #    NaN delays + apodization, element_splitting=3, fs override.
    small = dict(freq_center=3e6, pitch=0.4e-3, n_elements=16, width=0.35e-3, bandwidth=0.7)
    rngv = np.random.default_rng(7)
    sv = W.uniform_box(rngv, 25, (-4e-3, 4e-3), (3e-3, 14e-3))
    rv = rngv.standard_normal(25)
    ev, _, _ = element_positions(16, 0.4e-3, np.inf)
    dv = plane_wave(ev, 10 * pi / 180, speed_of_sound=1500.0)
    mv = MediumParams(speed_of_sound=1500.0, attenuation=0.7)
    simus_case(fs_mod, "simus_small_rigid", TransducerParams(**small, baffle="rigid"), mv, sv, rv, dv)
    simus_case(fs_mod, "simus_small_impedance", TransducerParams(**small, baffle=1.75), mv, sv, rv, dv)
    simus_case(fs_mod, "simus_small_ffd", TransducerParams(**small), mv, sv, rv, dv, ffd=True)
    dnan = dv.copy()
    dnan[[2, 9]] = np.nan
    apod = np.hanning(16) + 0.1
    simus_case(fs_mod, "simus_small_nan_apod", TransducerParams(**small), mv, sv, rv, dnan, apod=apod)
    simus_case(fs_mod, "simus_small_split3", TransducerParams(**small), mv, sv, rv, dv, element_splitting=3,
               fs=20e6)

    # 7. Multi-transmit with one shared plan (widest delay span), 3 plane waves, cfg1 probe.
    s3, r3 = W.cfg1_scatterers(150, seed=3)
    dels = W.plane_wave_delays(p1, m1, [-16.0, 0.0, 16.0])
    rp = _ref_params(fs_mod, p1)
    rm = fs_mod.MediumParams(speed_of_sound=1540.0, attenuation=0.0)
    ip = int(np.argmax(np.ptp(dels, axis=1)))
    plan = fs_mod.simus_precompute(s3, r3, dels[ip], rp, rm)
    rfs = np.stack([fs_mod.simus_compute(s3, r3, d, plan, rp, rm, strategy=fs_mod.SimusStrategy.PYTHON).rf
                    for d in dels], axis=-1)
    d = dict(kind="simus_multi", scatterers=s3, rc=r3, delays=dels, rf=rfs.astype(np.float32),
             plan_source=ip)
    d.update(_plan_dict(plan))
    _save("simus_multi3_cfg1", p1, m1, d)

    # 8. pfield cases.
    gx, gz = np.meshgrid(np.linspace(-19e-3, 19e-3, 32), np.linspace(5e-3, 50e-3, 48))
    g2 = W._f32(np.stack([gx, gz], -1))
    pfield_case(fs_mod, "pfield_cfg2_grid", p2, m2, g2, np.zeros(128))
    gx4, gz4 = np.meshgrid(np.linspace(-2e-2, 2e-2, 24), np.linspace(2e-3, 6e-2, 30))
    g4 = W._f32(np.stack([gx4, gz4], -1))
    pfield_case(fs_mod, "pfield_p4_focused", p4, MediumParams(), g4, d4)
    gxc, gzc = np.meshgrid(np.linspace(-3e-2, 3e-2, 20), np.linspace(-5e-3, 5e-2, 22))
    pfield_case(fs_mod, "pfield_c5_convex", pc, MediumParams(), W._f32(np.stack([gxc, gzc], -1)), dc)
    gxs, gzs = np.meshgrid(np.linspace(-5e-3, 5e-3, 12), np.linspace(1e-3, 15e-3, 14))
    gs = W._f32(np.stack([gxs, gzs], -1))
    pfield_case(fs_mod, "pfield_small_rigid_nan", TransducerParams(**small, baffle="rigid"), mv, gs, dnan, apod=apod)
    pfield_case(fs_mod, "pfield_small_ffd", TransducerParams(**small, baffle=0.5), mv, gs, dv, ffd=True)

    # 9. Plan-only known answers at the benchmark sizes (scalars + band edges).
    plans = {}
    s2full, r2full = W.cfg2_scatterers()
    for key, (pp, mm, sc_, rc_, dl_) in {
        "cfg1": (p1, m1, scat, rc, np.zeros(64)),
        "cfg2": (p2, m2, s2full, r2full, np.zeros(128)),
        "cfg4_pm12": (p1, m1, *W.cfg4_scatterers(), W.plane_wave_delays(p1, m1, [12.0])[0]),
        "p4_80mm": (p4, MediumParams(), np.stack([np.zeros(6), np.linspace(1e-2, 8e-2, 6)], -1), np.ones(6), d4),
    }.items():
        pl_ = fs_mod.simus_precompute(sc_, rc_, dl_, _ref_params(fs_mod, pp),
                                      fs_mod.MediumParams(speed_of_sound=mm.speed_of_sound,
                                                          attenuation=mm.attenuation))
        plans[key] = np.array([pl_.selected_freqs.shape[0], pl_.selected_freqs[0], pl_.selected_freqs[-1],
                               pl_.n_sub, pl_.seg_length, pl_.correction_factor, pl_.n_freq_full,
                               pl_.freq_idx_start, pl_.n_fft], dtype=np.float64)
    g2full = W.cfg2_grid()
    pp2 = fs_mod.pfield_precompute(g2full, np.zeros(128), _ref_params(fs_mod, p2),
                                   fs_mod.MediumParams(speed_of_sound=1540.0, attenuation=0.5))
    plans["pfield_cfg2"] = np.array([pp2.selected_freqs.shape[0], pp2.selected_freqs[0], pp2.selected_freqs[-1],
                                     pp2.n_sub, pp2.seg_length, pp2.correction_factor], dtype=np.float64)
    np.savez_compressed(HERE / "plans_known.npz", **plans)
    print("plans:", {k: v[:1] for k, v in plans.items()})

    # 10. The 200,000-scatterer frame's own simus and pfield plans.
    cfg2_full_plan_cases(fs_mod)


if __name__ == "__main__":
    main()
