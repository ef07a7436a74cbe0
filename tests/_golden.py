"""Helpers to load the golden fixtures written by ``tests/golden/make_golden.py``."""

from __future__ import annotations

from pathlib import Path
from types import SimpleNamespace

import numpy as np

from fastsimus_gb300.params import MediumParams, TransducerParams

GOLDEN = Path(__file__).resolve().parent / "golden"


def names(prefix: str = ""):
    """Fixtures computed on their own inputs' plans.  The ``*_fullplan`` fixtures, computed on
    the plan of a larger frame or grid, are listed by ``fullplan_names``."""
    return sorted(p.stem for p in GOLDEN.glob(f"{prefix}*.npz")
                  if p.stem != "plans_known" and not p.stem.endswith("_fullplan"))


def fullplan_names():
    return sorted(p.stem for p in GOLDEN.glob("*_fullplan.npz"))


def load(name: str) -> SimpleNamespace:
    z = np.load(GOLDEN / f"{name}.npz", allow_pickle=False)
    d = {k: z[k] for k in z.files}
    baffle = d["p_baffle"]
    baffle = str(baffle) if baffle.dtype.kind in "US" else float(baffle)
    width = float(d["p_width"])
    kerf = float(d["p_kerf"])
    params = TransducerParams(
        freq_center=float(d["p_freq_center"]), pitch=float(d["p_pitch"]), n_elements=int(d["p_n_elements"]),
        width=None if np.isnan(width) else width, kerf=None if np.isnan(kerf) else kerf,
        radius=float(d["p_radius"]), bandwidth=float(d["p_bandwidth"]), baffle=baffle)
    medium = MediumParams(speed_of_sound=float(d["p_speed_of_sound"]), attenuation=float(d["p_attenuation"]))
    ns = SimpleNamespace(name=name, params=params, medium=medium, **{k: v for k, v in d.items() if not k.startswith("p_")})
    for k in ("ffd",):
        if hasattr(ns, k):
            setattr(ns, k, bool(getattr(ns, k)))
    if hasattr(ns, "element_splitting"):
        es = int(ns.element_splitting)
        ns.element_splitting = None if es < 0 else es
    if hasattr(ns, "fs"):
        ns.fs = None if float(ns.fs) < 0 else float(ns.fs)
    return ns


def rel_l2(a, b) -> float:
    a = np.asarray(a, dtype=np.complex128 if np.iscomplexobj(a) or np.iscomplexobj(b) else np.float64)
    b = np.asarray(b, dtype=a.dtype)
    return float(np.linalg.norm((a - b).ravel()) / max(np.linalg.norm(b.ravel()), 1e-300))


def max_phase_err(s, s_ref, rel_floor=1e-3) -> float:
    """max |arg(S / S_ref)| over bins with |S_ref| > rel_floor * max |S_ref|."""
    s = np.asarray(s, dtype=np.complex128)
    s_ref = np.asarray(s_ref, dtype=np.complex128)
    m = np.abs(s_ref) > rel_floor * np.abs(s_ref).max()
    if not m.any():
        return 0.0
    return float(np.max(np.abs(np.angle(s[m] / s_ref[m]))))
