"""Recipe: time the oracle (the FP64 NumPy port) against the reference's own FP64 NumPy path.

Measurement infrastructure, not product code.  The CPU baseline that ``bench.py`` reports (and
its ``--impl reference`` arm) runs ``oracle/fastsimus_fp64.py``, because the reference itself
cannot be imported on a machine that lacks its Python dependencies.  This script measures how
the port's speed compares with the reference's on the same inputs, the same plan and one core
(one BLAS thread), so that the baseline can be read as a time of the reference:

* simus: the 128-element frame's plan (built from all 200,000 scatterers, 1,142 frequencies);
  the reference's ``simus_compute`` (PYTHON strategy) and the oracle's ``simus_compute`` on
  the same random subsets of the frame's scatterers; both include the irfft and gate;
* pfield: the 256 x 512 grid's plan (274 frequencies); the reference's ``pfield_compute``
  (VECTORIZED strategy) and the oracle's on the same random grid points;
* per-scatterer flatness: the oracle's time per scatterer at several subset sizes, which is
  what the bench's linear scaling from a sample to the full frame rests on.

It imports the reference unchanged, with the stand-ins of ``tests/golden/_refstubs`` for four
absent third-party packages (as ``tests/golden/make_golden.py`` does), and writes
``oracle/port_calibration.json``.

    python oracle/calibrate_port.py --reference-src <reference checkout>/src
"""

from __future__ import annotations

import argparse
import json
import os
import platform
import sys
import time
from pathlib import Path

for _v in ("OMP_NUM_THREADS", "OPENBLAS_NUM_THREADS", "MKL_NUM_THREADS"):
    os.environ[_v] = "1"

import numpy as np  # noqa: E402

HERE = Path(__file__).resolve().parent
REPO = HERE.parent
sys.path.insert(0, str(REPO))
OUT = HERE / "port_calibration.json"


def _best(fn, reps):
    best = float("inf")
    for _ in range(reps):
        t0 = time.perf_counter()
        fn()
        best = min(best, time.perf_counter() - t0)
    return best


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference-src", required=True)
    ap.add_argument("--simus-sizes", default="512,2048")
    ap.add_argument("--flat-sizes", default="1024,4096,8192,16384")
    ap.add_argument("--points", type=int, default=8192)
    ap.add_argument("--reps", type=int, default=2)
    args = ap.parse_args()

    sys.path.insert(0, str(REPO / "tests" / "golden"))
    import make_golden as MG

    ref = MG._load_reference(args.reference_src)
    import oracle.fastsimus_fp64 as O
    from fastsimus_gb300 import workloads as W

    p2, m2 = W.cfg2_probe(), W.cfg2_medium()
    rp = MG._ref_params(ref, p2)
    rm = ref.MediumParams(speed_of_sound=m2.speed_of_sound, attenuation=m2.attenuation)
    s_full, r_full = W.cfg2_scatterers(200_000)
    delays = np.zeros(p2.n_elements)
    plan_ref = ref.simus_precompute(s_full, r_full, delays, rp, rm)
    plan_or = O.simus_precompute(s_full, r_full, delays, p2, m2)
    rng = np.random.default_rng(3)
    simus_rows = []
    for n in (int(v) for v in args.simus_sizes.split(",")):
        idx = rng.choice(s_full.shape[0], n, replace=False)
        s, r = s_full[idx], r_full[idx]
        t_ref = _best(lambda: ref.simus_compute(s, r, delays, plan_ref, rp, rm,
                                                strategy=ref.SimusStrategy.PYTHON), args.reps)
        t_or = _best(lambda: O.simus_compute(s, r, delays, plan_or, p2, m2), args.reps)
        simus_rows.append({"scatterers": n, "reference_s": t_ref, "port_s": t_or, "port_over_reference": t_or / t_ref})
        print(simus_rows[-1], flush=True)

    g_full = W.cfg2_grid().reshape(-1, 2)
    pplan_ref = ref.pfield_precompute(W.cfg2_grid(), delays, rp, rm)
    pplan_or = O.pfield_precompute(W.cfg2_grid(), delays, p2, m2)
    gi = rng.choice(g_full.shape[0], args.points, replace=False)
    g = g_full[gi]
    t_pref = _best(lambda: ref.pfield_compute(g, delays, pplan_ref, rp, rm,
                                              strategy=ref.PfieldStrategy.VECTORIZED), args.reps)
    t_por = _best(lambda: O.pfield_compute(g, delays, pplan_or, p2, m2), args.reps)
    pfield_row = {"points": args.points, "reference_s": t_pref, "port_s": t_por, "port_over_reference": t_por / t_pref}
    print(pfield_row, flush=True)

    flat = []
    for n in (int(v) for v in args.flat_sizes.split(",")):
        idx = rng.choice(s_full.shape[0], n, replace=False)
        t = _best(lambda: O.simus_spectrum_selected(s_full[idx], r_full[idx], delays, plan_or, p2, m2), 1)
        flat.append({"scatterers": n, "port_s": t, "port_us_per_scatterer": t / n * 1e6})
        print(flat[-1], flush=True)

    ratio = float(np.mean([row["port_over_reference"] for row in simus_rows]))
    out = {
        "what": "single-core time of the oracle port vs the reference's own FP64 NumPy path, same inputs and "
                "plans (128-element frame, 1,142-frequency simus plan, 274-frequency pfield plan), one BLAS thread",
        "cpu": platform.processor() or platform.machine(), "machine": platform.machine(),
        "numpy": np.__version__,
        "simus": simus_rows, "pfield": pfield_row, "port_per_scatterer_flatness": flat,
        "simus_port_over_reference_mean": ratio,
        "pfield_port_over_reference": pfield_row["port_over_reference"],
    }
    OUT.write_text(json.dumps(out, indent=1) + "\n")
    print(f"wrote {OUT}")


if __name__ == "__main__":
    main()
