"""Recipe: compile the reference's own CUDA kernel from its source into ``oracle/_ref/``.

Test and measurement infrastructure, not product code.  The reference ships one CUDA kernel
for this path, ``src/fast_simus/kernels/simus_fused.cu`` (``simus_fused_kernel``), which it
compiles at run time through NVRTC with the problem shape as ``-D`` macros
(``kernels/cuda_simus.py:76-112``).  This script runs ``nvcc`` on that file where it lies in
the reference tree, with the same macro set and the same options translated to ``nvcc``
(``--use_fast_math``, ``-extra-device-vectorization``, C++17) for sm_103a, once per problem
shape that the tests and the benchmark use, and writes device-only fat binaries plus a
manifest:

    oracle/_ref/simus_fused_E{E}_U{U}_F{F}.fatbin
    oracle/_ref/ref_kernels.json      {"E64_U2_F635": {"file": ..., "defines": {...}}, ...}

Nothing of the reference's source is copied; the fat binaries are build outputs and stay out
of version control.  ``oracle/ref_gpu.py`` loads them with the CUDA driver API.

Run here (where the reference tree exists):  python oracle/ref_gpu_build.py [REFERENCE_ROOT]
"""

from __future__ import annotations

import json
import math
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "_ref"
# The reference tree: FASTSIMUS_REFERENCE_ROOT, or a checkout named "reference" beside this
# repository.
DEFAULT_REF = HERE.parent.parent / "reference"
KERNEL_REL = Path("src/fast_simus/kernels/simus_fused.cu")

# Pinned tuning of the shipped kernel (kernels/cuda_simus.py:50-54).
B_SCAT, ELEM_TILE, TG_SIZE, TILE_SE, GRID_BLOCKS = 10, 2, 128, 16, 256


def shapes():
    """(E, U, F) of every workload that runs the reference kernel: the 2,000-scatterer
    64-element case of the golden fixture and the 200,000-scatterer 128-element frame."""
    sys.path.insert(0, str(HERE.parent))
    import numpy as np

    import oracle.fastsimus_fp64 as O
    from fastsimus_gb300 import workloads as W

    out = []
    for probe, medium, scat in ((W.cfg1_probe(), W.cfg1_medium(), W.cfg1_scatterers(2000, seed=0)),
                                (W.cfg2_probe(), W.cfg2_medium(), W.cfg2_scatterers(200_000, seed=0))):
        s, r = scat
        plan = O.simus_precompute(s, r, np.zeros(probe.n_elements), probe, medium)
        out.append((probe.n_elements, int(plan.n_sub), int(plan.selected_freqs.shape[0])))
    return out


def defines(E: int, U: int, F: int) -> dict:
    """The -D set of kernels/cuda_simus.py:88-103."""
    return {"N_ELEM": E, "N_SUB": U, "N_FREQ": F, "N_ES": E * U, "TILE_SE": TILE_SE, "TG_SIZE": TG_SIZE,
            "MAX_FPT": (F + TG_SIZE - 1) // TG_SIZE, "B_SCAT": B_SCAT, "ELEM_TILE": ELEM_TILE}


def compile_one(src: Path, E: int, U: int, F: int) -> tuple[str, dict]:
    name = f"E{E}_U{U}_F{F}"
    dst = OUT / f"simus_fused_{name}.fatbin"
    d = defines(E, U, F)
    cmd = ["nvcc", "-fatbin", "-gencode", "arch=compute_103a,code=sm_103a", "-std=c++17", "--use_fast_math",
           "-extra-device-vectorization", *[f"-D{k}={v}" for k, v in d.items()], str(src), "-o", str(dst)]
    subprocess.run(cmd, check=True)
    return name, {"file": dst.name, "defines": d, "grid_blocks": GRID_BLOCKS, "block_threads": TG_SIZE,
                  "shmem_bytes": (7 * B_SCAT * E * U + 3 * E) * 4}


def build(ref_root: Path | None = None, quiet: bool = True) -> bool:
    """Compile every shape; returns False (and builds nothing) when the reference tree or
    nvcc is absent, as on a machine that only receives the prebuilt files."""
    ref_root = Path(ref_root or os.environ.get("FASTSIMUS_REFERENCE_ROOT", DEFAULT_REF))
    src = ref_root / KERNEL_REL
    if not src.is_file() or shutil.which("nvcc") is None:
        return False
    OUT.mkdir(exist_ok=True)
    manifest_path = OUT / "ref_kernels.json"
    want = shapes()
    if manifest_path.is_file():
        have = json.loads(manifest_path.read_text())
        if all(f"E{E}_U{U}_F{F}" in have and (OUT / have[f"E{E}_U{U}_F{F}"]["file"]).is_file() for E, U, F in want):
            if max((OUT / v["file"]).stat().st_mtime for v in have.values()) >= src.stat().st_mtime:
                return True
    with ThreadPoolExecutor(max_workers=len(want)) as ex:
        manifest = dict(ex.map(lambda s: compile_one(src, *s), want))
    manifest_path.write_text(json.dumps(manifest, indent=1))
    if not quiet:
        print(f"reference kernel built for {sorted(manifest)} in {OUT}")
    return True


if __name__ == "__main__":
    ok = build(Path(sys.argv[1]) if len(sys.argv) > 1 else None, quiet=False)
    sys.exit(0 if ok else 1)
