"""The plain sweep's work split (fsg_internal.h cta_of_unit, used by simus_band_kernel and
simus_config): a chunk's n_bands x chunk_tiles (band, tile) units over min(SMs, units) CTAs.
A host program compiled with nvcc from the library's own header checks, over many shapes, that
every unit is swept by exactly one CTA, that the CTAs sharing a band get distinct partial slots,
and that the slot count stays below the workspace's bound 1 + ceil(SMs / n_bands)."""

import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent

PROGRAM = r"""
#include <cstdio>
#include <vector>
#include "fsg_internal.h"
using fsg::cta_of_unit;
int main() {
  const int sms_list[] = {152, 148, 132, 7, 1};
  long long checked = 0;
  for (int sms : sms_list)
    for (int nb = 1; nb <= 200; nb += (nb < 40 ? 1 : 23))
      for (long long ct : {1LL, 2LL, 3LL, 5LL, 8LL, 17LL, 64LL, 551LL, 2000LL}) {
        const long long units = nb * ct;
        const int grid = (int)(units < sms ? units : sms);
        const int bound = 1 + (sms + nb - 1) / nb;
        std::vector<int> owner(units, -1);
        std::vector<std::vector<int>> slot_cta(nb, std::vector<int>(bound, -1));
        for (int c = 0; c < grid; ++c) {
          const long long u_end = (long long)(c + 1) * units / grid;
          for (long long u = (long long)c * units / grid; u < u_end;) {
            const int band = (int)(u / ct);
            const long long t_lo = u - band * ct;
            const long long t_hi = ct < t_lo + (u_end - u) ? ct : t_lo + (u_end - u);
            const int slot = c - cta_of_unit(band * ct, units, grid);
            if (slot < 0 || slot >= bound) { printf("slot %d out of [0, %d) sms=%d nb=%d ct=%lld\n", slot, bound, sms, nb, ct); return 1; }
            if (slot_cta[band][slot] != -1 && slot_cta[band][slot] != c) { printf("slot shared\n"); return 1; }
            slot_cta[band][slot] = c;
            for (long long t = t_lo; t < t_hi; ++t) {
              if (owner[band * ct + t] != -1) { printf("unit swept twice\n"); return 1; }
              owner[band * ct + t] = c;
            }
            u += t_hi - t_lo;
          }
        }
        for (long long i = 0; i < units; ++i)
          if (owner[i] < 0) { printf("unit %lld not swept\n", i); return 1; }
        ++checked;
      }
  printf("ok %lld\n", checked);
  return 0;
}
"""


def test_band_tile_split_covers_every_unit_once(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(nvcc).exists():
        pytest.skip("nvcc not available")
    src = tmp_path / "split.cu"
    src.write_text(PROGRAM)
    exe = tmp_path / "split"
    csrc = ROOT / "fastsimus_gb300" / "csrc"
    r = subprocess.run([nvcc, "-std=c++17", "-gencode", "arch=compute_103a,code=sm_103a", f"-I{csrc}",
                        f"-I{ROOT / 'include'}", str(src), "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = subprocess.run([str(exe)], capture_output=True, text=True)
    assert out.returncode == 0 and out.stdout.startswith("ok"), out.stdout + out.stderr
