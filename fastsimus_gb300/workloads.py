"""Seeded synthetic workloads with the shapes and value distributions of the benchmark
configurations.  No dataset is read: phantoms are drawn from ``numpy.random.default_rng``.

Positions are drawn in metres and rounded to FP32-representable values, then held as FP64,
so every implementation sees bit-identical FP64 inputs.

* ``cfg1``: 64-element linear array (pitch 0.30 mm, width 0.27 mm, fc 5 MHz, bandwidth 0.65),
  c = 1540 m/s, no attenuation, one 0-degree plane wave, 2,000 scatterers uniform in
  x in [-10, 10] mm, z in [5, 30] mm, reflectivity N(0, 1).
* ``cfg2``: 128-element array (pitch 0.30 mm, width 0.27 mm, fc 5.2 MHz, bandwidth 0.67),
  0.5 dB/cm/MHz, one 0-degree plane wave, 200,000 scatterers in x in [-19, 19] mm,
  z in [5, 50] mm, reflectivity zero inside three 2 mm disks centred at z = 15, 30, 45 mm;
  plus a 256 (x) by 512 (z) pfield grid over the same box.
* ``cfg3``: cfg1 probe, 75 plane waves at linspace(-16, 16) degrees, 16 phantoms with
  log-uniform counts in [10k, 200k] over the cfg1 box, 1-4 anechoic disks of radius 1-3 mm.
* ``cfg4``: cfg1 probe, 31 plane waves at linspace(-12, 12) degrees, 262,144 scatterers,
  N(0, 1) with a random 5 % scaled by 10.
* ``cfg5``: cfg1 probe; surrogate training samples (x, z, f, theta) uniform over the cfg1 box,
  f in fc (1 +- B/2), theta in [-16, 16] degrees; use case 1,000,000 scatterers x 75 waves.
"""

from __future__ import annotations

from math import pi

import numpy as np

from fastsimus_gb300.params import MediumParams, TransducerParams
from fastsimus_gb300.plan import element_positions
from fastsimus_gb300.tx_delay import plane_wave


def cfg1_probe() -> TransducerParams:
    return TransducerParams(freq_center=5e6, pitch=0.30e-3, n_elements=64, width=0.27e-3, height=5e-3,
                            elev_focus=20e-3, bandwidth=0.65)


def cfg1_medium() -> MediumParams:
    return MediumParams(speed_of_sound=1540.0, attenuation=0.0)


def cfg2_probe() -> TransducerParams:
    return TransducerParams(freq_center=5.2e6, pitch=0.30e-3, n_elements=128, width=0.27e-3, bandwidth=0.67)


def cfg2_medium() -> MediumParams:
    return MediumParams(speed_of_sound=1540.0, attenuation=0.5)


def _f32(a):
    return np.asarray(a, dtype=np.float32).astype(np.float64)


def uniform_box(rng, n, x_range, z_range):
    x = rng.uniform(x_range[0], x_range[1], n)
    z = rng.uniform(z_range[0], z_range[1], n)
    return _f32(np.stack([x, z], axis=-1))


def cfg1_scatterers(n: int = 2000, seed: int = 0):
    rng = np.random.default_rng(seed)
    scat = uniform_box(rng, n, (-10e-3, 10e-3), (5e-3, 30e-3))
    rc = rng.standard_normal(n)
    return scat, rc


def cfg2_scatterers(n: int = 200_000, seed: int = 0):
    rng = np.random.default_rng(seed)
    scat = uniform_box(rng, n, (-19e-3, 19e-3), (5e-3, 50e-3))
    rc = rng.standard_normal(n)
    for zc in (15e-3, 30e-3, 45e-3):
        inside = (scat[:, 0] ** 2 + (scat[:, 1] - zc) ** 2) <= (2e-3) ** 2
        rc[inside] = 0.0
    return scat, rc


def cfg2_grid(nx: int = 256, nz: int = 512):
    """(nz, nx, 2) grid over x in [-19, 19] mm, z in [5, 50] mm."""
    x = np.linspace(-19e-3, 19e-3, nx)
    z = np.linspace(5e-3, 50e-3, nz)
    xx, zz = np.meshgrid(x, z)
    return _f32(np.stack([xx, zz], axis=-1))


def plane_wave_delays(params: TransducerParams, medium: MediumParams, angles_deg):
    """(T, E) FP64 plane-wave delays x sin(theta) / c - min (tx_delay.py:116-189)."""
    epos, _, apex = element_positions(params.n_elements, params.pitch, params.radius)
    return np.stack([plane_wave(epos, float(a) * pi / 180.0, speed_of_sound=medium.speed_of_sound,
                                radius=params.radius, apex_offset=apex) for a in np.atleast_1d(angles_deg)])


def cfg3_phantoms(n_phantoms: int = 16, seed: int = 0, count_range=(10_000, 200_000)):
    """List of (scatterers (S_p, 2), rc (S_p,)) with log-uniform S_p and 1-4 anechoic disks."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n_phantoms):
        n = int(round(np.exp(rng.uniform(np.log(count_range[0]), np.log(count_range[1])))))
        scat = uniform_box(rng, n, (-10e-3, 10e-3), (5e-3, 30e-3))
        rc = rng.standard_normal(n)
        for _ in range(int(rng.integers(1, 5))):
            rad = rng.uniform(1e-3, 3e-3)
            xc = rng.uniform(-10e-3 + rad, 10e-3 - rad)
            zc = rng.uniform(5e-3 + rad, 30e-3 - rad)
            rc[((scat[:, 0] - xc) ** 2 + (scat[:, 1] - zc) ** 2) <= rad**2] = 0.0
        out.append((scat, rc))
    return out


def cfg4_scatterers(n: int = 262_144, seed: int = 0):
    rng = np.random.default_rng(seed)
    scat = uniform_box(rng, n, (-10e-3, 10e-3), (5e-3, 30e-3))
    rc = rng.standard_normal(n)
    bright = rng.choice(n, size=int(round(0.05 * n)), replace=False)
    rc[bright] *= 10.0
    return scat, rc


def cfg5_samples(n: int, params: TransducerParams | None = None, seed: int = 0, max_angle_deg: float = 16.0):
    """(n, 4) FP64 samples (x, z, f, theta) uniform over the cfg1 box, fc(1 +- B/2), +-16 deg."""
    params = params or cfg1_probe()
    rng = np.random.default_rng(seed)
    fc, b = params.freq_center, params.bandwidth
    x = rng.uniform(-10e-3, 10e-3, n)
    z = rng.uniform(5e-3, 30e-3, n)
    f = rng.uniform(fc * (1 - b / 2), fc * (1 + b / 2), n)
    th = rng.uniform(-max_angle_deg, max_angle_deg, n) * pi / 180.0
    return np.stack([_f32(x), _f32(z), f, th], axis=-1)
