"""Transmit delay laws (host, FP64): same formulas and conventions as the reference's
``tx_delay.py`` -- delays are made non-negative by subtracting their minimum.

* ``focused``        -- tx_delay.py:31-113
* ``plane_wave``     -- tx_delay.py:116-189
* ``diverging_wave`` -- tx_delay.py:192-276
"""

from __future__ import annotations

from math import cos, fmod, inf, pi, sin, sqrt, tan

import numpy as np


def focused(element_positions, focus, *, speed_of_sound: float, radius: float = inf, apex_offset: float = 0.0):
    """Delays of a spherical wave converging on ``focus`` (z > 0) or diverging from a virtual
    source behind the array (z < 0)."""
    ep = np.asarray(element_positions, dtype=np.float64)
    fo = np.asarray(focus, dtype=np.float64)
    d = np.sqrt(np.sum((ep - fo) ** 2, axis=-1))
    if radius == inf:
        sgn = np.sign(fo[-1])
    else:
        if fo.shape[0] != 2:
            raise ValueError(f"Convex arrays require 2D coordinates, got dim={fo.shape[0]}")
        sgn = np.sign(fo[0] ** 2 + (fo[-1] + apex_offset) ** 2 - radius**2)
    sgn = np.where(sgn == 0, -1, sgn)
    delays = -d * sgn / speed_of_sound
    return delays - np.min(delays)


def plane_wave(element_positions, tilt_rad: float, *, speed_of_sound: float, radius: float = inf,
               apex_offset: float = 0.0):
    """Delays of a plane wave tilted by ``tilt_rad`` from the array normal."""
    if abs(tilt_rad) >= pi / 2:
        raise ValueError("Tilt angles must satisfy |tilt_rad| < π/2")
    ep = np.asarray(element_positions, dtype=np.float64)
    xe, ze = ep[:, 0], ep[:, 1]
    if radius == inf:
        delays = xe * sin(tilt_rad) / speed_of_sound
    else:
        xn = radius * sin(tilt_rad)
        zn = radius * cos(tilt_rad) - apex_offset
        num = np.abs(ze + xn / (zn + apex_offset) * xe - xn**2 / (zn + apex_offset) - zn)
        delays = -(num / sqrt(1 + xn**2 / (zn + apex_offset) ** 2)) / speed_of_sound
    return delays - np.min(delays)


def diverging_wave(element_positions, tilt_rad: float, width_rad: float, *, aperture_length: float,
                   speed_of_sound: float):
    """Delays of a circular wave from a virtual source chosen so the wave spans ``width_rad``
    (linear arrays only)."""
    if width_rad <= 0 or width_rad >= pi:
        raise ValueError("Width angles must satisfy 0 < width_rad < π")
    tn = fmod(-tilt_rad + pi / 2, 2 * pi) - pi / 2
    sc = 1.0
    if abs(tn) > pi / 2:
        tn = pi - tn
        sc = -1.0
    z0 = sc * aperture_length / (tan(tn - width_rad / 2) - tan(tn + width_rad / 2))
    x0 = sc * z0 * tan(width_rad / 2 - tn) + aperture_length / 2
    return focused(element_positions, np.asarray([x0, z0]), speed_of_sound=speed_of_sound)
