"""Transducer and medium parameter models.

Same fields, defaults, validation rules and derived properties as the reference's pydantic
models (``transducer_params.py:10-160``, ``medium_params.py:6-22``) and the same presets
(``transducer_presets.py:12-102``), written as frozen dataclasses so the package needs no
pydantic at run time.  ``height`` and ``elev_focus`` are accepted and stored but, as in the
reference, read by nothing: the simulation is 2-D with 1/sqrt(r) spreading.
"""

from __future__ import annotations

from dataclasses import dataclass, field
from enum import StrEnum
from math import inf, isfinite


class BaffleType(StrEnum):
    """Acoustic boundary of the element plane (transducer_params.py:10-20)."""

    SOFT = "soft"
    RIGID = "rigid"


def _coerce_baffle(value):
    if isinstance(value, BaffleType):
        return value
    if isinstance(value, str):
        try:
            return BaffleType(value.lower())
        except ValueError as exc:
            raise ValueError(f"baffle must be 'soft', 'rigid' or a float >= 0, got {value!r}") from exc
    v = float(value)
    if not (v >= 0.0):
        raise ValueError(f"baffle impedance ratio must be >= 0, got {value!r}")
    return v


@dataclass(frozen=True)
class TransducerParams:
    """Linear or convex array description (transducer_params.py:23-160)."""

    freq_center: float
    pitch: float
    n_elements: int
    width: float | None = None
    kerf: float | None = None
    height: float = inf
    elev_focus: float = inf
    radius: float = inf
    bandwidth: float = 0.75
    baffle: BaffleType | float = field(default=BaffleType.SOFT)

    def __post_init__(self):
        def positive(name):
            v = getattr(self, name)
            if not (v > 0):
                raise ValueError(f"{name} must be > 0, got {v!r}")

        for name in ("freq_center", "pitch", "height", "elev_focus", "radius"):
            positive(name)
        if not isinstance(self.n_elements, int) or self.n_elements <= 0:
            raise ValueError(f"n_elements must be a positive integer, got {self.n_elements!r}")
        if not (0.0 < self.bandwidth <= 2.0):
            raise ValueError(f"bandwidth must be in (0, 2.0], got {self.bandwidth!r}")
        if self.width is not None and not (self.width > 0):
            raise ValueError(f"width must be > 0, got {self.width!r}")
        if self.kerf is not None and not (self.kerf >= 0):
            raise ValueError(f"kerf must be >= 0, got {self.kerf!r}")
        object.__setattr__(self, "baffle", _coerce_baffle(self.baffle))
        if self.width is None and self.kerf is None:
            raise ValueError("Either width or kerf must be provided")
        if self.width is not None and self.kerf is not None:
            raise ValueError("Cannot specify both width and kerf. Provide only one.")
        if self.width is not None and self.width > self.pitch:
            raise ValueError(f"Element width ({self.width}) cannot exceed pitch ({self.pitch})")
        if self.kerf is not None and self.kerf >= self.pitch:
            raise ValueError(f"Kerf ({self.kerf}) must be less than pitch ({self.pitch})")

    @property
    def element_width(self) -> float:
        if self.width is not None:
            return self.width
        return self.pitch - self.kerf

    @property
    def kerf_width(self) -> float:
        if self.kerf is not None:
            return self.kerf
        return self.pitch - self.width

    @property
    def is_linear(self) -> bool:
        return not isfinite(self.radius)


@dataclass(frozen=True)
class MediumParams:
    """Propagation medium (medium_params.py:6-22)."""

    speed_of_sound: float = 1540.0
    attenuation: float = 0.0

    def __post_init__(self):
        if not (self.speed_of_sound > 0):
            raise ValueError(f"speed_of_sound must be > 0, got {self.speed_of_sound!r}")
        if not (self.attenuation >= 0):
            raise ValueError(f"attenuation must be >= 0, got {self.attenuation!r}")


def P4_2v() -> TransducerParams:
    """Phased array, 2.72 MHz, 64 elements (transducer_presets.py:12-32)."""
    return TransducerParams(freq_center=2.72e6, pitch=300e-6, n_elements=64, kerf=50e-6, bandwidth=0.74,
                            radius=inf, height=14e-3, elev_focus=60e-3)


def L11_5v() -> TransducerParams:
    """Linear array, 7.6 MHz, 128 elements (transducer_presets.py:35-55)."""
    return TransducerParams(freq_center=7.6e6, pitch=300e-6, n_elements=128, kerf=30e-6, bandwidth=0.77,
                            radius=inf, height=5e-3, elev_focus=18e-3)


def L12_3v() -> TransducerParams:
    """Linear array, 7.54 MHz, 192 elements (transducer_presets.py:58-78)."""
    return TransducerParams(freq_center=7.54e6, pitch=200e-6, n_elements=192, kerf=30e-6, bandwidth=0.93,
                            radius=inf, height=5e-3, elev_focus=20e-3)


def C5_2v() -> TransducerParams:
    """Convex array, 3.57 MHz, 128 elements, 49.57 mm radius (transducer_presets.py:81-102)."""
    return TransducerParams(freq_center=3.57e6, pitch=508e-6, n_elements=128, kerf=48e-6, bandwidth=0.79,
                            radius=49.57e-3, height=13.5e-3, elev_focus=60e-3)
