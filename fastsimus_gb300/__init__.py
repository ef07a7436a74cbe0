"""fastsimus_gb300 -- GB300 (sm_103a) implementation of the FastSIMUS simus/pfield hot path.

Drop-in names of the reference's public API (``fast_simus/__init__.py:1-33``); the frequency
sweeps run in the native library ``_lib/libfsgb300.so`` through its C ABI
(``include/fsgb300.h``).
"""

from fastsimus_gb300.params import BaffleType, MediumParams, TransducerParams, C5_2v, L11_5v, L12_3v, P4_2v
from fastsimus_gb300.plan import PfieldPlan, SimusPlan, element_positions, pfield_precompute, simus_precompute
from fastsimus_gb300.tx_delay import diverging_wave, focused, plane_wave
from fastsimus_gb300.simus import SimusResult, SimusStrategy, simus, simus_compute, simus_gb300  # noqa: E402
from fastsimus_gb300.pfield import PfieldStrategy, pfield, pfield_compute  # noqa: E402

__all__ = [
    "BaffleType",
    "MediumParams",
    "PfieldPlan",
    "PfieldStrategy",
    "SimusPlan",
    "SimusResult",
    "SimusStrategy",
    "TransducerParams",
    "C5_2v",
    "L11_5v",
    "L12_3v",
    "P4_2v",
    "diverging_wave",
    "element_positions",
    "focused",
    "pfield",
    "pfield_compute",
    "pfield_precompute",
    "plane_wave",
    "simus",
    "simus_compute",
    "simus_precompute",
    "simus_gb300",
]

