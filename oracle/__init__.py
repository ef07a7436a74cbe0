"""CPU oracle for the FastSIMUS simus/pfield frequency sweep.

TEST INFRASTRUCTURE, NOT PRODUCT CODE.  Only ``tests/``, ``__graft_entry__.smoke()`` and the
``cpu_baseline`` / ``--impl reference`` legs of ``bench.py`` may import this package, and only
as the tests' expected results or as the timed CPU baseline.  The product path
(``fastsimus_gb300``) never imports it and has no CPU fallback.

``oracle.fastsimus_fp64`` restates, in plain FP64 NumPy, the reference's own CPU path
(charlesbmi/FastSIMUS ``src/fast_simus``): plan, sweep set-up, the per-frequency step body,
the irfft + smooth gate, pfield, and the transmit-delay laws.  Every function cites the
reference ``file:line`` it follows.

Parity pin: the restatement is checked in ``tests/test_oracle_golden.py`` against golden
vectors produced by the reference itself (``tests/golden/make_golden.py`` imports the
reference's unmodified source with small annotation stubs and writes ``tests/golden/*.npz``).
"""

from oracle.fastsimus_fp64 import (  # noqa: F401
    BAFFLE_RIGID,
    BAFFLE_SOFT,
    pfield,
    pfield_compute,
    pfield_precompute,
    plane_wave,
    focused,
    diverging_wave,
    simus,
    simus_compute,
    simus_precompute,
    simus_spectrum_selected,
    simus_multi_transmit,
    tx_field,
    element_positions,
)
