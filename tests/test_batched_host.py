"""Host-side logic of the batched sweep (no GPU): the tile-shape search space of the FP32
autotuner and the mapping of BatchTuning onto the C struct."""

import ctypes

from fastsimus_gb300 import _native
from fastsimus_gb300.batched import FP32_SHAPES, BatchTuning, fp32_search_space


def test_search_space_covers_every_compiled_shape_of_the_element_tile():
    for n_elements, eb in ((64, 64), (48, 64), (128, 128), (96, 128)):
        space = fp32_search_space(n_elements, 1_000_000)
        shapes = {(c.freqs_per_item, c.tile_scatterers, c.packed, c.ctas_per_sm, c.threads_per_cta) for c in space}
        want = {(fb, bt, pk, cps, nth) for fb, e, bt, pk, cps, nth in FP32_SHAPES if e == eb}
        assert shapes == want
        # two chunk sizes bracketing the batch for every shape
        assert len(space) == 2 * len(want)
        assert {c.chunk_scatterers for c in space} == {8192, 65536}


def test_search_space_of_a_small_batch_keeps_chunks_below_twice_the_scatterers():
    space = fp32_search_space(64, 5_000)
    assert {c.chunk_scatterers for c in space} == {8192}


def test_tuning_maps_onto_the_c_struct():
    t = BatchTuning(1, 8192, 2, 32, 0, 256).to_c()
    assert (t.freqs_per_item, t.chunk_scatterers, t.ctas_per_sm, t.tile_scatterers, t.packed, t.threads_per_cta) == (
        1, 8192, 2, 32, 0, 256)
    assert ctypes.sizeof(_native.FsgBatchTuning) == 32
    d = BatchTuning()  # the kernel's default shape
    assert (d.freqs_per_item, d.tile_scatterers, d.packed, d.ctas_per_sm, d.threads_per_cta) == (2, 64, 0, 1, 256)
