"""Shared helpers for the GPU tests: build the native library once, skip without CUDA."""

import pytest

torch = pytest.importorskip("torch")


def require_gpu():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from fastsimus_gb300 import build

    build.build()


def np64(t):
    return t.detach().to("cpu").numpy().astype("complex128" if t.is_complex() else "float64")
