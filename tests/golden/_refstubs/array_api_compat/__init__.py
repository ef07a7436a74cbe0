"""Minimal stand-in for ``array_api_compat`` (pinned 1.15.0 by the reference's uv.lock).

Only what the reference's NumPy code path touches: ``array_namespace`` returns NumPy,
the ``is_*_namespace`` predicates answer for NumPy only, and ``device`` reports "cpu".
Used solely by ``tests/golden/make_golden.py`` to run the reference unchanged.
"""

import numpy as _np

from . import common  # noqa: F401


def array_namespace(*arrays, **kwargs):
    return _np


def is_jax_namespace(xp):
    return False


def is_cupy_namespace(xp):
    return False


def is_numpy_namespace(xp):
    return xp is _np


def device(x, /):
    return "cpu"
