"""Minimal stand-in for ``array_api_extra`` (pinned 0.11.0 by the reference's uv.lock).

``sinc`` is the normalised sinc sin(pi x)/(pi x) with sinc(0) = 1, identical to
``numpy.sinc``; ``at(a)[idx].set(v)`` returns an updated copy, as the library does for
arrays that are not written in place.
"""

import numpy as _np


def sinc(x, /, *, xp=None):
    return _np.sinc(x)


class _AtIndexed:
    def __init__(self, arr, idx):
        self._arr = arr
        self._idx = idx

    def set(self, value, **kwargs):
        out = _np.array(self._arr, copy=True)
        out[self._idx] = value
        return out


class _At:
    def __init__(self, arr):
        self._arr = arr

    def __getitem__(self, idx):
        return _AtIndexed(self._arr, idx)


def at(arr, idx=None, /):
    if idx is None:
        return _At(arr)
    return _AtIndexed(arr, idx)
