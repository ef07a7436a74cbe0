"""Annotation-only stand-in for ``beartype``: the decorator returns the function unchanged."""


def beartype(fn=None, **kwargs):
    if fn is None:
        return lambda f: f
    return fn
