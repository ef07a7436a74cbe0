"""Annotation-only stand-in for ``jaxtyping``: shape-annotated types resolve to ``Any``
and ``jaxtyped`` returns the function unchanged."""

from typing import Any


class _Subscriptable:
    def __getitem__(self, item):
        return Any


Float = Complex = Bool = Int = Shaped = Num = Real = _Subscriptable()


def jaxtyped(fn=None, *, typechecker=None):
    if fn is None:
        return lambda f: f
    return fn
