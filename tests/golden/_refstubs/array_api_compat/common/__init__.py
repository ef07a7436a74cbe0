from . import _helpers  # noqa: F401
