"""Fixture-generation shim: runs the reference package in pure-Python mode."""
import os
import sys

_HERE = os.path.dirname(os.path.abspath(__file__))


def activate(reference_src):
    """Put the numba stand-in and the reference sources on ``sys.path``."""
    if _HERE not in sys.path:
        sys.path.insert(0, _HERE)
    if reference_src not in sys.path:
        sys.path.insert(1, reference_src)
    import _stub  # noqa: F401
    import _hook  # noqa: F401
