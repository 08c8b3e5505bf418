"""Minimal stand-in for numba, used only by gen_golden.py.

numba is not installed in the build container, and the reference numpy
package imports it at module scope.  The golden vectors are generated with the
plain numpy code paths (numba=False), so an identity ``jit`` and
``prange = range`` are all that the import needs.
"""
from . import typed  # noqa: F401


def jit(*args, **kwargs):
    if args and callable(args[0]):
        return args[0]
    return lambda f: f


prange = range
