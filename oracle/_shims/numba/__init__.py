"""Test-infrastructure shim: a stand-in for ``numba`` so that pyflowreg's own
Python source imports and runs unmodified without a JIT.

Only ``njit``/``jit`` are provided, as identity decorators that accept the
keyword arguments pyflowreg passes (``fastmath``, ``cache``, ``inline``,
``parallel``).  ``prange`` is plain ``range``.  The code then runs as ordinary
(slow) Python/numpy, which is what the golden-vector generator wants: the
reference's own arithmetic in IEEE double precision without fast-math
reassociation.

Only the golden-vector generator under ``tests/golden/`` puts this directory
on ``sys.path``; nothing in the product imports it.
"""


def njit(*args, **kwargs):
    if len(args) == 1 and callable(args[0]) and not kwargs:
        return args[0]

    def deco(fn):
        return fn

    return deco


jit = njit
prange = range
