"""Minimal stand-in for numba so the reference runs as plain Python.

Used only to generate golden fixtures: ``njit``/``cuda.jit`` return the
function unchanged and ``prange`` is ``range``.  numba's JIT keeps NumPy's
semantics for the code paths used (negative-index wrap, int truncation,
legacy MT19937 ``np.random``), so outputs match the JIT-compiled reference.
"""

import numpy as _np

float64 = _np.float64
float32 = _np.float32
int32 = _np.int32
int64 = _np.int64
complex128 = _np.complex128
prange = range
_threads = [1]


def _decorator(*args, **kwargs):
    if len(args) == 1 and callable(args[0]) and not kwargs:
        return args[0]

    def wrap(fn):
        return fn

    return wrap


njit = _decorator
jit = _decorator
vectorize = _decorator


def get_num_threads():
    return _threads[0]


def set_num_threads(n):
    _threads[0] = int(n)


class _Cuda:
    jit = staticmethod(_decorator)

    @staticmethod
    def is_available():
        return False

    def __getattr__(self, name):
        raise RuntimeError("numba.cuda is unavailable in the fixture shim")


cuda = _Cuda()
