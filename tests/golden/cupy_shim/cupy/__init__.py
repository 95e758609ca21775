"""NumPy stand-in for CuPy, used only by tests/golden/make_golden.py.

It lets the reference's own Python modules (dense_krylov.py, mpdok_ooc.py,
rbf_kernel.py) run on the CPU so their outputs can be frozen as golden
vectors.  Only the names those modules use are provided.
"""
import numpy as _np
from numpy import *  # noqa: F401,F403
from numpy import linalg, random  # noqa: F401

float32 = _np.float32
float64 = _np.float64


def asnumpy(a, *args, **kwargs):
    return _np.asarray(a)


class _NullStream:
    @staticmethod
    def synchronize():
        return None


class _Stream:
    null = _NullStream()


class _Device:
    def __init__(self, index=0):
        self.index = index

    @property
    def mem_info(self):
        return (1 << 40, 1 << 40)


class _Memory:
    class OutOfMemoryError(MemoryError):
        pass


class cuda:  # noqa: N801  (mirrors the cupy.cuda namespace)
    Stream = _Stream
    Device = _Device
    memory = _Memory


class _Pool:
    def free_all_blocks(self):
        return None


def get_default_memory_pool():
    return _Pool()


def get_default_pinned_memory_pool():
    return _Pool()
