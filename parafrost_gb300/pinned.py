"""Host arrays in page-locked memory (pfg_host_alloc).

Uploads from and downloads into page-locked buffers run as direct DMA instead
of going through the driver's staging copies, which is what a serving or
batching host wants for the arrays it hands to the engine again and again.
Without a device (or when the allocation fails) the arrays fall back to
ordinary memory; only the transfer speed differs.
"""
from __future__ import annotations

import ctypes as C
import weakref

import numpy as np

from . import _lib


def empty(n: int, dtype) -> np.ndarray:
    dtype = np.dtype(dtype)
    nbytes = max(int(n) * dtype.itemsize, 1)
    L = _lib.lib()
    ptr = L.pfg_host_alloc(nbytes)
    if not ptr:
        return np.empty(int(n), dtype=dtype)
    buf = (C.c_uint8 * nbytes).from_address(ptr)
    weakref.finalize(buf, L.pfg_host_free, ptr)
    return np.frombuffer(buf, dtype=dtype, count=int(n))


def copy(a: np.ndarray) -> np.ndarray:
    out = empty(a.size, a.dtype)
    out[:] = a.reshape(-1)
    return out


def is_pinned(a: np.ndarray) -> bool:
    b = a
    while isinstance(b, np.ndarray) and b.base is not None:
        b = b.base
    return isinstance(b, C.Array)


class ResultBuffers:
    """Reusable page-locked output arrays for Simplifier.download_all; they
    grow to the largest batch seen. The results handed out are views into
    them, valid until the next download into the same buffers."""

    FIELDS = (("lits", np.uint32), ("off", np.uint64), ("learnt", np.uint8), ("lbd", np.uint32),
              ("usage", np.uint8), ("elim", np.uint8), ("units", np.uint32), ("pend", np.uint32),
              ("stack", np.uint32), ("rends", np.uint64))

    def __init__(self):
        self.arrays = {name: np.empty(0, dtype=dt) for name, dt in self.FIELDS}

    def get(self, name: str, n: int) -> np.ndarray:
        a = self.arrays[name]
        if a.size < n:
            a = empty(max(n, a.size + a.size // 4), a.dtype)
            self.arrays[name] = a
        return a[:n]
