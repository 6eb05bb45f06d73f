"""The batched ensemble form over the C ABI (kg_batch_*): many FP32-form simulations of
different sizes and settings advanced together, their hydraulic passes in one persistent
launch.  ``Batch.member(id)`` returns a non-owning ``Simulation`` view for read-back."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import abi, lib as _lib
from .solver import KestrelError, Simulation


def _declare(L):
    vp, P = C.c_void_p, C.POINTER
    sig = {
        "kg_batch_create": ([C.c_int32, P(vp)], C.c_int),
        "kg_batch_destroy": ([vp], None),
        "kg_batch_last_error": ([vp], C.c_char_p),
        "kg_batch_add": ([vp, P(abi.Params), P(C.c_double), C.c_int64, C.c_int64, P(C.c_int32)], C.c_int),
        "kg_batch_member": ([vp, C.c_int32], vp),
        "kg_batch_remove": ([vp, C.c_int32], C.c_int),
        "kg_batch_step": ([vp, P(C.c_int32)], C.c_int),
        "kg_batch_finished": ([vp, C.c_int32, P(C.c_int32)], C.c_int),
        "kg_batch_stats": ([vp, P(C.c_int64), P(C.c_int64)], C.c_int),
        "kg_batch_stream": ([vp], vp),
        "kg_batch_set_graphs": ([vp, C.c_int32], C.c_int),
        "kg_batch_graph_stats": ([vp, P(C.c_int64)], C.c_int),
    }
    for name, (args, res) in sig.items():
        f = getattr(L, name)
        f.argtypes = args
        f.restype = res
    return L


class Batch:
    def __init__(self, max_members: int, graphs: bool = True):
        self.L = _declare(_lib.load())
        h = C.c_void_p()
        rc = self.L.kg_batch_create(max_members, C.byref(h))
        if rc != abi.KG_OK:
            raise KestrelError(rc, "kg_batch_create failed")
        self.h = h
        self.params = {}
        self._check(self.L.kg_batch_set_graphs(self.h, 1 if graphs else 0))

    def graph_stats(self):
        """(graph launches, in-place updates, instantiations, launches of an unchanged graph
        without a capture) of the rounds so far."""
        out = (C.c_int64 * 4)()
        self._check(self.L.kg_batch_graph_stats(self.h, out))
        return tuple(out)

    def _check(self, rc):
        if rc != abi.KG_OK:
            msg = self.L.kg_batch_last_error(self.h)
            raise KestrelError(rc, msg.decode() if msg else "")

    def add(self, params: abi.Params, b0: np.ndarray | None = None) -> int:
        mid = C.c_int32()
        if b0 is not None:
            b0 = np.ascontiguousarray(b0, dtype=np.float64)
            ny1, nx1 = b0.shape
            ptr = b0.ctypes.data_as(C.POINTER(C.c_double))
        else:
            nx1 = ny1 = 0
            ptr = None
        self._check(self.L.kg_batch_add(self.h, C.byref(params), ptr, nx1, ny1, C.byref(mid)))
        self.params[mid.value] = params
        return mid.value

    def member(self, mid: int) -> Simulation:
        handle = self.L.kg_batch_member(self.h, mid)
        if not handle:
            raise KeyError(mid)
        return Simulation.view(self.L, handle, self.params[mid])

    def remove(self, mid: int):
        self._check(self.L.kg_batch_remove(self.h, mid))
        self.params.pop(mid, None)

    def step(self) -> int:
        live = C.c_int32()
        self._check(self.L.kg_batch_step(self.h, C.byref(live)))
        return live.value

    def run(self):
        while self.step() > 0:
            pass

    def finished(self, mid: int) -> bool:
        f = C.c_int32()
        self._check(self.L.kg_batch_finished(self.h, mid, C.byref(f)))
        return bool(f.value)

    def stats(self):
        a, b = C.c_int64(), C.c_int64()
        self._check(self.L.kg_batch_stats(self.h, C.byref(a), C.byref(b)))
        return a.value, b.value

    def stream(self):
        return self.L.kg_batch_stream(self.h)

    def close(self):
        if self.h:
            self.L.kg_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
