"""Loads the sm_103a device library through its C ABI.

There is no CPU fallback: if the library is missing or no GPU is present the calls fail
with an error (KG_ERR_CUDA from kg_create) instead of computing anything on the host.
"""
from __future__ import annotations

import ctypes as C
import os

from . import abi
from .build import LIB, build

_lib = None


def load(auto_build: bool = True):
    global _lib
    if _lib is not None:
        return _lib
    if auto_build:
        build()  # compiles only when the library is missing or older than a source
    elif not os.path.exists(LIB):
        raise OSError(f"{LIB} is missing; run kestrel_gb300.build.build()")
    lib = C.CDLL(LIB)
    abi.declare(lib, "kg")
    lib.kg_version.restype = C.c_char_p
    lib.kg_kernel_launches.argtypes = [C.c_void_p]
    lib.kg_kernel_launches.restype = C.c_int64
    lib.kg_stream.argtypes = [C.c_void_p]
    lib.kg_stream.restype = C.c_void_p
    lib.kg_set_kernel_timing.argtypes = [C.c_void_p, C.c_int32]
    lib.kg_set_kernel_timing.restype = C.c_int
    lib.kg_set_fused_morpho.argtypes = [C.c_void_p, C.c_int32]
    lib.kg_set_fused_morpho.restype = C.c_int
    lib.kg_set_dry_skip.argtypes = [C.c_void_p, C.c_int32]
    lib.kg_set_dry_skip.restype = C.c_int
    lib.kg_get_kernel_time.argtypes = [C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_int64)]
    lib.kg_get_kernel_time.restype = C.c_int
    lib.kg_get_counters.argtypes = [C.c_void_p, C.POINTER(C.c_int64)]
    lib.kg_get_counters.restype = C.c_int
    lib.kg_get_transfer_bytes.argtypes = [C.c_void_p, C.POINTER(C.c_int64)]
    lib.kg_get_transfer_bytes.restype = C.c_int
    lib.kg_device_bytes.argtypes = [C.c_void_p]
    lib.kg_device_bytes.restype = C.c_int64
    lib.kg_slot_bytes.argtypes = [C.c_int32, C.c_int32, C.c_int32]
    lib.kg_slot_bytes.restype = C.c_int64
    lib.kg_host_times.argtypes = [C.c_void_p, C.POINTER(C.c_double)]
    lib.kg_host_times.restype = C.c_int
    _lib = lib
    return lib


def simulation(params, precision=abi.PREC_FP64, **kw):
    from .solver import Simulation
    return Simulation(load(), "kg", params, precision=precision, **kw)
