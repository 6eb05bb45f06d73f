"""Loader for the oracle (test infrastructure only): oracle/_build/libkestrel_oracle.so."""
import ctypes as C
import os
import subprocess

from kestrel_gb300 import abi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ORACLE_DIR = os.path.join(ROOT, "oracle")
ORACLE_SO = os.path.join(ORACLE_DIR, "_build", "libkestrel_oracle.so")

_lib = None


def load():
    global _lib
    if _lib is None:
        subprocess.run(["make", "-s", "-C", ORACLE_DIR], check=True)
        _lib = abi.declare(C.CDLL(ORACLE_SO), "ko")
        _lib.ko_timed_integrate.argtypes = [C.c_void_p, C.c_double, C.POINTER(abi.StepStats), C.POINTER(C.c_int32)]
        _lib.ko_timed_integrate.restype = C.c_double
        _lib.ko_timed_steps.argtypes = [C.c_void_p, C.c_int32, C.POINTER(abi.StepStats), C.POINTER(C.c_int32)]
        _lib.ko_timed_steps.restype = C.c_double
    return _lib


def simulation(params, **kw):
    from kestrel_gb300.solver import Simulation
    return Simulation(load(), "ko", params, **kw)
