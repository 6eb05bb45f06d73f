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
        _lib.ko_set_closure_nudge.argtypes = [C.c_int32]
        _lib.ko_set_closure_nudge.restype = None
    return _lib


def simulation(params, **kw):
    from kestrel_gb300.solver import Simulation
    return Simulation(load(), "ko", params, **kw)


def nudged_spread(params, fields=(1, 2, 3, 4, 11), modes=(1, -1, 2, 3, 4, 5), **kw):
    """How far the oracle's own result moves when its closure transcendentals are moved by
    one ulp (all up, all down, then per call at random under a few seeds): the largest
    relative L-inf change over the fields of the active tiles.  Also returns the unnudged
    simulation."""
    import numpy as np
    L = load()
    base = simulation(params, **kw)
    stats = base.run()
    worst = 0.0
    for d in modes:
        L.ko_set_closure_nudge(d)
        try:
            s = simulation(params, **kw)
            s.run()
        finally:
            L.ko_set_closure_nudge(0)
        if s.active_tiles() != base.active_tiles():
            return base, stats, float("inf")
        for f in fields:
            A = np.concatenate([s.field(t, f).ravel() for t in base.active_tiles()])
            B = np.concatenate([base.field(t, f).ravel() for t in base.active_tiles()])
            den = max(float(np.max(np.abs(B))), 1e-300)
            worst = max(worst, float(np.max(np.abs(A - B))) / den)
        s.close()
    return base, stats, worst
