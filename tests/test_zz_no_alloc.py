"""kg_hydraulic_rhs_noalloc against kg_hydraulic_rhs.

The allocation-free entry point is for hosts that own all device memory themselves and
do not let a library call cudaMalloc after start-up; it keeps its scratch (the CFL-minimum
word and the tile-block list) in a static device array shared by every call.  Two calls in
a row, each on a different state, must give the same advised time step and the same
ddtExplicit / ddtImplicit planes as the context-allocating entry point (bit for bit, the
bar of the other FP64 parity tests).  This file is collected last so that a failure here
never hides another test's result; it also passes on its own in a fresh process.
"""
import ctypes as C

import numpy as np
import pytest

import cases
from kestrel_gb300 import lib

pytestmark = pytest.mark.gpu


def test_rhs_noalloc_matches_allocating_entry_point():
    L = lib.load()
    L.kg_hydraulic_rhs_noalloc.argtypes = [C.c_void_p, C.c_double, C.c_int32, C.POINTER(C.c_double)]
    L.kg_hydraulic_rhs_noalloc.restype = C.c_int
    p = cases.ref_input("flux_hydro_2d", tend=2.0, nout=1)
    sim = lib.simulation(p)
    sim.step(p.tend)
    for call in range(2):
        t = sim.time[0]
        dt = C.c_double(-1.0)
        rc = L.kg_hydraulic_rhs_noalloc(sim.h, t, 1, C.byref(dt))
        assert rc == 0, L.kg_last_error(sim.h)
        got = {tile: [sim.rhs(tile, k) for k in range(1, 6)] for tile in sim.active_tiles()}
        ref_dt = sim.hydraulic_rhs(t, 1)
        assert dt.value == ref_dt, (call, dt.value, ref_dt)
        for tile, planes in got.items():
            for k, plane in enumerate(planes, start=1):
                assert np.array_equal(plane, sim.rhs(tile, k)), (call, tile, k)
        sim.step(p.tend)
        sim.step(p.tend)
