"""kg_hydraulic_rhs_noalloc against kg_hydraulic_rhs and the oracle.

The allocation-free entry point is for hosts that own all device memory themselves and
do not let a library call cudaMalloc after start-up; it keeps its scratch (the CFL-minimum
word and the tile-block list) in a static device array shared by every call.  Its results
must be those of the context-allocating entry point and of the oracle's
CalculateHydraulicRHS (bit for bit, the bar of the other FP64 parity tests), also in the
states where the context's neighbour table is refreshed lazily: right after the sources
are loaded and right after a step that activated tiles.  This file is collected last so
that a failure here never hides another test's result; it also passes on its own in a
fresh process.
"""
import ctypes as C

import numpy as np
import pytest

import _oracle
import cases
from kestrel_gb300 import abi, lib

pytestmark = pytest.mark.gpu


def noalloc():
    L = lib.load()
    L.kg_hydraulic_rhs_noalloc.argtypes = [C.c_void_p, C.c_double, C.c_int32, C.POINTER(C.c_double)]
    L.kg_hydraulic_rhs_noalloc.restype = C.c_int
    return L


def call(L, sim, t, substep=1):
    dt = C.c_double(-1.0)
    rc = L.kg_hydraulic_rhs_noalloc(sim.h, t, substep, C.byref(dt))
    return rc, dt.value


def rhs_planes(sim):
    return {tile: [sim.rhs(tile, k) for k in range(1, 6)] for tile in sim.active_tiles()}


def same_planes(a, b, what):
    assert a.keys() == b.keys(), what
    for tile in a:
        for k in range(5):
            assert np.array_equal(a[tile][k], b[tile][k]), (what, tile, k + 1)


def test_rhs_noalloc_matches_allocating_entry_point():
    """Two calls in a row, each on a different state, against kg_hydraulic_rhs."""
    L = noalloc()
    p = cases.ref_input("flux_hydro_2d", tend=2.0, nout=1)
    sim = lib.simulation(p)
    sim.step(p.tend)
    for n in range(2):
        t = sim.time[0]
        rc, dt = call(L, sim, t)
        assert rc == 0, L.kg_last_error(sim.h)
        got = rhs_planes(sim)
        ref_dt = sim.hydraulic_rhs(t, 1)
        assert dt == ref_dt, (n, dt, ref_dt)
        same_planes(got, rhs_planes(sim), f"call {n}")
        sim.step(p.tend)
        sim.step(p.tend)


def test_rhs_noalloc_after_load_and_after_activation():
    """On a fresh context straight after kg_load_sources, and straight after each step
    that activated tiles (the 256^2 cap release on 16^2-cell tiles: the flow activates a
    tile row every few steps), the call equals the oracle's CalculateHydraulicRHS; the runs
    then continue identically."""
    L = noalloc()
    p = cases.cap_release_256(tend=4.0)
    g, o = lib.simulation(p), _oracle.simulation(p)
    checked = 0
    n_prev = -1
    for n in range(400):
        tiles = o.active_tiles()
        assert g.active_tiles() == tiles, n
        if len(tiles) != n_prev:
            t = o.time[0]
            rc, dt = call(L, g, t)
            assert rc == 0, L.kg_last_error(g.h)
            assert dt == o.hydraulic_rhs(t, 1), n
            same_planes(rhs_planes(g), rhs_planes(o), f"step {n}")
            checked += 1
            n_prev = len(tiles)
        if o.time[0] >= p.tend:
            break
        g.step(p.tend)
        o.step(p.tend)
    assert checked >= 3, checked
    for tile in o.active_tiles():
        for f in (1, 2, 3, 4):
            assert np.array_equal(g.field(tile, f), o.field(tile, f)), (tile, f)


def test_rhs_noalloc_leaves_device_memory_alone():
    """A call leaves the device's free memory unchanged and the transfer counters count
    its copies."""
    torch = pytest.importorskip("torch")
    L = noalloc()
    p = cases.ref_input("flux_hydro_2d", tend=1.0, nout=1)
    sim = lib.simulation(p)
    sim.step(p.tend)
    assert call(L, sim, sim.time[0])[0] == 0  # first call on the device: symbol look-up
    torch.cuda.synchronize()
    b0 = (C.c_int64 * 2)()
    L.kg_get_transfer_bytes(sim.h, b0)
    free0 = torch.cuda.mem_get_info(0)[0]
    for _ in range(3):
        assert call(L, sim, sim.time[0])[0] == 0
    torch.cuda.synchronize()
    free1 = torch.cuda.mem_get_info(0)[0]
    b1 = (C.c_int64 * 2)()
    L.kg_get_transfer_bytes(sim.h, b1)
    assert free1 == free0, (free0, free1)
    nblocks = len(sim.active_tiles()) * ((sim.nX + 15) // 16) * ((sim.nY + 15) // 16)
    assert b1[0] - b0[0] == 3 * (nblocks * 16 + 8), (b0[0], b1[0], nblocks)
    assert b1[1] - b0[1] == 3 * 8, (b0[1], b1[1])


def test_rhs_noalloc_refuses_fp32_and_oversized_active_sets():
    """The FP32 form is refused with KG_ERR_UNSUPPORTED; an active set above the static
    limit (65,536 blocks of 16x16 cells) with KG_ERR_PARAM, after which the context still
    evaluates its RHS through the allocating entry point."""
    L = noalloc()
    g32 = lib.simulation(cases.ref_input("flux_hydro_2d", tend=1.0, nout=1), precision=abi.PREC_FP32)
    assert abi.KG_ERR[call(L, g32, 0.0)[0]] == "KG_ERR_UNSUPPORTED"
    g32.close()
    # two periodic tiles of 4096 x 2064 cells (a tile holds at most 2^24 cells): 2 x 256 x
    # 129 = 66,048 blocks, about 12 GB in FP64
    nx, ny = 4096, 2064
    p = cases.ref_input("lake_at_rest_hydro_2d", tend=1.0, nout=1, nXtiles=2, nYtiles=1, nXpertile=nx, nYpertile=ny,
                        Xtilesize=float(nx), Ytilesize=float(ny))
    p.cubes[0].length = float(2 * nx)
    p.cubes[0].width = float(ny)
    big = lib.simulation(p)
    rc, _ = call(L, big, 0.0)
    assert abi.KG_ERR[rc] == "KG_ERR_PARAM", rc
    assert b"65536" in L.kg_last_error(big.h)
    assert big.hydraulic_rhs(0.0, 1) > 0.0
    big.close()
