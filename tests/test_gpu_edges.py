"""GPU parity at the edges of the tile machinery and over a full run.

- The halt-edge fatal error (src/UpdateTiles.f90:61-69): under 'halt', adding a tile on the
  domain edge returns KG_ERR_HALT_EDGE through libkestrel_gb300.so, at source placement
  and in the middle of a run, exactly where the oracle stops.
- Periodic morphodynamics with missing diagonal tiles: the reference adds no corner ghost
  tiles on a periodic domain (src/UpdateTiles.f90:415-418) while its vertex bed source and
  redistribution reach the diagonal tile; both libraries let a missing diagonal contribute
  nothing and skip its cells, and must agree within the morphodynamic bar (1e-10).
- The 256^2 cap release (plain FP64, Chezy) over its full 30 s, field by field, bit for bit.
"""
import numpy as np
import pytest

import _oracle
import cases
from kestrel_gb300 import abi, config, lib
from kestrel_gb300.solver import KestrelError
from test_gpu_parity import compare_state, pair
from test_oracle import _halt_input

pytestmark = pytest.mark.gpu


def test_halt_edge_at_placement():
    """The cap covers cells of the west edge tile: kg_load_sources refuses it."""
    p = config.parse(_halt_input(-20.5, 1.0)).params
    for make in (lib.simulation, _oracle.simulation):
        with pytest.raises(KestrelError) as e:
            make(p)
        assert abi.KG_ERR[e.value.code] == "KG_ERR_HALT_EDGE" and "outside the domain" in str(e.value)


def test_halt_edge_mid_run():
    """The cap sits in an interior tile next to the edge tile; the first activation check
    of the run reaches the edge tile.  The GPU library stops with KG_ERR_HALT_EDGE at the
    same step as the oracle."""
    p = config.parse(_halt_input(-13.0, 5.0)).params
    g, o = pair(p)
    n = 0
    codes = {}
    while True:
        for name, s in (("gpu", g), ("oracle", o)):
            try:
                s.step(p.tend)
            except KestrelError as e:
                codes[name] = e.code
        if codes or n > 2000:
            break
        n += 1
    assert set(codes) == {"gpu", "oracle"}, (n, codes)
    assert abi.KG_ERR[codes["gpu"]] == abi.KG_ERR[codes["oracle"]] == "KG_ERR_HALT_EDGE"
    assert g.time[0] == o.time[0] < p.tend


PERIODIC_MORPHO = """Domain:
nXtiles = 6
nYtiles = 6
nXpertile = 8
nYpertile = 8
Xtilesize = 16
Boundary Conditions = periodic
Cap:
  capX = -47.867778915771765
  capY = -41.49383808639782
  capRadius = 7.563777886388609
  capHeight = 2.0165894394179498
  capShape = para
  capConc = 0.2917986243935994
Parameters:
Drag = Manning
Erosion = On
Eddy Viscosity = 0.01
Solver:
Limiter = WENO
Tile Buffer = 3
T end = 0.5
Output:
N out = 1
Topog:
Type = Function
Topog function = flat
"""


def test_periodic_morphodynamics_missing_diagonal_tiles():
    p = config.parse(PERIODIC_MORPHO).params
    g, o = pair(p)
    sg, so = g.run(), o.run()
    assert (sg.steps, sg.rejected) == (so.steps, so.rejected)
    act, gh = set(o.active_tiles()), set(o.ghost_tiles())

    def wrap(i, j):
        return (i - 1) % p.nXtiles + 1 + ((j - 1) % p.nYtiles) * p.nXtiles

    missing = 0
    for t in act:
        i, j = (t - 1) % p.nXtiles + 1, (t - 1) // p.nXtiles + 1
        missing += sum(wrap(i + a, j + b) not in act | gh for a in (-1, 1) for b in (-1, 1))
    assert missing > 0
    compare_state(g, o, fields=(1, 2, 3, 4, 5, 11), tol=1e-10, what="periodic morpho")
    for t in o.active_tiles():
        bo = o.vertex(t, 1)
        assert np.max(np.abs(g.vertex(t, 1) - bo)) <= 1e-10 * max(float(np.max(np.abs(bo))), 1e-300), t
    cg, _, kg = g.redistribution_stats()
    co, _, ko = o.redistribution_stats()
    assert (cg, kg) == (co, ko) and co > 0, (cg, kg, co, ko)


@pytest.mark.slow
def test_cap_release_full_30s_bitexact():
    """The plain FP64 configuration to its end time: every field, the tile lists, the
    step counts and the volume accounting equal the oracle's (1,505 steps; the oracle takes
    about four minutes on one core)."""
    p = cases.cap_release_256(tend=30.0, nout=10)
    g, o = pair(p)
    sg, so = g.run(), o.run()
    assert (sg.steps, sg.rejected) == (so.steps, so.rejected)
    compare_state(g, o, fields=(1, 2, 3, 4, 5, 6, 7, 9), what="cap_release_30s")
    assert np.array_equal(g.volume(), o.volume())
    for t in o.active_tiles():
        for w in range(6):
            assert np.array_equal(g.maxima(t, w), o.maxima(t, w)), (t, w)
