"""The FP32 form (KG_PREC_FP32) against the FP64 oracle on the same inputs.

The FP32 form keeps the free surface, the bed, the depth differences w - b, the w and
Hnpsi RHS rows, their stage updates and the dt reduction in FP64, and computes the
reconstruction, fluxes, closures and momentum rows in FP32.  Its stated error against
the FP64 oracle, per field, relative L-inf over the active cells (w: relative to the
largest depth, the scale its error lives on):

  hydraulic runs (cap release 3 s, reference cap/flux inputs)   w, Hn <= 5e-6, momenta <= 2e-5,
                                                                Hnpsi <= 1e-6
  morphodynamic reference inputs (cap_morpho 1 s, flux_morpho 2 s)  every field <= 1e-5
  the 2048^2 morphodynamic configuration on a 256^2 window of its terrain, 750 steps:
                                                                w, Hn <= 1e-5, bt <= 1e-4
Conservation of volume and solids stays at FP64 round-off (<= 1e-12, the reference's own
bar is 1e-10), depth stays >= 0, a lake at rest stays at rest to |u| <= 1e-5 m/s, and the
active and ghost tile sets are identical to the oracle's.
"""
import numpy as np
import pytest

import _oracle
import cases
import test_oracle
from kestrel_gb300 import abi, lib

pytestmark = pytest.mark.gpu


def fp32(p, **kw):
    return lib.simulation(p, precision=abi.PREC_FP32, **kw)


def field_errors(g, o):
    tiles = o.active_tiles()
    get = lambda s, f: np.concatenate([s.field(t, f).ravel() for t in tiles])
    depth = np.max(np.abs(get(o, 5)))
    errs = {}
    for f, name in ((1, "w"), (2, "rhoHnu"), (3, "rhoHnv"), (4, "Hnpsi"), (5, "Hn"), (11, "bt")):
        a, b = get(g, f), get(o, f)
        den = depth if f == 1 else np.max(np.abs(b))
        errs[name] = float(np.max(np.abs(a - b)) / den) if den > 0 else float(np.max(np.abs(a - b)))
    return errs


HYDRO = [
    ("cap_release_256", 3.0),
    ("cap_dilute_2d", 8.0),
    ("cap_conc_2d", 2.0),
    ("flux_hydro_2d", 3.0),
    ("flux_edwards2019_2d", 3.0),
]


@pytest.mark.parametrize("name,tend", HYDRO)
def test_fp32_hydraulic_error(name, tend):
    p = cases.cap_release_256(tend=tend, nout=1) if name == "cap_release_256" else cases.ref_input(name, tend=tend, nout=1)
    g, o = fp32(p), _oracle.simulation(p)
    sg, so = g.run(), o.run()
    assert g.active_tiles() == o.active_tiles() and g.ghost_tiles() == o.ghost_tiles()
    assert sg.steps == so.steps
    e = field_errors(g, o)
    assert e["w"] <= 5e-6 and e["Hn"] <= 5e-6, e
    assert e["rhoHnu"] <= 2e-5 and e["rhoHnv"] <= 2e-5, e
    assert e["Hnpsi"] <= 1e-6, e
    for t in g.active_tiles():
        assert (g.field(t, 5) >= 0).all()


@pytest.mark.parametrize("name,tend", [("cap_morpho_2d", 1.0), ("flux_morpho_2d", 2.0)])
def test_fp32_morphodynamic_error(name, tend):
    p = cases.ref_input(name, tend=tend, nout=1)
    g, o = fp32(p), _oracle.simulation(p)
    g.run()
    o.run()
    assert g.active_tiles() == o.active_tiles() and g.ghost_tiles() == o.ghost_tiles()
    e = field_errors(g, o)
    assert max(e["w"], e["Hn"], e["rhoHnu"], e["rhoHnv"]) <= 1e-5, e
    assert e["Hnpsi"] <= 1e-5 and e["bt"] <= 1e-5, e
    for t in g.active_tiles():
        assert g.field(t, 11).min() >= -p.EroDepth


# The seven flow-consistency inputs; the one-point flux series (flux_single_pt) differs from
# flux_hydro_2d only in the source-rate branch, which the FP64 parity test covers.
FP32_CONSERVATION = [c for c in test_oracle.CONSERVATION if c[0] != "flux_single_pt"]


@pytest.mark.parametrize("name,tend,nout", FP32_CONSERVATION)
def test_fp32_conservation(name, tend, nout):
    p = cases.ref_input(name, tend=tend, nout=nout)
    sim, vol_err, sol_err = test_oracle.check_conservation(p, fp32)
    assert vol_err <= 1e-12 and sol_err <= 1e-12, (vol_err, sol_err)
    for t in sim.active_tiles():
        assert (sim.field(t, 5) >= -1e-14).all()


@pytest.mark.parametrize("name", ["lake_at_rest_hydro_2d", "lake_at_rest_morpho_2d"])
def test_fp32_lake_at_rest(name):
    p = cases.ref_input(name, tend=2.0, nout=2)
    g = fp32(p)
    h0 = {t: g.field(t, 5).copy() for t in g.active_tiles()}
    g.run()
    for t in g.active_tiles():
        assert np.max(np.abs(g.field(t, 6))) <= 1e-5 and np.max(np.abs(g.field(t, 7))) <= 1e-5
        assert np.max(np.abs(g.field(t, 5) - h0[t])) <= 1e-6 * max(np.max(np.abs(h0[t])), 1.0)


def test_fp32_rejects_noalloc_entry_point():
    """The allocation-free RHS entry point serves FP64 contexts only."""
    import ctypes as C
    L = lib.load()
    L.kg_hydraulic_rhs_noalloc.argtypes = [C.c_void_p, C.c_double, C.c_int32, C.POINTER(C.c_double)]
    L.kg_hydraulic_rhs_noalloc.restype = C.c_int
    g = fp32(cases.ref_input("flux_hydro_2d", tend=1.0, nout=1))
    dt = C.c_double()
    assert abi.KG_ERR[L.kg_hydraulic_rhs_noalloc(g.h, 0.0, 1, C.byref(dt))] == "KG_ERR_UNSUPPORTED"


def test_fp32_morpho_flux_window_depth_error():
    """The 2048^2 morphodynamic configuration's own terrain, source and closures (Voellmy,
    mixed erosion with 2 m erodible depth, eddy viscosity 1e-2) on a 256^2 window of its
    terrain in 32^2 tiles (workloads.morpho_flux_window): after 750 accepted steps (t = 15 s,
    with about 2,400 refused attempts) the FP32 form's depth is within 1e-5 of the largest
    depth of the FP64 oracle's, relative L-inf, with identical step and refusal counts and
    identical active tiles (measured: 4.3e-6).  On this rough terrain the error then grows as wet/dry fronts move apart (3.6e-5 at t = 20 s), while the
    oracle's own result moves by only about 1e-10 when its transcendentals are nudged."""
    from kestrel_gb300 import workloads
    p, b0 = workloads.morpho_flux_window(tend=15.0)
    g, o = fp32(p, b0=b0), _oracle.simulation(p, b0=b0)
    sg, so = g.integrate_to(15.0), o.integrate_to(15.0)
    assert (sg.steps, sg.rejected) == (so.steps, so.rejected), (sg.steps, sg.rejected, so.steps, so.rejected)
    assert sg.steps >= 600
    assert g.active_tiles() == o.active_tiles()
    e = field_errors(g, o)
    assert e["Hn"] <= 1e-5 and e["w"] <= 1e-5, e
    assert e["bt"] <= 1e-4, e


def test_fp32_state_round_trip():
    """The FP32 form stores its momenta as floats packed in the momentum plane: the
    per-tile getters, kg_get_state and kg_set_tile_field convert, and a context restarted
    from kg_get_state (kg_load_state) continues with the uninterrupted one (within 1e-6:
    the restart rebuilds the cell topography from the vertices with the FP64 path's
    compensated sums, the running form updates it incrementally)."""
    from kestrel_gb300.solver import Simulation
    p = cases.ref_input("cap_morpho_2d", tend=0.5, nout=1)
    g = fp32(p)
    g.run()
    ids, st, bt, t = g.get_state()
    for k, tile in enumerate(ids):
        for f in range(4):
            assert np.array_equal(st[k, f], g.field(tile, f + 1)), (tile, f)
        m = st[k, 1]
        assert np.array_equal(m, m.astype(np.float32).astype(np.float64))  # FP32 values
    r = Simulation(lib.load(), "kg", p, precision=abi.PREC_FP32, load_sources=False)
    r.load_state(ids, st, bt, t)
    for s in (g, r):
        s.integrate_to(0.8)
    a, b = g.get_state(), r.get_state()
    assert a[0] == b[0] and abs(a[3] - b[3]) <= 1e-9
    for f in range(4):
        x, y = a[1][:, f], b[1][:, f]
        assert np.max(np.abs(x - y)) <= 1e-6 * max(float(np.max(np.abs(x))), 1e-300), f
    assert np.max(np.abs(a[2] - b[2])) <= 1e-6 * max(float(np.max(np.abs(a[2]))), 1e-300)
    # writing one momentum leaves the other and the free surface alone
    tile = ids[0]
    w0, m2 = g.field(tile, 1).copy(), g.field(tile, 3).copy()
    new = np.full_like(m2, 0.125)
    g.set_field(tile, 2, new)
    assert np.array_equal(g.field(tile, 2), new)
    assert np.array_equal(g.field(tile, 3), m2) and np.array_equal(g.field(tile, 1), w0)


def _fused_case(name):
    from kestrel_gb300 import config, workloads
    if name == "periodic_morpho":
        import test_gpu_edges
        return config.parse(test_gpu_edges.PERIODIC_MORPHO).params, None
    if name == "window":
        return workloads.morpho_flux_window(tend=3.0)
    return cases.ref_input(name, tend={"cap_morpho_2d": 1.0, "flux_morpho_2d": 2.0}[name], nout=1), None


@pytest.mark.parametrize("name", ["cap_morpho_2d", "flux_morpho_2d", "periodic_morpho", "window"])
def test_fp32_fused_morpho_stages_match_three_launches(name):
    """The FP32 form runs each stage of the morphodynamic operator as one launch (E - D of a
    16 x 16 block and the ring of cells around it, the vertex source and bed update, then the
    cell bed and w / Hnpsi update, from shared memory; the refinement tests in the third).
    With kg_set_fused_morpho(0) the same stage runs as the per-item E - D, vertex and cell
    launches.  Both end in the same state bit for bit, with the same accepted and refused
    steps and redistribution walks: on 50^2 tiles (partial blocks), on 8^2 tiles of a
    periodic domain whose diagonal tiles are missing, and on the 2048^2 configuration's
    terrain window in 32^2 tiles."""
    p, b0 = _fused_case(name)
    L = lib.load()
    runs = []
    for fused in (1, 0):
        s = fp32(p, b0=b0)
        assert L.kg_set_fused_morpho(s.h, fused) == abi.KG_OK
        st = s.run()
        state = {t: [s.field(t, f).copy() for f in (1, 2, 3, 4, 5, 11)] + [s.vertex(t, 1).copy()] for t in s.active_tiles()}
        runs.append((st.steps, st.rejected, s.time[0], s.redistribution_stats(), s.ghost_tiles(), state,
                     L.kg_kernel_launches(s.h)))
        s.close()
    a, b = runs
    assert a[:5] == b[:5], (a[:5], b[:5])
    assert a[5].keys() == b[5].keys()
    for t in a[5]:
        for x, y in zip(a[5][t], b[5][t]):
            assert np.array_equal(x, y), t
    assert a[6] < b[6]  # fewer launches with the fused stages


@pytest.mark.parametrize("name,tend", [("flux_hydro_2d", 3.0), ("cap_morpho_2d", 1.0), ("window", 5.0)])
def test_fp32_dry_skip_matches_full_blocks(name, tend):
    """The FP32 form skips the reconstruction, flux and RHS work of a block whose cells and
    two-cell halo hold no water (kg_set_dry_skip, on by default) and carries its state
    forward.  The full computation of such a block changes it only by round-off of the dry
    bed, so both runs take the same accepted and refused steps, activate the same tiles and
    end within 1e-8 of the largest depth (w, Hn) and 1e-6 of the largest momentum of each
    other; the FP32 error bounds against the oracle above hold with the skip on."""
    if name == "window":
        from kestrel_gb300 import workloads
        p, b0 = workloads.morpho_flux_window(tend=tend)
    else:
        p, b0 = cases.ref_input(name, tend=tend, nout=1), None
    L = lib.load()
    runs = []
    for skip in (1, 0):
        s = fp32(p, b0=b0)
        assert L.kg_set_dry_skip(s.h, skip) == abi.KG_OK
        st = s.run()
        runs.append((st.steps, st.rejected, s.active_tiles(), s.ghost_tiles(),
                     {t: [s.field(t, f).copy() for f in (1, 2, 3, 5)] for t in s.active_tiles()}))
        s.close()
    a, b = runs
    assert a[:4] == b[:4], (a[:2], b[:2])
    depth = max(float(np.max(np.abs(v[3]))) for v in b[4].values())
    mom = max(max(float(np.max(np.abs(v[1]))), float(np.max(np.abs(v[2])))) for v in b[4].values())
    for t in a[4]:
        x, y = a[4][t], b[4][t]
        assert np.max(np.abs(x[0] - y[0])) <= 1e-8 * depth, t
        assert np.max(np.abs(x[3] - y[3])) <= 1e-8 * depth, t
        assert np.max(np.abs(x[1] - y[1])) <= 1e-6 * mom and np.max(np.abs(x[2] - y[2])) <= 1e-6 * mom, t
