"""GPU parity of every erosion, deposition, transition, damping and switch closure.

Each case runs the reference's cap_morpho_2d input (Variable drag, which blends Chezy and
Pouliquen by the switch function; morphodynamics on) with one closure selector changed, on
the sm_103a path through the C ABI and on the oracle, to t = 1 s.  Bar: equal accepted and
refused step counts, equal redistribution lists, and every field and the vertex bed within
1e-10 relative L-inf (CUDA's tanh/log/pow/cos differ from glibc's in the last bits) -- or,
where the reference's algorithm is itself sensitive to such last-bit differences, within
ten times the spread the oracle shows when its own closure transcendentals are moved by
one ulp (measured in the same test; the redistribution walk is ordered by FP64 excess
values, src/Redistribute.f90:69-475, so a last-bit change can reorder two interacting
cells: about 1e-3 for the rat3, cos, linear and equal switches on this input, round-off
for the others).

Closures (src/Closures.f90): erosion Fluid/Granular/Mixed/Simple (:566-675), deposition
None/Simple/Spearman-Manning (:320-356), erosion transitions smooth/step/off (:684-732),
morphodynamic damping none/tanh/rat3 (:744-791), switch functions (:797-915).
"""
import numpy as np
import pytest

import _oracle
import cases
from kestrel_gb300 import abi, lib
from test_gpu_parity import compare_state, rel_linf

pytestmark = pytest.mark.gpu

SELECTORS = {"erosion": abi.EROSION, "deposition": abi.DEPOSITION, "erosion_transition": abi.ETRANS,
             "morpho_damping": abi.DAMP, "fswitch": abi.SWITCH}

CASES = (
    # erosion laws on a clear-water cap (no deposition term, so the law alone moves the bed)
    [("erosion", v, dict(conc=0.0)) for v in ("fluid", "granular", "simple", "mixed")]
    + [("deposition", v, {}) for v in ("none", "simple", "spearman manning")]
    # a shallow erodible layer, so the transitions see bt reach -EroDepth
    + [("erosion_transition", v, dict(conc=0.0, EroDepth=2e-4)) for v in ("smooth", "step", "off")]
    + [("morpho_damping", v, {}) for v in ("none", "tanh", "rat3")]
    + [("fswitch", v, {}) for v in ("tanh", "rat3", "cos", "linear", "equal", "zero", "one", "step")]
)


@pytest.mark.parametrize("key,value,extra", CASES, ids=[f"{k}={v}" for k, v, _ in CASES])
def test_closure_parity(key, value, extra):
    p = cases.ref_input("cap_morpho_2d", tend=1.0, nout=1)
    setattr(p, key, SELECTORS[key][value])
    if "conc" in extra:
        p.caps[0].psi = extra["conc"]
    if "EroDepth" in extra:
        p.EroDepth = extra["EroDepth"]
    o, so, spread = _oracle.nudged_spread(p)
    tol = max(1e-10, 10.0 * spread)
    assert tol <= 5e-2, spread
    g = lib.simulation(p)
    sg = g.run()
    assert (sg.steps, sg.rejected) == (so.steps, so.rejected), (sg.steps, sg.rejected, so.steps, so.rejected)
    compare_state(g, o, tol=tol, what=f"{key}={value}")
    moved = 0.0
    for t in o.active_tiles():
        bo = o.vertex(t, 1)
        moved = max(moved, float(np.max(np.abs(bo))))
        assert rel_linf(g.vertex(t, 1), bo) <= tol or np.max(np.abs(bo)) == 0.0, t
        assert g.field(t, 11).min() >= -p.EroDepth
    cg, _, kg = g.redistribution_stats()
    co, _, ko = o.redistribution_stats()
    assert (cg, kg) == (co, ko), (cg, kg, co, ko)
    assert moved > 0.0, "the bed never moved: the closure was not exercised"
