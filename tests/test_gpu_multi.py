"""Several simulations alive on one GPU at the same time.

Each context's run settings and source table are bound to the device before its kernels
run, so interleaving the steps of contexts with different inputs must leave every one of
them exactly where it would be alone.
"""
import numpy as np
import pytest

import cases
from kestrel_gb300 import abi, lib

pytestmark = pytest.mark.gpu


def state(sim):
    return {t: [sim.field(t, f).copy() for f in (1, 2, 3, 4, 11)] for t in sim.active_tiles()}


@pytest.mark.parametrize("prec", [abi.PREC_FP64, abi.PREC_FP32])
def test_interleaved_contexts_match_alone(prec):
    inputs = [cases.ref_input("flux_hydro_2d", tend=2.0, nout=1),
              cases.ref_input("cap_morpho_2d", tend=0.5, nout=1),
              cases.ref_input("flux_edwards2019_2d", tend=2.0, nout=1)]
    alone = []
    for p in inputs:
        s = lib.simulation(p, precision=prec)
        s.run()
        alone.append((s.time, state(s)))
        s.close()
    sims = [lib.simulation(p, precision=prec) for p in inputs]
    live = list(range(len(sims)))
    while live:
        for k in list(live):
            sims[k].step(inputs[k].tend)
            if sims[k].time[0] >= inputs[k].tend:
                live.remove(k)
    for k, s in enumerate(sims):
        assert s.time == alone[k][0]
        got = state(s)
        assert got.keys() == alone[k][1].keys()
        for t in got:
            for a, b in zip(got[t], alone[k][1][t]):
                assert np.array_equal(a, b), (k, t)
