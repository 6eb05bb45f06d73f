"""The batched ensemble form: members of different sizes, tile shapes and settings
advanced together, their hydraulic passes in one persistent launch.  Each member must
end exactly where the same input ends when run alone in the FP32 form (the batch changes
only how the work is launched, not its arithmetic), including members that join late
and members whose neighbours leave."""
import numpy as np
import pytest

import cases
from kestrel_gb300 import abi, lib
from kestrel_gb300.batch import Batch

pytestmark = pytest.mark.gpu


def snapshot(sim):
    return sim.time, {t: [sim.field(t, f).copy() for f in (1, 2, 3, 4, 11)] for t in sim.active_tiles()}


def alone(p):
    s = lib.simulation(p, precision=abi.PREC_FP32)
    s.run()
    out = snapshot(s)
    s.close()
    return out


def same(a, b):
    assert a[0] == b[0], (a[0], b[0])
    assert a[1].keys() == b[1].keys()
    for t in a[1]:
        for x, y in zip(a[1][t], b[1][t]):
            assert np.array_equal(x, y), t


INPUTS = [
    lambda: cases.ref_input("flux_hydro_2d", tend=2.0, nout=1),
    lambda: cases.ref_input("cap_morpho_2d", tend=0.5, nout=1),
    lambda: cases.ref_input("flux_edwards2019_2d", tend=2.0, nout=2),
    lambda: cases.cap_release_256(tend=1.0, nout=1),
    lambda: cases.ref_input("flux_morpho_2d", tend=2.0, nout=1),
    lambda: cases.ref_input("cap_dilute_2d", tend=1.0, nout=1),
]


def test_batch_members_match_alone():
    ps = [f() for f in INPUTS]
    ref = [alone(p) for p in ps]
    b = Batch(8)
    ids = [b.add(p) for p in ps]
    b.run()
    for k, i in enumerate(ids):
        assert b.finished(i)
        same(snapshot(b.member(i)), ref[k])
    launches, rounds = b.stats()
    assert launches > 0 and rounds > 0
    b.close()


def test_batch_graphs_on_and_off_identical():
    """The rounds replayed through CUDA graphs (the default) and launched directly on the
    stream give bit-identical members; with graphs on, every segment ran as a graph, and
    after the first of each kind the graphs were updated in place or launched unchanged."""
    ps = [f() for f in INPUTS]
    out = {}
    for graphs in (True, False):
        b = Batch(8, graphs=graphs)
        ids = [b.add(p) for p in ps]
        b.run()
        out[graphs] = [snapshot(b.member(i)) for i in ids]
        gl, gu, gi, gr = b.graph_stats()
        _, rounds = b.stats()
        if graphs:
            assert gl >= rounds and gl == gu + gi + gr and gu + gr > gi > 0, (gl, gu, gi, gr, rounds)
        else:
            assert gl == 0
        b.close()
    for x, y in zip(out[True], out[False]):
        same(x, y)


def test_batch_late_join_and_leave():
    ps = [f() for f in INPUTS[:3]]
    ref = [alone(p) for p in ps]
    b = Batch(4)
    a0 = b.add(ps[0])
    a1 = b.add(ps[1])
    for _ in range(3):
        b.step()
    b.remove(a1)              # a member leaves mid-run
    a2 = b.add(ps[2])         # another joins into the freed slot
    b.run()
    same(snapshot(b.member(a0)), ref[0])
    same(snapshot(b.member(a2)), ref[2])
    b.close()


def test_served_requests_same_alone_and_mixed():
    """Continuous batching: requests arriving together overlap on the device, are admitted
    as memory frees up (a budget that fits two at a time), and each result equals the same
    request served alone."""
    from kestrel_gb300 import serve, workloads
    reqs = []
    for k, (side, tend) in enumerate([(256, 6.0), (256, 4.0), (256, 3.0), (256, 5.0)]):
        p, b0, d = workloads.ensemble_member(900 + k, side=side, tend=tend)
        reqs.append(serve.Request(arrival=0.0, params=p, b0=b0, desc=d))
    budget = 2.05 * serve.worst_case_bytes(reqs[0].params)  # equal sides and tiles: two fit
    srv = serve.Server(hbm_budget=budget, max_members=4)
    rep = srv.run(reqs)
    srv.close()
    assert rep["peak_members"] == 2 and rep["requests"] == 4, rep
    for r in reqs:
        solo = serve.Server(hbm_budget=budget, max_members=1)
        one = serve.Request(arrival=0.0, params=r.params, b0=r.b0)
        solo.run([one])
        solo.close()
        a, b = r.result, one.result
        assert a["time"] == b["time"] and a["steps"] == b["steps"] and a["rejected"] == b["rejected"]
        assert np.array_equal(a["volume"], b["volume"])
        assert a["state"].keys() == b["state"].keys()
        for t in a["state"]:
            assert np.array_equal(a["state"][t], b["state"][t])
