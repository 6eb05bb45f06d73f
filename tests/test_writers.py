"""The reference's text outputs (src/Output.f90) written from read-back state: exact column
layout and Fortran edit descriptors, and a round trip through the restart reader's parse
(src/Restart.f90:151-328).  Runs on the oracle (no GPU); the GPU test compares the
library's files with the oracle's byte for byte on a bit-exact case."""
import os

import numpy as np
import pytest

import _oracle
import cases
from kestrel_gb300 import lib, writers


def test_fortran_edit_descriptors():
    assert writers.fortran_es(1234.5, 18, 10, 3) == " 1.2345000000E+003"
    assert writers.fortran_es(-0.000123, 18, 10, 3) == "-1.2300000000E-004"
    assert writers.fortran_es(0.0, 18, 10, 3) == " 0.0000000000E+000"
    assert writers.fortran_es(1.0, 24, 15) == "   1.000000000000000E+00"
    assert writers.fortran_es(1e-120, 24, 15) == "   1.000000000000000-120"
    assert len(writers.fortran_es(3.5e7, 24, 15)) == 24


def test_outputs_layout_and_round_trip(tmp_path):
    p = cases.ref_input("cap_dilute_2d", tend=1.0, nout=2)
    sim = _oracle.simulation(p)
    writers.run_with_output(sim, str(tmp_path))
    names = sorted(os.listdir(tmp_path))
    assert names == ["000000.txt", "000000.txt_topo", "000001.txt", "000001.txt_topo", "000002.txt",
                     "000002.txt_topo", "Maximums.txt", "Volume.txt"]
    vol = open(tmp_path / "Volume.txt").read().splitlines()
    assert len(vol) == 4 and vol[0].startswith("        time,                   volume")
    assert all(len(r) == 12 + 6 * 26 for r in vol[1:])
    snap = open(tmp_path / "000002.txt").read().splitlines()
    assert len(snap[1]) == 8 + 18 * 20 and snap[1 + p.nXpertile] == ""
    cells, topo = writers.read_snapshot(str(tmp_path / "000002.txt"), p.nXpertile, p.nYpertile)
    assert sorted(cells) == sim.active_tiles()
    for t in sim.active_tiles():
        for name, f in (("w", 1), ("x_flux", 2), ("y_flux", 3), ("Hnpsi", 4), ("flow_depth", 5)):
            a, b = cells[t][name], sim.field(t, f)
            assert np.allclose(a, b, rtol=1e-10, atol=1e-300), (t, name)
        assert np.allclose(topo[t][1], sim.vertex(t, 1), rtol=1e-10, atol=1e-300)
    mx = open(tmp_path / "Maximums.txt").read().splitlines()
    assert len(mx[1]) == 8 + 15 * 20


@pytest.mark.gpu
def test_gpu_outputs_match_oracle_byte_for_byte(tmp_path):
    p = cases.ref_input("cap_dilute_2d", tend=1.0, nout=2)
    writers.run_with_output(lib.simulation(p), str(tmp_path / "gpu"))
    writers.run_with_output(_oracle.simulation(p), str(tmp_path / "oracle"))
    for name in os.listdir(tmp_path / "oracle"):
        assert open(tmp_path / "gpu" / name).read() == open(tmp_path / "oracle" / name).read(), name


@pytest.mark.gpu
@pytest.mark.parametrize("name,tend", [("cap_dilute_2d", 1.0), ("cap_morpho_2d", 0.5)])
def test_restart_from_snapshot(tmp_path, name, tend):
    """Restart from the text snapshot at the midpoint: the restored state equals the saved
    one to the file's 10 significant digits, and continuing to t_end stays within 1e-5 of the
    uninterrupted run (the snapshot's rounding is the only difference)."""
    p = cases.ref_input(name, tend=tend, nout=2)
    a = lib.simulation(p)
    writers.run_with_output(a, str(tmp_path))
    mid = p.tstart + 0.5 * (p.tend - p.tstart)
    b = writers.restart_from_snapshot(None, p, str(tmp_path / "000001.txt"), mid)
    cells, topo = writers.read_snapshot(str(tmp_path / "000001.txt"), p.nXpertile, p.nYpertile)
    assert b.active_tiles() == sorted(cells)
    for t in b.active_tiles():
        assert np.array_equal(b.field(t, 1), cells[t]["w"])
        assert np.array_equal(b.vertex(t, 1), topo[t][1])
    b.integrate_to(p.tend)
    assert b.time[0] == a.time[0]
    for t in a.active_tiles():
        depth = max(np.max(np.abs(a.field(u, 5))) for u in a.active_tiles())
        assert np.max(np.abs(b.field(t, 1) - a.field(t, 1))) <= 1e-5 * depth, t


@pytest.mark.parametrize("name,tend", [("cap_morpho_2d", 1.0), ("flux_hydro_2d", 2.0)])
def test_oracle_restart_full_precision(name, tend):
    """LoadInitialCondition in the oracle (ko_load_state): restarting at the midpoint from
    the exact state restores every field but the velocities (which the reference keeps
    from the last RHS and the restart recomputes), the same ghost tiles, and continues to
    t_end bit for bit with the uninterrupted run."""
    p = cases.ref_input(name, tend=tend, nout=2)
    a = _oracle.simulation(p)
    a.integrate_to(0.5 * tend)
    ids = a.active_tiles()
    state = np.stack([np.stack([a.field(t, f) for f in (1, 2, 3, 4)]) for t in ids])
    b = _oracle.simulation(p, load_sources=False)
    b.load_state(ids, state, np.stack([a.vertex(t, 1) for t in ids]), a.time[0])
    assert b.active_tiles() == ids and sorted(b.ghost_tiles()) == sorted(a.ghost_tiles())
    for t in ids:
        for f in (1, 2, 3, 4, 5, 8, 9, 10, 11, 12, 13):
            assert np.array_equal(a.field(t, f), b.field(t, f)), (t, f)
    a.integrate_to(tend)
    b.integrate_to(tend)
    assert a.active_tiles() == b.active_tiles() and a.time == b.time
    for t in a.active_tiles():
        for f in (1, 2, 3, 4, 11):
            assert np.array_equal(a.field(t, f), b.field(t, f)), (t, f)


def test_oracle_restart_from_snapshot(tmp_path):
    """The text snapshot round trip through the oracle: the restored w equals the file's
    10-digit values and the continued run stays within 1e-5 of the uninterrupted one."""
    p = cases.ref_input("cap_morpho_2d", tend=0.5, nout=2)
    a = _oracle.simulation(p)
    writers.run_with_output(a, str(tmp_path))
    mid = p.tstart + 0.5 * (p.tend - p.tstart)
    b = writers.restart_from_snapshot(_oracle.load(), p, str(tmp_path / "000001.txt"), mid, prefix="ko")
    cells, topo = writers.read_snapshot(str(tmp_path / "000001.txt"), p.nXpertile, p.nYpertile)
    assert b.active_tiles() == sorted(cells)
    for t in b.active_tiles():
        assert np.array_equal(b.field(t, 1), cells[t]["w"])
        assert np.array_equal(b.vertex(t, 1), topo[t][1])
    b.integrate_to(p.tend)
    depth = max(np.max(np.abs(a.field(u, 5))) for u in a.active_tiles())
    for t in a.active_tiles():
        assert np.max(np.abs(b.field(t, 1) - a.field(t, 1))) <= 1e-5 * depth, t
