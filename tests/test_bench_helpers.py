"""The bench's host logic (no GPU): the committed ncu summaries carry the per-cell figures
the bench line reads, the two rooflines are the stated ratios, a spin-up keeps its wall-time
limit and reports how far it got, and a secondary figure that fails, crashes or runs out of
time becomes an error entry instead of losing the bench line."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
import bench  # noqa: E402


@pytest.mark.parametrize("kernel,workload", [("k_hydro32", "morpho_flux_2048_fp32"), ("k_hydro", "morpho_flux_2048_fp64")])
def test_profiles_carry_the_figures_the_bench_reads(kernel, workload):
    for key in ("dram_bytes_per_cell_pass", "fp64_pipe_cycles_per_cell_pass"):
        v = bench.profile_figure(kernel, workload, key)
        assert v is not None and v > 0, (kernel, key)


def test_roofline_arithmetic():
    # traffic: bytes per cell and pass x cells
    per = bench.profile_figure("k_hydro32", "morpho_flux_2048_fp32", "dram_bytes_per_cell_pass")
    assert bench.profile_traffic("k_hydro32", "morpho_flux_2048_fp32", 1000.0) == per * 1000.0
    # FP64 pipe: cycles per cell x cells / pass time, over SMs x clock
    r = bench.fp64_pipe_roofline("k_hydro32", "morpho_flux_2048_fp32", 152 * 2000.0, 1.0, 2000.0, 152)
    cyc = bench.profile_figure("k_hydro32", "morpho_flux_2048_fp32", "fp64_pipe_cycles_per_cell_pass")
    assert r["bound"] == "fp64_pipe" and r["frac"] == pytest.approx(cyc * 152 * 2000.0 / 1e-3 / (152 * 2000e6))
    assert bench.fp64_pipe_roofline("k_hydro32", "no_such_workload", 1.0, 1.0, 2000.0, 152) is None
    assert bench.fp64_pipe_roofline("k_hydro32", "morpho_flux_2048_fp32", 1.0, 0.0, 2000.0, 152) is None


def test_peaks_are_read_or_fall_back():
    peak, kind = bench.measured_peaks()
    assert peak > 1000.0 and kind in ("measured", "fallback")
    assert bench.measured_sm_max_mhz() > 1000.0
    assert set(bench.ALG_BYTES) == {"fp64_hydro", "fp64_morpho", "fp32_hydro", "fp32_morpho"}


class _FakeSim:
    """Advances simulated time by `dt` per step, sleeping `wall` seconds per step."""

    def __init__(self, dt, wall=0.0, tiles=3):
        self.t, self.dt, self.wall, self.n = 0.0, dt, wall, tiles

    @property
    def time(self):
        return self.t, self.dt

    def step(self, t_stop):
        import time as _t
        if self.wall:
            _t.sleep(self.wall)
        self.t = min(t_stop, self.t + self.dt)

    def integrate_to(self, t):
        self.t = t

    def active_tiles(self):
        return list(range(self.n))


class _P:
    nXtiles = nYtiles = 10


def test_spin_up_records_the_timeline_and_keeps_its_deadline():
    out = bench.spin_up(_FakeSim(dt=5.0), _P, 40.0, every=20.0, deadline_s=10.0)
    assert [row[0] for row in out] == [20.0, 40.0] and out[0][1:] == [3, 3.0]
    with pytest.raises(TimeoutError) as e:
        bench.spin_up(_FakeSim(dt=1e-3, wall=0.01), _P, 40.0, every=20.0, deadline_s=0.2)
    assert e.value.timeline and e.value.timeline[-1][0] < 20.0  # where it stood when time ran out


def test_a_failing_extra_is_an_error_entry_not_a_lost_line(monkeypatch):
    import argparse
    import subprocess

    class R:
        def __init__(self, rc, out, err):
            self.returncode, self.stdout, self.stderr = rc, out, err

    args = argparse.Namespace(sparse_window=200.0, members=256, requests=24, rate=20.0, tend_min=60.0, tend_max=600.0,
                              budget_gb=150.0, serve_tend_scale=0.1, batch_graphs=1, serve_graphs=0)
    monkeypatch.setattr(subprocess, "run", lambda *a, **k: R(-11, "", "Fatal Python error: Segmentation fault\n"))
    got = bench.run_extra("serve_fp32", args)
    assert got["error"] == "exit code -11" and "Segmentation" in got["stderr_tail"]
    monkeypatch.setattr(subprocess, "run", lambda *a, **k: R(0, 'noise\n{"value": 1.5}\n', ""))
    assert bench.run_extra("serve_fp32", args) == {"value": 1.5}

    def slow(*a, **k):
        raise subprocess.TimeoutExpired(a[0], k.get("timeout"))
    monkeypatch.setattr(subprocess, "run", slow)
    assert "no result" in bench.run_extra("ensemble_fp32", args, timeout_s=1.0)["error"]
