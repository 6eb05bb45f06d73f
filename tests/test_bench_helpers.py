"""The bench's roofline inputs (no GPU): the committed ncu summaries carry the per-cell
figures the bench line reads, and the two rooflines are the stated ratios."""
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
