"""Copies the reference's own test input files used by the parity tests into
tests/golden/inputs/ (the GPU test machine has no copy of the reference tree).

Run from the repository root with the reference checked out at REF (default
/root/reference):  python tests/golden/make_inputs.py [REF]
"""
import os
import shutil
import sys

NAMES = ["cap_dilute_2d", "cap_conc_2d", "cap_morpho_2d", "flat_depositional_2d", "flux_edwards2019_2d",
         "flux_hydro_2d", "flux_morpho_2d", "flux_single_pt", "lake_at_rest_hydro_2d", "lake_at_rest_morpho_2d",
         "tile_indep_static_100m", "tile_indep_static_50m", "tile_indep_dynamic_100m", "tile_indep_dynamic_20m"]
# The 1D inputs of the reference's suite (tests/runall.jl tests_1d, tests_noflow): 1D grids
# are outside the implemented path, and the tests check that they are refused cleanly.
NAMES_1D = ["flat_depositional", "cap_dilute", "cap_conc", "cap_morpho", "flux_hydro", "flux_edwards2019", "flux_morpho",
            "lake_at_rest_hydro", "lake_at_rest_morpho"]


def main(ref):
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "inputs")
    os.makedirs(out, exist_ok=True)
    for n in NAMES + NAMES_1D:
        shutil.copyfile(os.path.join(ref, "tests", f"Input_{n}.txt"), os.path.join(out, f"Input_{n}.txt"))
    print(f"copied {len(NAMES) + len(NAMES_1D)} input files to {out}")


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
