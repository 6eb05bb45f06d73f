"""Input-file parsing: the reference's keys and defaults (src/*Settings.f90, Parameters.f90)."""
import math
import os

import pytest

from kestrel_gb300 import abi, config


def test_defaults_match_reference():
    p = config.default_params()
    assert p.limiter == abi.LIMITER["minmod2"] and p.heightThreshold == 1e-6 and p.TileBuffer == 1
    assert p.cfl == 0.25 and p.SpongeStrength == 0.2 and p.g == 9.81 and p.ChezyCo == 0.01
    assert p.ManningCo == 0.03 and p.CoulombCo == 0.1 and p.PouliquenBeta == 0.136
    assert p.maxPack == 0.65 and p.rhow == 1000 and p.rhos == 2000 and p.BedPorosity == 0.35
    assert p.SolidDiameter == 1e-3 and p.EddyViscosity == 0.0
    # Erosion defaults to Mixed and switches morphodynamics on (src/Parameters.f90:573-577).
    assert p.erosion == abi.EROSION["mixed"] and p.MorphodynamicsOn == 1


def test_parse_reference_input():
    import cases
    p = cases.ref_input("flux_hydro_2d")
    assert (p.nXtiles, p.nYtiles, p.nXpertile, p.nYpertile) == (40, 40, 50, 50)
    assert p.Xtilesize == 50 and p.Ytilesize == 50
    assert p.nSources == 1 and p.sources[0].n_series == 2 and p.sources[0].flux[1] == 10.0
    assert p.drag == abi.DRAG["chezy"] and p.MorphodynamicsOn == 0
    assert p.topog == abi.TOPO["xslope"] and p.topog_params[0] == -0.1


def test_cap_volume_relations():
    txt = """Domain:
nXtiles = 4
nYtiles = 4
nXpertile = 8
nYpertile = 8
Xtilesize = 8
Cap:
  capX = 0
  capY = 0
  capRadius = 2
  capVolume = 10
  capShape = para
Solver:
T end = 1
Topog:
Type = Function
Topog function = flat
"""
    p = config.parse(txt).params
    assert math.isclose(p.caps[0].height, 2.0 * 10 / math.pi / 2 / 2)


def test_rejects_unknown_drag():
    with pytest.raises(config.InputError):
        config.parse("Domain:\nnXtiles = 1\nnYtiles = 1\nnXpertile = 4\nnYpertile = 4\nXtilesize = 4\n"
                     "Parameters:\nDrag = Bogus\nSolver:\nT end = 1\n")


def _all_inputs():
    import glob
    import os
    import cases
    return sorted(os.path.basename(f)[len("Input_"):-len(".txt")] for f in glob.glob(os.path.join(cases.INPUTS, "Input_*.txt")))


def test_every_reference_input_parses_and_1d_grids_are_refused():
    """Every input file of the reference's suite parses. Unknown labels are skipped with a
    warning, as src/Messages.f90:299-304 does. The 2D inputs create an oracle context; the
    1D ones (nYtiles = nYpertile = 1) get KG_ERR_UNSUPPORTED from the oracle and from the
    GPU library, before any device call."""
    import ctypes as C
    import _oracle
    import cases
    from kestrel_gb300 import lib
    L, O = lib.load(), _oracle.load()
    names = _all_inputs()
    assert len(names) >= 23
    n1d = 0
    for name in names:
        p = cases.ref_input(name)
        one_d = p.nYtiles * p.nYpertile == 1
        n1d += one_d
        h = C.c_void_p()
        rc = O.ko_create(C.byref(p), C.byref(h))
        if one_d:
            assert abi.KG_ERR[rc] == "KG_ERR_UNSUPPORTED", name
            assert abi.KG_ERR[L.kg_create(C.byref(p), abi.PREC_FP64, C.byref(C.c_void_p()))] == "KG_ERR_UNSUPPORTED", name
        else:
            assert rc == abi.KG_OK, (name, O.ko_last_error(None))
            O.ko_destroy(h)
    assert n1d == 9


def test_reader_line_rules():
    """The reference's reader rules (src/Input.f90:91-123, :205-212): leading blanks
    ignored, '#' ends a line's content, lines starting with '%' or '#' are comments, a line
    with ':' names a block (text after the colon dropped); CRLF files read the same."""
    import cases
    base = open(os.path.join(cases.INPUTS, "Input_flux_hydro_2d.txt")).read()
    p0 = bytes(config.parse(base).params)
    variants = [
        base.replace("nXtiles = 40", "nXtiles = 40   # forty tiles").replace("Chezy Co = 0.04", "Chezy Co = 0.04 # drag"),
        "# header\n% another\n" + base.replace("Domain:", "# the domain\nDomain:"),
        base.replace("nXtiles = 40", "\t   nXtiles = 40").replace("Domain:", "   Domain:"),
        base.replace("Domain:", "Domain: the grid"),
        base.replace("\n", "\r\n"),
    ]
    for v in variants:
        assert bytes(config.parse(v).params) == p0
