"""Input-file parser: the reference's keyword=value format, keys and defaults.

Mirrors src/Input.f90:127-365 (block structure), src/DomainSettings.f90,
src/Parameters.f90, src/SolverSettings.f90, src/InitConds.f90, src/TopogSettings.f90 and
src/OutputSettings.f90 (N out), and fills the kg_params POD struct of
include/kestrel_gpu.h.  Keys are matched case-insensitively in the Domain, Parameters,
Solver, Output and Topog blocks and case-sensitively in Source/Cap/Cube blocks, as the
reference does; unknown keys are ignored with a warning list, as the reference only warns
(src/Messages.f90:299-304).
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

from . import abi

BLOCKS = ("Domain", "Source", "Cap", "Cube", "Parameters", "Solver", "Topog", "Output")


class InputError(ValueError):
    """Raised where the reference calls FatalErrorMessage while reading input."""


@dataclass
class ParsedInput:
    params: abi.Params
    warnings: list = field(default_factory=list)
    output: dict = field(default_factory=dict)
    topog: dict = field(default_factory=dict)  # raster inputs: type, raster file, dem directory


def _list(v: str):
    v = v.strip()
    if v.startswith("(") and v.endswith(")"):
        v = v[1:-1]
    return [float(x) for x in v.split(",") if x.strip() != ""]


def _real(v: str) -> float:
    v = v.strip()
    if v.startswith("(") and v.endswith(")"):
        v = v[1:-1]
    return float(v.replace("d", "e").replace("D", "e"))


def read_blocks(text: str):
    """Split the input text into blocks of (key, value) pairs, in file order."""
    blocks = []  # list of (name, [(key, value)])
    cur = None
    for raw in text.splitlines():
        line = raw.strip()
        if "#" in line:
            line = line[: line.index("#")].strip()
        if not line or line.startswith("%%"):
            continue
        if "=" in line:
            if cur is None:
                continue
            k, v = line.split("=", 1)
            cur[1].append((k.strip(), v.strip()))
        elif ":" in line:
            name = line.split(":", 1)[0].strip()
            if name in BLOCKS:
                cur = (name, [])
                blocks.append(cur)
            else:
                cur = None
    return blocks


def default_params() -> abi.Params:
    """kg_params with every default of the reference applied."""
    p = abi.Params()
    # Domain (src/DomainSettings.f90:38; 'halt' boundaries)
    p.bcs = abi.BCS["halt"]
    # Parameters (src/Parameters.f90:41-77)
    p.geometric_factors = 1
    p.g = 9.81
    p.rhow, p.rhos = 1000.0, 2000.0
    p.ChezyCo, p.ManningCo, p.CoulombCo = 0.01, 0.03, 0.1
    p.PouliquenMinSlope, p.PouliquenMaxSlope = 0.1, 0.4
    p.PouliquenIntermediateSlope, p.PouliquenBeta = 0.2, 0.136
    p.Edwards2019betastar, p.Edwards2019kappa, p.Edwards2019Gamma = 0.136, 1.0, 0.0
    p.VoellmySwitchRate, p.VoellmySwitchValue = 3.0, 0.2
    p.EroRate, p.EroRateGranular, p.EroDepth, p.EroCriticalHeight = 0.001, 4.0, 1.0, 0.01
    p.BedPorosity, p.maxPack, p.SolidDiameter, p.EddyViscosity = 0.35, 0.65, 1e-3, 0.0
    p.drag = abi.DRAG["chezy"]
    p.erosion = abi.EROSION["mixed"]
    p.MorphodynamicsOn = 1
    p.deposition = abi.DEPOSITION["spearman manning"]
    p.erosion_transition = abi.ETRANS["smooth"]
    p.morpho_damping = abi.DAMP["tanh"]
    p.fswitch = abi.SWITCH["tanh"]
    # Solver (src/SolverSettings.f90:42-51)
    p.limiter = abi.LIMITER["minmod2"]
    p.heightThreshold = 1e-6
    p.TileBuffer = 1
    p.cfl = 0.25
    p.maxdt = 1.7976931348623157e308
    p.tstart = 0.0
    p.SpongeStrength = 0.2
    p.Nout = 100
    p.topog = abi.TOPO["flat"]
    return p


def parse(text: str) -> ParsedInput:
    """Parse an input file's text into kg_params (2D runs)."""
    p = default_params()
    topo = {}
    warn = []
    out = {}
    blocks = read_blocks(text)
    have = {b[0] for b in blocks}
    if "Domain" not in have:
        raise InputError("Required block 'Domain' not found")
    xt = yt = None
    caps, cubes, srcs = [], [], []
    for name, kv in blocks:
        if name == "Domain":
            for k, v in kv:
                key = k.lower()
                if key == "nxtiles":
                    p.nXtiles = int(_real(v))
                elif key == "nytiles":
                    p.nYtiles = int(_real(v))
                elif key == "nxpertile":
                    p.nXpertile = int(_real(v))
                elif key == "nypertile":
                    p.nYpertile = int(_real(v))
                elif key == "xtilesize":
                    if yt is None:
                        xt = _real(v)
                elif key == "ytilesize":
                    if xt is None:
                        yt = _real(v)
                elif key == "boundary conditions":
                    bc = v.strip().lower()
                    if bc not in abi.BCS:
                        raise InputError(f"unrecognised boundary condition {v!r}")
                    p.bcs = abi.BCS[bc]
                elif key == "boundary hn":
                    p.bcsHnval = _real(v)
                elif key == "boundary u":
                    p.bcsuval = _real(v)
                elif key == "boundary v":
                    p.bcsvval = _real(v)
                elif key == "boundary psi":
                    p.bcspsival = _real(v)
                elif key in ("lat", "latitude", "lon", "longitude"):
                    pass
                else:
                    warn.append(f"Domain: unrecognised {k}")
        elif name == "Cap":
            caps.append(dict(kv))
        elif name == "Cube":
            cubes.append(dict(kv))
        elif name == "Source":
            srcs.append(dict(kv))
        elif name == "Parameters":
            _params_block(p, kv, warn)
        elif name == "Solver":
            _solver_block(p, kv, warn)
        elif name == "Topog":
            topo = _topog_block(p, kv, warn)
        elif name == "Output":
            for k, v in kv:
                out[k.lower()] = v
                if k.lower() == "n out":
                    p.Nout = int(_real(v))
                    if p.Nout < 1:
                        raise InputError("N out must be >= 1")
    # Tile sizes (src/DomainSettings.f90:185-196)
    if xt is not None:
        p.Xtilesize = xt
        p.Ytilesize = xt * float(p.nYpertile) / float(p.nXpertile)
    elif yt is not None:
        p.Ytilesize = yt
        p.Xtilesize = yt * float(p.nXpertile) / float(p.nYpertile)
    else:
        raise InputError("Xtilesize or Ytilesize is required")
    _caps(p, caps, warn)
    _cubes(p, cubes, warn)
    _sources(p, srcs, warn)
    return ParsedInput(params=p, warnings=warn, output=out, topog=topo)


def _params_block(p, kv, warn):
    set_ = set()
    for k, v in kv:
        key = k.lower()
        lv = v.strip().lower()
        set_.add(key)
        if key == "switch function":
            p.fswitch = abi.SWITCH.get(lv, abi.SWITCH["tanh"])
        elif key == "deposition":
            p.deposition = abi.DEPOSITION.get(lv, abi.DEPOSITION["spearman manning"])
        elif key == "morphodynamic damping":
            p.morpho_damping = abi.DAMP.get(lv, abi.DAMP["tanh"])
        elif key in ("iverson", "geometric factors"):
            p.geometric_factors = 0 if lv == "off" else 1
        elif key == "g":
            p.g = _real(v)
        elif key == "drag":
            if lv not in abi.DRAG:
                raise InputError(f"Drag value {v!r} is not recognised")
            p.drag = abi.DRAG[lv]
        elif key == "chezy co":
            p.ChezyCo = _real(v)
        elif key == "manning co":
            p.ManningCo = _real(v)
        elif key == "coulomb co":
            p.CoulombCo = _real(v)
        elif key == "pouliquen min":
            p.PouliquenMinSlope = _real(v)
        elif key == "pouliquen max":
            p.PouliquenMaxSlope = _real(v)
        elif key == "pouliquen intermediate":
            p.PouliquenIntermediateSlope = _real(v)
        elif key == "pouliquen beta":
            p.PouliquenBeta = _real(v)
        elif key == "edwards2019 betastar":
            p.Edwards2019betastar = _real(v)
        elif key == "edwards2019 kappa":
            p.Edwards2019kappa = _real(v)
        elif key == "edwards2019 gamma":
            p.Edwards2019Gamma = _real(v)
        elif key == "voellmy switch rate":
            p.VoellmySwitchRate = _real(v)
        elif key == "voellmy switch value":
            p.VoellmySwitchValue = _real(v)
        elif key == "erosion":
            if lv not in abi.EROSION:
                raise InputError(f"Erosion value {v!r} is not recognised")
            p.erosion = abi.EROSION[lv]
            p.MorphodynamicsOn = 0 if lv == "off" else 1
        elif key == "erosion rate":
            p.EroRate = _real(v)
        elif key == "granular erosion rate":
            p.EroRateGranular = _real(v)
        elif key == "erosion depth":
            p.EroDepth = _real(v)
        elif key == "erosion transition":
            p.erosion_transition = abi.ETRANS.get(lv, abi.ETRANS["smooth"])
        elif key == "erosion critical height":
            p.EroCriticalHeight = _real(v)
        elif key == "bed porosity":
            p.BedPorosity = _real(v)
        elif key == "rhow":
            p.rhow = _real(v)
        elif key == "rhos":
            p.rhos = _real(v)
        elif key in ("maxpack", "max pack"):
            p.maxPack = _real(v)
        elif key == "solid diameter":
            p.SolidDiameter = _real(v)
        elif key == "eddy viscosity":
            p.EddyViscosity = _real(v)
        elif key == "settling speed":
            p.ws0 = _real(v)
            p.ws0_given = 1
        else:
            warn.append(f"Parameters: unrecognised {k}")
    # Positivity checks the reference enforces (src/Parameters.f90 FatalError_Positive)
    for attr in ("g", "ChezyCo", "ManningCo", "CoulombCo", "rhow", "rhos", "SolidDiameter", "maxPack"):
        if getattr(p, attr) <= 0:
            raise InputError(f"{attr} must be positive")
    if not (0.0 <= p.BedPorosity < 1.0):
        raise InputError("Bed Porosity must be in [0, 1)")


def _solver_block(p, kv, warn):
    for k, v in kv:
        key = k.lower()
        if key == "t end":
            p.tend = _real(v)
        elif key == "limiter":
            p.limiter = abi.LIMITER.get(v.strip().lower(), abi.LIMITER["minmod2"])
        elif key == "height threshold":
            p.heightThreshold = _real(v)
        elif key == "tile buffer":
            p.TileBuffer = int(_real(v))
        elif key == "cfl":
            p.cfl = _real(v)
        elif key == "max dt":
            p.maxdt = _real(v)
        elif key == "t start":
            p.tstart = _real(v)
        elif key == "sponge strength":
            p.SpongeStrength = _real(v)
        elif key in ("restart", "initial condition"):
            if key == "restart" and v.strip().lower() == "on":
                warn.append("Solver: Restart is outside the hot path and is ignored")
        else:
            warn.append(f"Solver: unrecognised {k}")
    if p.tend <= p.tstart:
        raise InputError("T end must exceed T start")
    if p.cfl <= 0 or p.heightThreshold <= 0 or p.maxdt <= 0:
        raise InputError("cfl, Height threshold and max dt must be positive")


def _topog_block(p, kv, warn):
    """Topog block (src/TopogSettings.f90:88-140).  'Raster'/'DEM' selects the raster
    topography (the file is read by kestrel_gb300.dem and passed to kg_upload_raster);
    'SRTM' needs the SRTM tile mosaic built through GDAL and PROJ and is refused."""
    typ = None
    extra = {}
    for k, v in kv:
        key = k.lower()
        if key == "type":
            typ = v.strip().lower()
            extra["type"] = typ
        elif key in ("raster file", "dem directory", "embed raster", "rebuild dem"):
            extra[key] = v.strip()
        elif key == "topog function":
            name = v.strip().lower()
            if name not in abi.TOPO_NPARAMS:
                raise InputError(f"the 'Topog function = {v.strip()}' is not recognized")
            p.topog = abi.TOPO[name]
        elif key == "topog params":
            vals = _list(v)
            p.n_topog_params = len(vals)
            for i, x in enumerate(vals[: abi.MAX_TOPO_PARAMS]):
                p.topog_params[i] = x
        else:
            warn.append(f"Topog: unrecognised {k}")
    if typ in (None, "function"):
        name = next((n for n, v in abi.TOPO.items() if v == p.topog), None)
        need = abi.TOPO_NPARAMS.get(name, 0)
        if p.n_topog_params < need:
            words = {1: "one", 2: "two", 3: "three", 6: "six"}
            raise InputError(f"{words.get(need, need)} 'Topog params' are needed for 'Topog function = {name}'; "
                             f"received {p.n_topog_params}")
    if typ in ("dem", "raster"):
        p.topog = abi.TOPO["raster"]
    elif typ == "srtm":
        raise InputError("SRTM topography needs the SRTM mosaic built through GDAL and PROJ, which are not available")
    elif typ not in (None, "function"):
        raise InputError(f"Topog type {typ!r} is not recognised")
    return extra


def _cap_shape(v):
    s = v.strip().lower()
    return abi.SHAPE.get(s, abi.SHAPE["para"])


def _caps(p, caps, warn):
    """Cap_Set, src/InitConds.f90:254-425."""
    if len(caps) > abi.MAX_CAPS:
        raise InputError("too many caps")
    p.nCaps = len(caps)
    for k, d in enumerate(caps):
        c = p.caps[k]
        c.x = c.y = c.radius = c.height = c.psi = c.u = c.v = 0.0
        c.shape = abi.SHAPE["para"]
        has = lambda key: key in d
        if has("capX"):
            c.x = _real(d["capX"])
        if has("capY"):
            c.y = _real(d["capY"])
        set_r = set_h = set_v = False
        vol = 0.0
        if has("capRadius"):
            c.radius = _real(d["capRadius"]); set_r = True
        if has("capHeight") and not (set_v and set_r):
            c.height = _real(d["capHeight"]); set_h = True
        if has("capVolume") and not (set_r and set_h):
            vol = _real(d["capVolume"]); set_v = True
        if has("capU"):
            c.u = _real(d["capU"])
        if has("capV"):
            c.v = _real(d["capV"])
        if has("capConc"):
            c.psi = _real(d["capConc"])
        if has("capShape"):
            c.shape = _cap_shape(d["capShape"])
        pi = math.pi
        if set_r and set_v:
            if c.shape == abi.SHAPE["flat"]:
                c.height = vol / pi / c.radius / c.radius
            elif c.shape == abi.SHAPE["para"]:
                c.height = 2.0 * vol / pi / c.radius / c.radius
        if set_h and set_v and not set_r:
            if c.shape == abi.SHAPE["flat"]:
                c.radius = math.sqrt(vol / pi / c.height)
            elif c.shape == abi.SHAPE["para"]:
                c.radius = math.sqrt(2.0 * vol / pi / c.height)


def _cubes(p, cubes, warn):
    """Cube_Set, src/InitConds.f90:430-660."""
    if len(cubes) > abi.MAX_CUBES:
        raise InputError("too many cubes")
    p.nCubes = len(cubes)
    for k, d in enumerate(cubes):
        c = p.cubes[k]
        c.x = c.y = c.length = c.width = c.height = c.psi = c.u = c.v = 0.0
        c.shape = abi.SHAPE["flat"]
        for key, attr in (("cubeX", "x"), ("cubeY", "y"), ("cubeLength", "length"),
                          ("cubeWidth", "width"), ("cubeHeight", "height"), ("cubeConc", "psi"),
                          ("cubeU", "u"), ("cubeV", "v")):
            if key in d:
                setattr(c, attr, _real(d[key]))
        if "cubeShape" in d:
            s = d["cubeShape"].strip().lower()
            c.shape = abi.SHAPE["level"] if s == "level" else abi.SHAPE["flat"]


def _sources(p, srcs, warn):
    """Source_Set, src/InitConds.f90:45-220."""
    if len(srcs) > abi.MAX_SOURCES:
        raise InputError("too many sources")
    p.nSources = len(srcs)
    for k, d in enumerate(srcs):
        s = p.sources[k]
        for need in ("sourceX", "sourceY", "sourceRadius", "sourceTime", "sourceFlux", "sourceConc"):
            if need not in d:
                raise InputError(f"Source {k + 1}: {need} is required")
        s.x = _real(d["sourceX"])
        s.y = _real(d["sourceY"])
        s.radius = _real(d["sourceRadius"])
        t, q, c = _list(d["sourceTime"]), _list(d["sourceFlux"]), _list(d["sourceConc"])
        if not (len(t) == len(q) == len(c)):
            raise InputError("sourceTime, sourceFlux and sourceConc must have equal lengths")
        if len(t) > abi.MAX_SERIES:
            raise InputError("flux series too long")
        s.n_series = len(t)
        for i in range(len(t)):
            s.time[i], s.flux[i], s.psi[i] = t[i], q[i], c[i]


def parse_file(path: str) -> ParsedInput:
    with open(path) as f:
        return parse(f.read())
