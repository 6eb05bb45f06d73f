"""ctypes mirror of include/kestrel_gpu.h (the drop-in C ABI).

The structures here must stay byte-identical to the header; ``tests/test_abi.py`` checks
sizes and the exported symbol list of the built library against the header.
"""
import ctypes as C

KG_OK = 0
KG_ERR = {
    -1: "KG_ERR_PARAM", -2: "KG_ERR_OOM", -3: "KG_ERR_HALT_EDGE", -4: "KG_ERR_NAN",
    -5: "KG_ERR_CUDA", -6: "KG_ERR_UNSUPPORTED", -7: "KG_ERR_STATE", -8: "KG_ERR_DT",
    -9: "KG_ERR_NOT_FOUND", -10: "KG_ERR_TIMEOUT",
}

DRAG = {"chezy": 0, "coulomb": 1, "voellmy": 2, "pouliquen": 3, "edwards2019": 4,
        "variable": 5, "manning": 6}
EROSION = {"off": 0, "mixed": 1, "on": 1, "simple": 2, "fluid": 3, "granular": 4}
DEPOSITION = {"none": 0, "simple": 1, "spearman manning": 2}
ETRANS = {"smooth": 0, "step": 1, "off": 2}
DAMP = {"none": 0, "off": 0, "tanh": 1, "rat3": 2}
SWITCH = {"tanh": 0, "rat3": 1, "cos": 2, "linear": 3, "equal": 4, "0.5": 4, "off": 5,
          "0": 5, "zero": 5, "1": 6, "one": 6, "step": 7}
LIMITER = {"minmod1": 0, "minmod2": 1, "van albada": 2, "albada": 2, "weno": 3, "none": 4}
BCS = {"halt": 0, "periodic": 1, "dirichlet": 2, "sponge": 3}
TOPO = {"upload": 0, "flat": 1, "xslope": 2, "yslope": 3, "xyslope": 4, "xsinslope": 5,
        "xysinslope": 6, "xhump": 7, "xtanh": 8, "xparab": 9, "xyparab": 10, "raster": 11,
        "x2slopes": 12, "usgs": 13, "flume": 14, "channel power law": 15, "channel trapezium": 16,
        "xbislope": 17, "xtrislope": 18}
# Topog params each analytic surface needs (src/TopogSettings.f90:202-345).
TOPO_NPARAMS = {"flat": 0, "xslope": 1, "yslope": 1, "xyslope": 2, "x2slopes": 3, "usgs": 2, "flume": 6,
                "channel power law": 3, "channel trapezium": 3, "xbislope": 3, "xtrislope": 6, "xsinslope": 1,
                "xysinslope": 1, "xhump": 2, "xtanh": 3, "xparab": 1, "xyparab": 2}
SHAPE = {"flat": 0, "para": 1, "parabolic": 1, "level": 2}
PREC_FP64, PREC_FP32 = 0, 1

MAX_CAPS = MAX_CUBES = MAX_SOURCES = 16
MAX_SERIES = 64
MAX_TOPO_PARAMS = 8


class Cap(C.Structure):
    _fields_ = [(n, C.c_double) for n in ("x", "y", "radius", "height", "psi", "u", "v")] + [
        ("shape", C.c_int32), ("_pad", C.c_int32)]


class Cube(C.Structure):
    _fields_ = [(n, C.c_double) for n in ("x", "y", "length", "width", "height", "psi", "u", "v")] + [
        ("shape", C.c_int32), ("_pad", C.c_int32)]


class FluxSource(C.Structure):
    _fields_ = [("x", C.c_double), ("y", C.c_double), ("radius", C.c_double),
                ("n_series", C.c_int32), ("_pad", C.c_int32),
                ("time", C.c_double * MAX_SERIES), ("flux", C.c_double * MAX_SERIES),
                ("psi", C.c_double * MAX_SERIES)]


def _d(*names):
    return [(n, C.c_double) for n in names]


def _i(*names):
    return [(n, C.c_int32) for n in names]


class Params(C.Structure):
    _fields_ = (
        _i("nXtiles", "nYtiles", "nXpertile", "nYpertile") + _d("Xtilesize", "Ytilesize")
        + _i("bcs", "_pad0") + _d("bcsHnval", "bcsuval", "bcsvval", "bcspsival")
        + _i("geometric_factors", "MorphodynamicsOn") + _d("g", "rhow", "rhos")
        + _d("ChezyCo", "ManningCo", "CoulombCo")
        + _d("PouliquenMinSlope", "PouliquenMaxSlope", "PouliquenIntermediateSlope", "PouliquenBeta")
        + _d("Edwards2019betastar", "Edwards2019kappa", "Edwards2019Gamma")
        + _d("VoellmySwitchRate", "VoellmySwitchValue")
        + _d("EroRate", "EroRateGranular", "EroDepth", "EroCriticalHeight", "BedPorosity")
        + _d("maxPack", "SolidDiameter", "EddyViscosity")
        + _i("ws0_given", "_pad1") + _d("ws0")
        + _i("drag", "erosion", "deposition", "erosion_transition", "morpho_damping", "fswitch")
        + _i("limiter", "TileBuffer")
        + _d("heightThreshold", "cfl", "maxdt", "tstart", "tend", "SpongeStrength")
        + _i("Nout", "_pad2")
        + _i("nCaps", "nCubes", "nSources", "_pad3")
        + [("caps", Cap * MAX_CAPS), ("cubes", Cube * MAX_CUBES), ("sources", FluxSource * MAX_SOURCES)]
        + _i("topog", "n_topog_params") + [("topog_params", C.c_double * MAX_TOPO_PARAMS)]
    )


class StepStats(C.Structure):
    _fields_ = [("t", C.c_double), ("dt", C.c_double), ("steps", C.c_int64),
                ("rejected", C.c_int64), ("cell_updates", C.c_int64),
                ("n_active", C.c_int32), ("n_ghost", C.c_int32),
                ("kernel_launches", C.c_int64)]


class Raster(C.Structure):
    """kg_raster: georeferencing of an elevation raster (north-up GDAL geotransform)."""
    _fields_ = [("nx", C.c_int64), ("ny", C.c_int64)] + [
        (n, C.c_double) for n in ("origin_x", "origin_y", "pixel_w", "pixel_h", "nodata", "center_e", "center_n")]


def declare(lib, prefix):
    """Attach argtypes/restype for the kg_-style API under ``prefix`` ('kg' or 'ko')."""
    P = C.POINTER
    vp = C.c_void_p
    sig = {
        "create": ([P(Params), C.c_int32, P(vp)] if prefix == "kg" else [P(Params), P(vp)], C.c_int),
        "destroy": ([vp], None),
        "last_error": ([vp], C.c_char_p),
        "upload_b0": ([vp, P(C.c_double), C.c_int64, C.c_int64], C.c_int),
        "upload_raster": ([vp, P(C.c_double), P(Raster)], C.c_int),
        "load_sources": ([vp], C.c_int),
        "step": ([vp, C.c_double, P(StepStats)], C.c_int),
        "integrate_to": ([vp, C.c_double, P(StepStats)], C.c_int),
        "run": ([vp, P(StepStats)], C.c_int),
        "hydraulic_rhs": ([vp, C.c_double, C.c_int32, P(C.c_double)], C.c_int),
        "get_active_tiles": ([vp, P(C.c_int32), P(C.c_int32)], C.c_int),
        "get_ghost_tiles": ([vp, P(C.c_int32), P(C.c_int32)], C.c_int),
        "get_tile_field": ([vp, C.c_int32, C.c_int32, P(C.c_double)], C.c_int),
        "get_state": ([vp, P(C.c_int32), P(C.c_int32), P(C.c_double), P(C.c_double)], C.c_int),
        "set_tile_field": ([vp, C.c_int32, C.c_int32, P(C.c_double)], C.c_int),
        "get_tile_vertex": ([vp, C.c_int32, C.c_int32, P(C.c_double)], C.c_int),
        "get_tile_rhs": ([vp, C.c_int32, C.c_int32, P(C.c_double)], C.c_int),
        "get_tile_maxima": ([vp, C.c_int32, C.c_int32, P(C.c_double)], C.c_int),
        "volume": ([vp, P(C.c_double)], C.c_int),
        "get_time": ([vp, P(C.c_double), P(C.c_double)], C.c_int),
        "redistribution_stats": ([vp, P(C.c_int64), P(C.c_int64), P(C.c_int64)], C.c_int),
    }
    for name, (args, res) in sig.items():
        f = getattr(lib, f"{prefix}_{name}")
        f.argtypes = args
        f.restype = res
    return lib
