"""The C ABI: header <-> ctypes mirror <-> exported symbols (no GPU needed)."""
import ctypes as C
import os
import re

import pytest

from kestrel_gb300 import abi, build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "kestrel_gpu.h")


def header_functions():
    txt = open(HEADER).read()
    return sorted(set(re.findall(r"\b(kg_[a-z0-9_]+)\s*\(", txt)))


def test_header_declares_the_api():
    names = header_functions()
    for n in ("kg_create", "kg_destroy", "kg_step", "kg_integrate_to", "kg_run", "kg_hydraulic_rhs",
              "kg_load_sources", "kg_upload_b0", "kg_volume", "kg_get_tile_field"):
        assert n in names


def test_library_exports_every_header_symbol():
    path = build.build()
    lib = C.CDLL(path)
    missing = [n for n in header_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_struct_sizes_match_c():
    # kg_params layout: compile a tiny C program against the header and compare sizeof.
    import subprocess, tempfile
    src = r'''
#include <stdio.h>
#include <stddef.h>
#include "kestrel_gpu.h"
int main(void){printf("%zu %zu %zu %zu %zu %zu %zu %zu %zu\n", sizeof(kg_params), sizeof(kg_cap), sizeof(kg_cube),
 sizeof(kg_flux_source), sizeof(kg_step_stats), offsetof(kg_params, sources), offsetof(kg_params, topog_params),
 sizeof(kg_raster), offsetof(kg_raster, center_n));return 0;}
'''
    with tempfile.TemporaryDirectory() as d:
        cpath, exe = os.path.join(d, "t.c"), os.path.join(d, "t")
        open(cpath, "w").write(src)
        subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), cpath, "-o", exe], check=True)
        out = subprocess.run([exe], capture_output=True, text=True, check=True).stdout.split()
    got = [int(x) for x in out]
    want = [C.sizeof(abi.Params), C.sizeof(abi.Cap), C.sizeof(abi.Cube), C.sizeof(abi.FluxSource),
            C.sizeof(abi.StepStats), abi.Params.sources.offset, abi.Params.topog_params.offset,
            C.sizeof(abi.Raster), abi.Raster.center_n.offset]
    assert got == want


def test_create_without_gpu_fails_loudly():
    """With no GPU there is no silent CPU fallback: kg_create reports KG_ERR_CUDA."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from kestrel_gb300 import lib
    import cases
    L = lib.load()
    h = C.c_void_p()
    rc = L.kg_create(C.byref(cases.cap_release_256()), abi.PREC_FP64, C.byref(h))
    assert rc == -5 and not h.value


def _bad_params():
    """One caller error per case, each on a copy of a valid struct: (what, mutate, code)."""
    def setf(name, value):
        return lambda p: setattr(p, name, value)

    def series(p):
        p.nSources = 1
        p.sources[0].n_series = 0

    return [
        ("zero tiles", setf("nXtiles", 0), "KG_ERR_PARAM"),
        ("one cell per tile row", setf("nXpertile", 1), "KG_ERR_PARAM"),
        ("1D grid", lambda p: (setattr(p, "nYtiles", 1), setattr(p, "nYpertile", 1)), "KG_ERR_UNSUPPORTED"),
        ("too many tiles", lambda p: (setattr(p, "nXtiles", 1 << 16), setattr(p, "nYtiles", 1 << 15)), "KG_ERR_PARAM"),
        ("negative tile size", setf("Xtilesize", -16.0), "KG_ERR_PARAM"),
        ("NaN tile size", setf("Ytilesize", float("nan")), "KG_ERR_PARAM"),
        ("zero cfl", setf("cfl", 0.0), "KG_ERR_PARAM"),
        ("zero height threshold", setf("heightThreshold", 0.0), "KG_ERR_PARAM"),
        ("NaN maxdt", setf("maxdt", float("nan")), "KG_ERR_PARAM"),
        ("negative TileBuffer", setf("TileBuffer", -1), "KG_ERR_PARAM"),
        ("17 caps", setf("nCaps", 17), "KG_ERR_PARAM"),
        ("negative sources", setf("nSources", -1), "KG_ERR_PARAM"),
        ("empty flux series", series, "KG_ERR_PARAM"),
        ("drag id", setf("drag", 7), "KG_ERR_PARAM"),
        ("erosion id", setf("erosion", -1), "KG_ERR_PARAM"),
        ("limiter id", setf("limiter", 5), "KG_ERR_PARAM"),
        ("boundary id", setf("bcs", 4), "KG_ERR_PARAM"),
        ("topography id", setf("topog", 19), "KG_ERR_PARAM"),
        ("switch id", setf("fswitch", 8), "KG_ERR_PARAM"),
    ]


@pytest.mark.parametrize("what,mutate,code", _bad_params(), ids=[c[0] for c in _bad_params()])
def test_create_rejects_bad_params_before_the_device(what, mutate, code):
    """A struct outside what the kernels index and branch on is refused by kg_create before
    any device call (so the same status comes back on a machine without a GPU), with the
    reason in kg_last_error(NULL); the oracle's C entry gives the same status and reason."""
    import _oracle
    from kestrel_gb300 import lib
    import cases
    p = cases.cap_release_256()
    mutate(p)
    L, O = lib.load(), _oracle.load()
    h = C.c_void_p()
    rc = L.kg_create(C.byref(p), abi.PREC_FP64, C.byref(h))
    assert abi.KG_ERR.get(rc) == code and not h.value
    msg = L.kg_last_error(None).decode()
    assert msg
    ho = C.c_void_p()
    rco = O.ko_create(C.byref(p), C.byref(ho))
    assert rco == rc and not ho.value
    assert O.ko_last_error(None).decode() == msg


def test_create_error_reaches_the_python_mirror():
    from kestrel_gb300 import lib
    from kestrel_gb300.solver import KestrelError
    import cases
    p = cases.cap_release_256()
    p.cfl = -1.0
    with pytest.raises(KestrelError, match="cfl, heightThreshold and maxdt must be positive") as ei:
        lib.simulation(p)
    assert abi.KG_ERR[ei.value.code] == "KG_ERR_PARAM"


def test_create_rejects_an_unknown_precision():
    from kestrel_gb300 import lib
    import cases
    L = lib.load()
    h = C.c_void_p()
    assert abi.KG_ERR[L.kg_create(C.byref(cases.cap_release_256()), 7, C.byref(h))] == "KG_ERR_UNSUPPORTED"
    assert b"precision" in L.kg_last_error(None)


def _header_prototypes():
    """(return type, name, [parameter types]) of every function the header declares."""
    txt = open(HEADER).read()
    out = []
    for m in re.finditer(r"^(const char\*|void\*|void|int64_t|int|kg_ctx\*)\s+(kg_[a-z0-9_]+)\(([^)]*)\);", txt, re.M):
        params = [a.strip() for a in m.group(3).split(",")] if m.group(3).strip() != "void" else []
        types = [re.sub(r"\s*\b[a-z_0-9]+(\[\d+\])?$", lambda q: "*" if q.group(1) else "", a).strip() for a in params]
        out.append((m.group(1), m.group(2), types))
    return out


def test_every_entry_point_refuses_a_null_handle():
    """Every function that takes a context or batch handle returns KG_ERR_PARAM (or NULL / 0
    for the non-status getters, nothing for the destructors) when the handle is NULL, with
    every other argument zero or NULL: the library never dereferences a caller's NULL."""
    L = C.CDLL(build.build())  # its own function objects: the shared declarations stay as they are
    protos = [p for p in _header_prototypes() if p[2] and p[2][0].replace("const ", "") in ("kg_ctx*", "kg_batch*")]
    assert len(protos) >= 35
    for ret, name, types in protos:
        f = getattr(L, name)
        args = []
        for t in types:
            if "*" in t:
                args.append(C.c_void_p(None))
            elif t == "double":
                args.append(C.c_double(0.0))
            elif t == "int64_t":
                args.append(C.c_int64(0))
            else:
                args.append(C.c_int32(0))
        f.argtypes = [type(a) for a in args]
        f.restype = {"int": C.c_int, "int64_t": C.c_int64, "void": None, "const char*": C.c_char_p,
                     "void*": C.c_void_p, "kg_ctx*": C.c_void_p}[ret]
        got = f(*args)
        if ret == "int":
            assert abi.KG_ERR.get(got) == "KG_ERR_PARAM", (name, got)
        elif ret in ("int64_t",):
            assert got == 0, name
        elif ret in ("void*", "kg_ctx*"):
            assert got is None, name


@pytest.mark.parametrize("nx,ny", [(64, 64), (50, 50), (16, 8)])
def test_slot_bytes_follow_the_layout(nx, ny):
    """kg_slot_bytes (host arithmetic, no device) counts every per-slot array of the HBM
    layout, and the serving loop's admission uses that count."""
    from kestrel_gb300 import lib, serve
    L = lib.load()
    SC, SFX, SFY, SV, nE = nx * ny, (nx + 1) * ny, nx * (ny + 1), (nx + 1) * (ny + 1), max(nx, ny)
    doubles = (4 * 4 * SC                                   # Q: 4 buffers of w, rhoHnu, rhoHnv, Hnpsi
               + 2 * (4 * SC + SC)                          # E, I: two RHS sets
               + 2 * (4 * SC + 5 * SFX + 5 * SFY + 2 * SV)  # CT, FX, FY, BV: two topography sets
               + 2 * SC + 5 * SC + SC + 2 * SC              # UV, MS, EMD, B0S
               + 9 * SC + 12 * nE + 11 * SC                 # G9, GE, MX
               + 2 * SC)                                    # source-override Hn and rho
    ints = 8 + 1                                            # nbr[8], tile_of_slot
    fp32 = (2 * (3 * SC * 8 + 6 * SC * 4 + 2 * (SFX + SFY) * 4)  # TD, TF, TFX, TFY: two sets
            + 3 * SC * 8 + 14 * SC * 4                           # M0, MF: the M attempt's step start and stage
            + SV * 8)                                            # BVA: the second copy of the vertex bt
    base = 8 * doubles + 4 * ints + 2                       # + kind, has_source bytes
    assert L.kg_slot_bytes(nx, ny, abi.PREC_FP64) == base
    assert L.kg_slot_bytes(nx, ny, abi.PREC_FP32) == base + fp32
    assert serve.slot_bytes(nx, ny) == base + fp32
    assert L.kg_slot_bytes(0, ny, abi.PREC_FP64) == 0 and L.kg_slot_bytes(nx, ny, 9) == 0


def _fortran_type_fields(text, name):
    """[(field, fortran type)] of `type, bind(C) :: name` in a Fortran listing."""
    m = re.search(r"type, bind\(C\) :: " + name + r"\b[^\n]*\n(.*?)\n\s*end type", text, re.S)
    assert m, name
    out = []
    for line in m.group(1).splitlines():
        line = line.split("!")[0].strip()
        if not line:
            continue
        ftype, names = [x.strip() for x in line.split("::")]
        for n in re.findall(r"[A-Za-z_0-9]+(?:\(\d+\))?", names):
            out.append((n, ftype))
    return out


@pytest.mark.parametrize("name,cls", [("kg_params", "Params"), ("kg_cap", "Cap"), ("kg_cube", "Cube"),
                                      ("kg_flux_source", "FluxSource"), ("kg_raster", "Raster"),
                                      ("kg_step_stats", "StepStats")])
def test_fortran_binding_matches_the_structs(name, cls):
    """The bind(C) derived types of the Fortran binding list every field of the C struct, in
    order, with the same kind and array bound (padding fields without their underscore)."""
    text = open(os.path.join(ROOT, "include", "kestrel_gpu.f90")).read()
    got = _fortran_type_fields(text, name)
    kinds = {C.c_double: "real(c_double)", C.c_int32: "integer(c_int32_t)", C.c_int64: "integer(c_int64_t)"}
    subtypes = {abi.Cap: "type(kg_cap)", abi.Cube: "type(kg_cube)", abi.FluxSource: "type(kg_flux_source)"}
    want = []
    for fname, ft in getattr(abi, cls)._fields_:
        if hasattr(ft, "_length_"):
            base = ft._type_
            want.append((f"{fname.lstrip('_')}({ft._length_})", subtypes.get(base) or kinds[base]))
        else:
            want.append((fname.lstrip("_"), kinds[ft]))
    assert got == want


def test_fortran_interfaces_match_the_header():
    """Every bind(C) interface of the Fortran binding names a header function and takes its
    number of arguments; value arguments are the header's scalars, the rest its pointers."""
    text = open(os.path.join(ROOT, "include", "kestrel_gpu.f90")).read()
    protos = {n: types for _, n, types in _header_prototypes()}
    blocks = re.findall(r"(?:function|subroutine) (kg_[a-z0-9_]+)\(([^)]*)\) bind\(C, name=\"(kg_[a-z0-9_]+)\"\)(.*?)end (?:function|subroutine)",
                        text, re.S)
    assert len(blocks) >= 20
    for fname, args, cname, body in blocks:
        assert fname == cname and cname in protos, cname
        names = [a.strip() for a in args.split(",") if a.strip()]
        types = protos[cname]
        assert len(names) == len(types), cname
        for a, t in zip(names, types):
            decl = re.search(r"^\s*([^!\n]*)::[^!\n]*\b" + a + r"\b", body, re.M)
            assert decl, (cname, a)
            attrs = decl.group(1)
            if "*" in t:  # a pointer: by reference, or an explicit c_ptr passed by value
                assert "value" not in attrs or "type(c_ptr)" in attrs, (cname, a, t)
            else:         # a scalar: by value
                assert "value" in attrs and "type(c_ptr)" not in attrs, (cname, a, t)


def test_fortran_dropin_keeps_the_reference_interfaces():
    """The drop-in module offers Run, IntegrateTo and CalculateHydraulicRHS with the
    reference's argument lists (src/TimeStepper.f90:73,116, src/HydraulicRHS.f90:64-73) and
    binds only functions the header declares; every entry point it calls is interfaced in
    the binding module."""
    text = open(os.path.join(ROOT, "include", "kestrel_gpu_dropin.f90")).read()
    binding = open(os.path.join(ROOT, "include", "kestrel_gpu.f90")).read()
    for sig in ("subroutine Run(RunParams, grid)", "subroutine IntegrateTo(RunParams, tend, grid)",
                "subroutine CalculateHydraulicRHS(RunParams, grid, tileWorkspace, t, substep, advisedTimeStep)"):
        assert sig in text, sig
    header = {n for _, n, _ in _header_prototypes()}
    bound = set(re.findall(r'bind\(C, name="(kg_[a-z0-9_]+)"\)', binding))
    assert bound <= header, bound - header
    called = set(re.findall(r"\b(kg_[a-z0-9_]+)\(", text)) - {"kg_check", "kg_params", "kg_raster", "kg_step_stats"}
    assert called <= bound, called - bound
    # every statement block the module opens is closed (comments left out)
    lines = [line.split("!")[0].strip().lower() for line in text.splitlines()]
    for kw in ("module", "subroutine", "function"):
        closed = sum(1 for line in lines if re.match(r"end " + kw + r"\b", line))
        opened = sum(1 for line in lines if not line.startswith("end") and re.match(r"(?:[a-z()_0-9, ]*\s)?" + kw + r"\s+[a-z_]", line))
        assert opened == closed, (kw, opened, closed)
