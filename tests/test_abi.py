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
