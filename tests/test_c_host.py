"""The C ABI driven from a C program (tests/c_host/kg_host.c), the way a non-Python host
binds it: without a GPU kg_create refuses (KG_ERR_CUDA) instead of computing on the host;
on a GPU the C host's run of the reference's cap_dilute_2d input matches the same run
driven through the Python mirror, bit for bit."""
import ctypes as C
import os
import subprocess

import pytest

import cases
from kestrel_gb300 import abi, build, lib

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def host_binary(tmp_path):
    so = build.build()
    exe = str(tmp_path / "kg_host")
    subprocess.run(["gcc", "-O2", "-std=c99", "-I", os.path.join(ROOT, "include"), os.path.join(HERE, "c_host", "kg_host.c"),
                    "-o", exe, "-L", os.path.dirname(so), "-l:" + os.path.basename(so),
                    "-Wl,-rpath," + os.path.dirname(so)], check=True)
    return exe


def run_host(tmp_path, p, precision=abi.PREC_FP64, lines=False):
    path = str(tmp_path / "params.bin")
    with open(path, "wb") as f:
        f.write(bytes(p))
    out = subprocess.run([host_binary(tmp_path), path, str(precision)], capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stdout + out.stderr
    return out.stdout.splitlines() if lines else out.stdout.split()


def test_c_host_without_gpu(tmp_path):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    out = run_host(tmp_path, cases.ref_input("cap_dilute_2d", tend=0.5, nout=1), lines=True)
    cuda_err = next(k for k, v in abi.KG_ERR.items() if v == "KG_ERR_CUDA")
    assert out == [f"create {cuda_err}", "no CUDA device is available"]


def test_c_host_bad_struct(tmp_path):
    """A struct the library refuses gives the same status and reason to a C host, on any
    machine (the check comes before the device)."""
    p = cases.ref_input("cap_dilute_2d", tend=0.5, nout=1)
    p.limiter = 99
    out = run_host(tmp_path, p, lines=True)
    param_err = next(k for k, v in abi.KG_ERR.items() if v == "KG_ERR_PARAM")
    assert out == [f"create {param_err}", "a closure, limiter, boundary or topography selector is out of range"]


@pytest.mark.gpu
def test_c_host_matches_python(tmp_path):
    p = cases.ref_input("cap_dilute_2d", tend=1.0, nout=1)
    words = run_host(tmp_path, p)
    assert words[0] == "ok", words
    sim = lib.simulation(p)
    st = sim.integrate_to(p.tend)
    vol = sim.volume()
    sw = 0.0
    for t in sim.active_tiles():
        for x in sim.field(t, 1).reshape(-1):
            sw += float(x)
    assert float(words[1]) == st.t and int(words[2]) == st.steps and int(words[3]) == st.rejected
    assert int(words[4]) == len(sim.active_tiles())
    assert [float(x) for x in words[5:9]] == list(vol)
    assert float(words[9]) == sw and float(words[10]) == sw
