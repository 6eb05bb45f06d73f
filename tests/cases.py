"""Shared test configurations.

Inputs come either from the reference's own test input files (copied as small fixtures
into tests/golden/inputs/, so that nothing reads the reference tree at run time) or from
synthetic configurations built in code with the reference's keys.
"""
import os

from kestrel_gb300 import abi, config

HERE = os.path.dirname(os.path.abspath(__file__))
INPUTS = os.path.join(HERE, "golden", "inputs")


def ref_input(name, tend=None, nout=None, **over):
    p = config.parse_file(os.path.join(INPUTS, f"Input_{name}.txt")).params
    if tend is not None:
        p.tend = tend
    if nout is not None:
        p.Nout = nout
    for k, v in over.items():
        setattr(p, k, v)
    return p


def cap_release_256(tend=30.0, nout=1):
    """The 256x256 plain FP64 cap release (kestrel_gb300.workloads)."""
    from kestrel_gb300 import workloads
    return workloads.cap_release_256(tend=tend, nout=nout)
