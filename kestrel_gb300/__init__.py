"""kestrel_gb300 -- GB300-native (sm_103a CUDA) implementation of Kestrel's time-step hot path.

The product is the C-ABI shared library built from ``kestrel_gb300/csrc`` (declared in
``include/kestrel_gpu.h``); this package holds the host-side pieces around it: the
input-file parser (``config``), the ctypes binding (``abi``, ``lib``) and the
Run/IntegrateTo mirror (``solver``).
"""
from . import abi, config  # noqa: F401

__all__ = ["abi", "config"]
