"""GB300-native engine for the per-pseudo-iteration hot path of kwonhwi1/3dcode.

The package holds the CUDA sources (csrc/), the in-tree build (build.py), the ctypes
binding of the C ABI plus the host solve loop (native.py), the descriptor structs
(abi.py), the reference's input.inp reader (config.py) and the synthetic case
generator (cases.py).
"""
from . import abi, cases  # noqa: F401
