"""GB300-native comoving-radiation step of PyBlastAfterglowMag.

The compute path is libpbag.so (include/pbag.h): hand-written sm_103a CUDA
kernels behind a C ABI. This package holds its Python binding (_lib, abi),
the in-tree build (build) and a synthetic-history generator (histories).
"""
from . import abi  # noqa: F401
from ._lib import Context, PbagError, grids, load, shock_limits  # noqa: F401

__all__ = ["abi", "Context", "PbagError", "grids", "load", "shock_limits"]
