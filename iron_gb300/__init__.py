"""iron_gb300 -- GB300-native finite-element assembly engine for OpenCMISS-Iron's element-loop hot path.

The CUDA engine (libgfe.so, built from iron_gb300/csrc for sm_103a) is driven through a thin
C ABI (include/gfe.h).  This package is the host side: Iron-numbered generated meshes, the
device-resident assembly objects, and an Iron-shaped API (`iron_gb300.iron`).
"""
from ._lib import GfeError, GFE_FP64, GFE_MIXED, load as load_library  # noqa: F401

__version__ = "0.1.0"
