"""velvet_gb300 — GB300-native XPBD cloth solver behind Velvet's solver surface.

The product is libvelvet_gb300.so (CUDA for sm_103a + C++ host code, C ABI in
include/velvet_gb300.h).  This package holds its build recipe, a ctypes binding
(`ClothSolver`, `BatchSolver`, `ClothServer`) and the synthetic workloads the tests and
the benchmark use.  Nothing here computes physics on the CPU: if the library is absent,
every call raises.
"""
from ._abi import VtError, VtParams, VtSdfCollider, default_params, lib  # noqa: F401
from .solver import (GRID_VARIANTS, BatchSolver, ClothServer, ClothSolver, colmajor,  # noqa: F401
                     grid_variant_name, hash_objects, render_params, rgba_to_rgb, stream_handle, write_ppm)

__all__ = [
    "BatchSolver", "ClothServer", "ClothSolver", "VtError", "VtParams", "VtSdfCollider", "default_params", "lib",
    "colmajor", "hash_objects", "stream_handle", "GRID_VARIANTS", "grid_variant_name",
]
