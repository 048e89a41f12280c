"""asgkron: GB300-native operator application y = A*f for the ASGarD sparse-grid DG prototype.

The compute path is libasgkron.so (hand-written CUDA for sm_103a behind the C ABI in
include/asgkron.h).  This package is the host-side mirror of the reference's MATLAB
interface: element tables and connectivity (grid), apply_A / Plan (api), the 1-D operator
builder (operators, pdes).
"""
from . import _build
from ._lib import AsgError, lib
from .api import DEFAULT_DROP_TOL, Plan, apply_A, clear_plan_cache
from .grid import (ElementTable, connect_nD, connectivity_cells, element_idx1d, global_matrix, hash_table_nD,
                   hash_table_sparse_nD)

__all__ = [
    "AsgError", "lib", "Plan", "apply_A", "clear_plan_cache", "DEFAULT_DROP_TOL", "ElementTable",
    "hash_table_sparse_nD", "hash_table_nD", "element_idx1d", "global_matrix", "connect_nD",
    "connectivity_cells", "build",
]


def build(force=False, verbose=False):
    """Compile libasgkron.so for sm_103a (in-tree) and return its path."""
    return _build.build(force=force, verbose=verbose)
