"""Element tables, 1-D index maps and connectivity through the C ABI.

Python mirror of hash_table_sparse_nD.m, hash_table_nD.m, global_matrix.m and connect_nD.m;
all computation happens in libasgkron (host C++), these wrappers only size the buffers.
"""
import ctypes as C

import numpy as np

from ._lib import ASG_GRID_FG, ASG_GRID_SG, check, lib


def _grid(grid_type):
    if grid_type in ("SG", ASG_GRID_SG):
        return ASG_GRID_SG
    if grid_type in ("FG", ASG_GRID_FG):
        return ASG_GRID_FG
    raise ValueError("grid_type must be 'SG' or 'FG'")


def _iptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_int))


class ElementTable:
    """hash_table.elements / elements_idx of the reference, as dense arrays.

    levels, cells: [N, d] int32; keys: uint64 md keys (0-based: md_lev_pos_to_idx - 1)."""

    def __init__(self, levels, cells, keys=None):
        self.levels = levels
        self.cells = cells
        self.keys = keys

    @property
    def num_elems(self):
        return self.levels.shape[0]

    @property
    def num_dims(self):
        return self.levels.shape[1]

    def idx1d(self):
        """1-based 1-D index per element and dimension (A_data.element_local_index_D)."""
        return element_idx1d(self.levels, self.cells)


def hash_table_sparse_nD(lev_vec, max_lev, grid_type="SG"):
    """Element table in hash_table_sparse_nD.m order (hash_table_sparse_nD.m:35-116)."""
    lv = np.ascontiguousarray(np.asarray(lev_vec, dtype=np.int32).reshape(-1))
    d = lv.size
    cnt = C.c_longlong(0)
    check(lib().asg_hash_table_sparse_nd(d, _iptr(lv), int(max_lev), _grid(grid_type), None, None, None, 0, C.byref(cnt)))
    n = cnt.value
    levels = np.zeros((n, d), dtype=np.int32)
    cells = np.zeros((n, d), dtype=np.int32)
    keys = np.zeros(n, dtype=np.uint64)
    check(lib().asg_hash_table_sparse_nd(d, _iptr(lv), int(max_lev), _grid(grid_type), _iptr(levels), _iptr(cells),
                                         keys.ctypes.data_as(C.POINTER(C.c_ulonglong)), n, C.byref(cnt)))
    return ElementTable(levels, cells, keys)


def hash_table_nD(lev, num_dims, grid_type="SG"):
    """Old-hash element order (hash_table_nD.m:29-136)."""
    cnt = C.c_longlong(0)
    check(lib().asg_hash_table_nd(int(num_dims), int(lev), _grid(grid_type), None, None, 0, C.byref(cnt)))
    n = cnt.value
    levels = np.zeros((n, num_dims), dtype=np.int32)
    cells = np.zeros((n, num_dims), dtype=np.int32)
    check(lib().asg_hash_table_nd(int(num_dims), int(lev), _grid(grid_type), _iptr(levels), _iptr(cells), n,
                                  C.byref(cnt)))
    return ElementTable(levels, cells)


def element_idx1d(levels, cells):
    levels = np.ascontiguousarray(levels, dtype=np.int32)
    cells = np.ascontiguousarray(cells, dtype=np.int32)
    out = np.zeros_like(levels)
    check(lib().asg_element_idx1d(levels.shape[1], levels.shape[0], _iptr(levels), _iptr(cells), _iptr(out)))
    return out


def global_matrix(table):
    """A_data of global_matrix.m:31-70: element_global_row_index (1-based) and
    element_local_index_D{d} (1-based 1-D indices)."""
    idx = table.idx1d()
    return {
        "element_global_row_index": np.arange(1, table.num_elems + 1),
        "element_local_index_D": [idx[:, d].copy() for d in range(table.num_dims)],
        "idx1d": idx,
    }


def connect_nD(table, levsum, levmax, grid_type="SG"):
    """CSR (row_ptr, cols 0-based, sorted per row) of connect_nD.m:34-105 for the table."""
    levels = np.ascontiguousarray(table.levels, dtype=np.int32)
    cells = np.ascontiguousarray(table.cells, dtype=np.int32)
    n, d = levels.shape
    npairs = C.c_longlong(0)
    check(lib().asg_connect_nd(d, n, _iptr(levels), _iptr(cells), int(levsum), int(levmax), _grid(grid_type), None,
                               None, 0, C.byref(npairs)))
    row_ptr = np.zeros(n + 1, dtype=np.int64)
    cols = np.zeros(max(1, npairs.value), dtype=np.int32)
    check(lib().asg_connect_nd(d, n, _iptr(levels), _iptr(cells), int(levsum), int(levmax), _grid(grid_type),
                               row_ptr.ctypes.data_as(C.POINTER(C.c_longlong)), _iptr(cols), npairs.value,
                               C.byref(npairs)))
    return row_ptr, cols[:npairs.value]


def connectivity_cells(row_ptr, cols):
    """The reference's pde.connectivity cell array: per element a sorted 1-based id list."""
    return [cols[row_ptr[i]:row_ptr[i + 1]].astype(np.int64) + 1 for i in range(len(row_ptr) - 1)]
