"""CPU-side checks of the C ABI library: it loads, exports every declared symbol, and its
host-side index builders match the reference's gold files bit for bit."""
import ctypes as C
import os
import re

import numpy as np
import pytest

import asgkron
from asgkron import _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
G = os.path.join(ROOT, "tests", "golden")


def declared_symbols():
    hdrs = [os.path.join(ROOT, "include", f) for f in os.listdir(os.path.join(ROOT, "include")) if f.endswith(".h")]
    names = set()
    for h in hdrs:
        src = open(h).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        for m in re.finditer(r"\b(asg_[a-z0-9_]+)\s*\(", src):
            names.add(m.group(1))
    return sorted(names)


def test_library_exports_every_declared_symbol():
    L = asgkron.lib()
    names = declared_symbols()
    assert len(names) >= 15
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing
    # and the ctypes signature table covers them all
    assert set(names) <= set(_lib.SIGNATURES), set(names) - set(_lib.SIGNATURES)


def test_version_and_error_text():
    assert b"sm_103a" in asgkron.lib().asg_version()
    st = asgkron.lib().asg_plan_create(None, None)
    assert st == _lib.ASG_ERR_INVALID
    assert "NULL" in _lib.last_error()


def test_invalid_dims_rejected_without_gpu():
    d = _lib.PlanDesc()
    d.num_dims, d.deg, d.num_terms, d.num_elems = 7, 2, 1, 0
    h = C.c_void_p()
    assert asgkron.lib().asg_plan_create(C.byref(d), C.byref(h)) == _lib.ASG_ERR_UNSUPPORTED
    assert "nkron=7" in _lib.last_error()
    d.num_dims, d.deg = 6, 5  # 5^6 = 15625 > 4096
    assert asgkron.lib().asg_plan_create(C.byref(d), C.byref(h)) == _lib.ASG_ERR_UNSUPPORTED


@pytest.mark.parametrize("levels", [[7], [5, 2], [3, 2, 3]])
@pytest.mark.parametrize("grid", ["SG", "FG"])
def test_hash_table_sparse_nd_gold(levels, grid):
    e = np.load(os.path.join(G, "element_table.npz"))
    t = asgkron.hash_table_sparse_nD(levels, 7, grid)
    d = len(levels)
    np.testing.assert_array_equal(np.concatenate([t.levels, t.cells], axis=1),
                                  e["table_%dd_%s" % (d, grid)].astype(np.int32))
    np.testing.assert_array_equal(t.keys.astype(np.int64), e["ids_%dd_%s" % (d, grid)].ravel().astype(np.int64))


def test_idx1d_gold():
    e = np.load(os.path.join(G, "element_table.npz"))
    for k in e.files:
        if k.startswith("1d_index_"):
            lev, cell = (int(v) for v in k.split("_")[2:4])
            if lev > 30:
                continue
            got = asgkron.element_idx1d(np.array([[lev]]), np.array([[cell]]))
            assert int(got[0, 0]) == int(e[k].ravel()[0]), k


@pytest.mark.parametrize("d,lev,grid,levsum,levmax", [(2, 3, "FG", 6, 3), (3, 4, "SG", 4, 4)])
def test_connect_nd_gold(d, lev, grid, levsum, levmax):
    c = np.load(os.path.join(G, "connectivity.npz"))
    t = asgkron.hash_table_nD(lev, d, grid)
    rp, cols = asgkron.connect_nD(t, levsum, levmax, "SG")
    cells = asgkron.connectivity_cells(rp, cols)
    assert len(cells) == t.num_elems
    for i, row in enumerate(cells):
        np.testing.assert_array_equal(row, c["connect_n_%d_%d_%s_%d" % (d, lev, grid, i + 1)].ravel().astype(np.int64))


def test_connect_1d_via_nd_gold():
    """A 1-D element table with levsum=levmax=L reproduces connect_1D(L) row by row."""
    c = np.load(os.path.join(G, "connectivity.npz"))
    for L in (2, 3, 8):
        t = asgkron.hash_table_nD(L, 1, "SG")  # 1-D elements in 1-D index order
        rp, cols = asgkron.connect_nD(t, L, L)
        idx = t.idx1d()[:, 0] - 1
        dense = np.zeros((2 ** L, 2 ** L), dtype=np.int64)
        for i in range(t.num_elems):
            dense[idx[i], idx[cols[rp[i]:rp[i + 1]]]] = 1
        np.testing.assert_array_equal(dense, c["connect_1_%d" % L].astype(np.int64))


def test_global_matrix_idx_matches_definition():
    t = asgkron.hash_table_sparse_nD([4, 4], 8)
    A = asgkron.global_matrix(t)
    lev, cell = t.levels[:, 0], t.cells[:, 0]
    want = np.where(lev == 0, 1, 2 ** np.maximum(lev - 1, 0) + cell + 1)
    np.testing.assert_array_equal(A["element_local_index_D"][0], want)
    assert t.num_elems == 48  # continuity2 lev 4 (the CPU-runnable configuration)


C_CALLER = r"""
#include <stdio.h>
#include "asgkron.h"

int main(void) {
  double x[10], w[10], H0[16], G0[16], op[64];
  asg_partial_term div;
  double sx = 0, sw = 0, sh = 0, so = 0;
  int i;
  if (asg_gauss_legendre_f64(10, -1.0, 1.0, x, w) != ASG_OK) return 2;
  if (asg_multiwavelet_filters_f64(4, H0, G0) != ASG_OK) return 3;
  div.kind = 1; div.LF = -1.0; div.bcl = 'P'; div.bcr = 'P'; div.g_quad = NULL; div.g_face = NULL;
  if (asg_coeff_matrix_f64(2, 2, -1.0, 1.0, 1, &div, op) != ASG_OK) return 4;
  if (asg_coeff_matrix_f64(0, 2, -1.0, 1.0, 1, &div, op) != ASG_ERR_INVALID) return 5;
  for (i = 0; i < 10; ++i) { sx += x[i] * x[i]; sw += w[i]; }
  for (i = 0; i < 16; ++i) sh += H0[i] * H0[i] + G0[i] * G0[i];
  for (i = 0; i < 64; ++i) so += op[i] * (i + 1);
  printf("%.17g %.17g %.17g %.17g\n", sx, sw, sh, so);
  return 0;
}
"""


def test_c_caller_links_the_library(tmp_path):
    """A C99 program that includes only asgkron.h, links libasgkron.so and calls the host entry
    points gets the results the Python binding gets: the boundary is plain C."""
    import subprocess

    import numpy as np
    from asgkron import coeff, operators

    src = tmp_path / "caller.c"
    src.write_text(C_CALLER)
    exe = tmp_path / "caller"
    libdir = os.path.dirname(_lib._build.LIB_PATH)
    asgkron.lib()  # built
    r = subprocess.run(["gcc", "-std=c99", "-Wall", "-Werror", "-pedantic", "-I", os.path.join(ROOT, "include"),
                        str(src), "-o", str(exe), "-L", libdir, "-lasgkron", "-Wl,-rpath," + libdir],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0, (r.returncode, r.stderr)
    sx, sw, sh, so = (float(v) for v in r.stdout.split())
    x, w = coeff.gauss_legendre(10)
    H0, G0 = coeff.multiwavelet_filters(4)
    op = coeff.term_matrix(2, -1.0, 1.0, 2, [operators.div_term(None, -1.0, "P", "P")])
    assert abs(sx - np.sum(x * x)) <= 1e-15
    assert abs(sw - 2.0) <= 1e-14
    assert abs(sh - (np.sum(H0 * H0) + np.sum(G0 * G0))) <= 1e-13
    assert abs(so - np.sum(op.ravel() * np.arange(1, 65))) <= 1e-12 * max(1.0, abs(so))
