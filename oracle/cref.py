"""Build and call the C oracle (apply_a_ref.c) -- TEST INFRASTRUCTURE ONLY.

Used by the tests as a fast faithful checker and by bench.py's CPU-baseline / reference
legs as the timed CPU implementation of the path.  Compiled with gcc -O3 -fopenmp into
oracle/_build/ (portable flags: the same recipe builds on x86_64 and aarch64).
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "apply_a_ref.c")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "liboracle_apply.so")

_L = None


def build(force=False):
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(SRC):
        return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    tmp = LIB + ".tmp%d" % os.getpid()
    cmd = ["gcc", "-O3", "-fopenmp", "-shared", "-fPIC", "-o", tmp, SRC]
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB)
    return LIB


def _lib():
    global _L
    if _L is None:
        build()
        L = C.CDLL(LIB)
        L.oracle_apply_rows.restype = C.c_int
        L.oracle_apply_rows.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p,
                                        C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_int]
        _L = L
    return _L


def apply_rows(term_mats, idx1d_1based, deg, f, rows=None, pairs0=None, nthreads=0):
    """FP64 rows of y = A f with the reference loop (pairs0: (row_ptr, 0-based cols) or None)."""
    mats = [[np.asfortranarray(m, dtype=np.float64) for m in row] for row in term_mats]
    T, D = len(mats), len(mats[0])
    idx = np.ascontiguousarray(np.asarray(idx1d_1based) - 1, dtype=np.int32)
    N = idx.shape[0]
    B = deg ** D
    rows = np.arange(N, dtype=np.int32) if rows is None else np.ascontiguousarray(rows, dtype=np.int32)
    ptrs = (C.c_void_p * (T * D))(*[mats[t][d].ctypes.data for t in range(T) for d in range(D)])
    lds = np.array([mats[t][d].shape[0] for t in range(T) for d in range(D)], dtype=np.int32)
    f = np.ascontiguousarray(f, dtype=np.float64)
    y = np.zeros(rows.size * B)
    rp = cl = None
    if pairs0 is not None:
        rp = np.ascontiguousarray(pairs0[0], dtype=np.int64)
        cl = np.ascontiguousarray(pairs0[1], dtype=np.int32)
    st = _lib().oracle_apply_rows(D, deg, T, N, idx.ctypes.data, ptrs, lds.ctypes.data,
                                  rp.ctypes.data if rp is not None else None,
                                  cl.ctypes.data if cl is not None else None, f.ctypes.data, rows.ctypes.data,
                                  rows.size, y.ctypes.data, int(nthreads))
    if st != 0:
        raise ValueError("oracle_apply_rows: bad arguments")
    return y
