"""Compile the MEX gateways (dg-sparsegrid_gb300/mex/*.c) against the stand-in mex.h in
tests/mex/ and call their mexFunction through ctypes -- what MATLAB would do, without MATLAB.

Each gateway becomes its own shared object (each defines mexFunction), linked against
libasgkron.so; arrays are passed as column-major doubles, cells as nested lists."""
import ctypes as C
import os
import subprocess

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
MEX_SRC = os.path.join(ROOT, "dg-sparsegrid_gb300", "mex")
STUB = os.path.join(ROOT, "tests", "mex")
OUT = os.path.join(STUB, "_build")


def build(gateway):
    """Compile <gateway>.c with the stub; returns the shared object's path."""
    from asgkron import _build

    lib = _build.build()
    libdir = os.path.dirname(lib)
    os.makedirs(OUT, exist_ok=True)
    so = os.path.join(OUT, gateway + "_stub.so")
    srcs = [os.path.join(MEX_SRC, gateway + ".c"), os.path.join(STUB, "mexstub.c")]
    deps = srcs + [os.path.join(MEX_SRC, "asgkron_mex.h"), os.path.join(STUB, "mex.h"), lib]
    if os.path.exists(so) and all(os.path.getmtime(d) <= os.path.getmtime(so) for d in deps):
        return so
    tmp = so + ".tmp%d" % os.getpid()
    cmd = ["gcc", "-std=c99", "-O1", "-Wall", "-Wextra", "-Werror", "-shared", "-fPIC", "-I" + STUB,
           "-I" + os.path.join(ROOT, "include"), "-o", tmp] + srcs + [lib, "-Wl,-rpath," + libdir]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("gateway build failed:\n%s\n%s" % (" ".join(cmd), r.stderr))
    os.replace(tmp, so)
    return so


class MexError(RuntimeError):
    def __init__(self, ident, msg):
        super().__init__("%s: %s" % (ident, msg))
        self.ident = ident
        self.msg = msg


class Mx:
    """A stand-in mxArray owned by the test (see Gateway.keep)."""

    def __init__(self, ptr):
        self.ptr = ptr


class Gateway:
    def __init__(self, name):
        L = C.CDLL(build(name))
        P = C.c_void_p
        for fn, res, args in (("stub_double", P, [C.c_size_t, C.c_size_t, P]), ("stub_cell", P, [C.c_size_t, C.c_size_t]),
                              ("stub_set_cell", None, [P, C.c_size_t, P]), ("stub_get_cell", P, [P, C.c_size_t]),
                              ("stub_set_complex", None, [P, C.c_int]), ("stub_m", C.c_size_t, [P]),
                              ("stub_n", C.c_size_t, [P]), ("stub_is_cell", C.c_int, [P]),
                              ("stub_data", C.POINTER(C.c_double), [P]), ("stub_destroy", None, [P]),
                              ("stub_call", C.c_int, [C.c_int, C.POINTER(P), C.c_int, C.POINTER(P)]),
                              ("stub_err_id", C.c_char_p, []), ("stub_err_msg", C.c_char_p, []),
                              ("stub_locked", C.c_int, []), ("stub_clear", None, [])):
            f = getattr(L, fn)
            f.restype = res
            f.argtypes = args
        self.L = L

    def arr(self, x):
        """An mxArray from a numpy array (column-major copy), a nested list (cell) or a scalar."""
        L = self.L
        if isinstance(x, list):
            rows = len(x)
            cols = len(x[0]) if rows else 0
            c = L.stub_cell(rows, cols)
            for i in range(rows):
                for j in range(cols):
                    L.stub_set_cell(c, i + j * rows, self.arr(x[i][j]))
            return c
        a = np.asarray(x, dtype=np.float64)
        if a.ndim == 0:
            a = a.reshape(1, 1)
        elif a.ndim == 1:
            a = a.reshape(-1, 1)
        a = np.asfortranarray(a)
        return L.stub_double(a.shape[0], a.shape[1], a.ctypes.data)

    def value(self, h):
        """numpy array (or nested list for a cell) of an mxArray."""
        L = self.L
        m, n = L.stub_m(h), L.stub_n(h)
        if L.stub_is_cell(h):
            return [[self.value(L.stub_get_cell(h, i + j * m)) for j in range(n)] for i in range(m)]
        if m * n == 0:
            return np.zeros((m, n))
        return np.ctypeslib.as_array(L.stub_data(h), shape=(m * n,)).reshape((m, n), order="F").copy()

    def keep(self, x):
        """An input that outlives calls (the caller frees it with ``free``): edit it in place
        between calls the way MATLAB may modify an unshared array."""
        return Mx(self.arr(x))

    def free(self, mx):
        self.L.stub_destroy(mx.ptr)

    def data(self, mx):
        """Writable view of a kept input's doubles (column-major), for in-place edits."""
        m, n = self.L.stub_m(mx.ptr), self.L.stub_n(mx.ptr)
        return np.ctypeslib.as_array(self.L.stub_data(mx.ptr), shape=(m * n,))

    def call(self, nlhs, *args):
        """mexFunction(nlhs, plhs, nrhs, prhs) on numpy arrays, nested lists (cells), scalars or
        kept inputs (Mx); returns the outputs as numpy values (cells as nested lists)."""
        L = self.L
        made = [self.arr(a) for a in args if not isinstance(a, Mx)]
        it = iter(made)
        ins = [a.ptr if isinstance(a, Mx) else next(it) for a in args]
        prhs = (C.c_void_p * max(1, len(ins)))(*ins)
        plhs = (C.c_void_p * max(1, nlhs))()
        rc = L.stub_call(nlhs, plhs, len(ins), prhs)
        outs = []
        if rc == 0:
            for i in range(nlhs):
                outs.append(self.value(plhs[i]))
                L.stub_destroy(plhs[i])
        for h in made:
            L.stub_destroy(h)
        if rc != 0:
            raise MexError(L.stub_err_id().decode(), L.stub_err_msg().decode())
        return outs

    def clear(self):
        self.L.stub_clear()
