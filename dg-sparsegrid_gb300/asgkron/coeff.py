"""Native (C++) producer of the 1-D operators: Gauss-Legendre rules, multiwavelet filters, the
forward transform and pde.terms{t}.terms_1D{d}.mat (asg_gauss_legendre_f64,
asg_multiwavelet_filters_f64, asg_fmwt_matrix_f64, asg_coeff_matrix_f64).

Same arguments and results as the numpy builder in ``asgkron.operators`` (lgwt.m,
MultiwaveletGen.m, OperatorTwoScale_wavelet2.m, coeff_matrix.m + pterm_coeff_matrix.m +
sd_term_coeff_matrix.m).  The chain of partial terms is formed in realspace, where the
factors are block-tridiagonal, and rotated once; the result equals the factor-by-factor
rotation to the transform's orthogonality round-off.  Coefficient functions g(x) stay in
Python: they are sampled at the cells' Gauss nodes and faces and passed as arrays.
"""
import ctypes as C

import numpy as np

from ._lib import PartialTermDesc, check, lib

_KINDS = {"mass": 0, "div": 1, "grad": 2}


def _dptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _size(deg, lev):
    """(n, valid): n = deg 2^lev when the library accepts (deg, lev), else 1 so that the call
    still reaches the library and reports the error."""
    ok = deg >= 1 and lev >= 0 and deg * 2 ** lev <= 16384
    return (deg * 2 ** lev if ok else 1), ok


def gauss_legendre(n, a=-1.0, b=1.0):
    """n-point Gauss-Legendre nodes (ascending) and weights on [a, b] (lgwt.m)."""
    x, w = np.empty(n), np.empty(n)
    check(lib().asg_gauss_legendre_f64(int(n), float(a), float(b), _dptr(x), _dptr(w)))
    return x, w


def quad_points(deg):
    """max(deg+1, 10) points on [-1, 1] (default_quad_number.m:2)."""
    return gauss_legendre(max(deg + 1, 10))


def multiwavelet_filters(deg):
    """H0, G0 (deg x deg) of MultiwaveletGen.m."""
    H0, G0 = np.empty((deg, deg)), np.empty((deg, deg))
    check(lib().asg_multiwavelet_filters_f64(int(deg), _dptr(H0), _dptr(G0)))
    return H0, G0


def fmwt_matrix(deg, lev):
    """Forward multiwavelet transform (deg 2^lev square, OperatorTwoScale_wavelet2.m:127-144)."""
    n, _ = _size(deg, lev)
    F = np.empty((n, n))
    check(lib().asg_fmwt_matrix_f64(int(deg), int(lev), _dptr(F)))
    return F


def term_matrix(deg, lo, hi, lev, pterms):
    """Chained 1-D operator (M \\ L_1)(M \\ L_2)... in wavelet space for partial terms of
    ``asgkron.operators.PartialTerm`` (sd_term_coeff_matrix.m:9-22)."""
    if not pterms:
        raise ValueError("term_matrix: at least one partial term")
    n, ok = _size(deg, lev)
    if ok:
        N = 2 ** lev
        h = (hi - lo) / N
        xq, _ = quad_points(deg)
        xcell = ((xq[None, :] + 1) / 2 + np.arange(N)[:, None]) * h + lo  # [N, nq]
        faces = lo + np.arange(N + 1) * h
    descs = (PartialTermDesc * len(pterms))()
    keep = []
    for k, pt in enumerate(pterms):
        descs[k].kind = _KINDS[pt.kind]
        descs[k].LF = -pt.LF if pt.kind == "grad" else pt.LF  # the value given to GRAD
        descs[k].bcl = pt.BCL.encode()
        descs[k].bcr = pt.BCR.encode()
        if ok:  # otherwise the library rejects (deg, lev) before reading g
            gq = np.ascontiguousarray(pt.g(xcell) * np.ones_like(xcell), dtype=np.float64)
            gf = np.ascontiguousarray(np.asarray(pt.g(faces), dtype=np.float64) * np.ones_like(faces))
            keep += [gq, gf]
            descs[k].g_quad = _dptr(gq)
            descs[k].g_face = _dptr(gf)
    out = np.empty((n, n))
    check(lib().asg_coeff_matrix_f64(int(deg), int(lev), float(lo), float(hi), len(pterms), descs, _dptr(out)))
    return out
