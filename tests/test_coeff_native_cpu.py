"""The native (C++) 1-D operator builder (asg_coeff_matrix_f64 and its helpers, asgkron.coeff)
against the reference's quadrature / two-scale / transform gold data, the oracle's
restatement of coeff_matrix.m, and the numpy builder.  Host code only: no GPU needed."""
import os

import numpy as np
import pytest

from asgkron import coeff as N
from asgkron import operators as P
from asgkron import pdes
from asgkron._lib import AsgError
from oracle import asgard_oracle as O

G = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def test_native_gauss_legendre_gold():
    q = np.load(os.path.join(G, "quadrature.npz"))
    x, w = N.gauss_legendre(32, -5, 2)
    np.testing.assert_allclose(x, q["lgwt_roots_32_neg5_2"].ravel(), atol=5e-15)
    np.testing.assert_allclose(w, q["lgwt_weights_32_neg5_2"].ravel(), atol=5e-16)
    x, w = N.gauss_legendre(1, 0.0, 3.0)
    assert x[0] == 1.5 and w[0] == 3.0


@pytest.mark.parametrize("k", range(1, 9))
def test_native_multiwavelet_filters_match_reference_mat(k):
    z = np.load(os.path.join(G, "two_scale_rel.npz"))
    H0, G0 = N.multiwavelet_filters(k)
    tol = 1e-14 if k <= 5 else 5e-12  # Gram-Schmidt round-off grows with the degree
    np.testing.assert_allclose(H0, z["H0_%d" % k], rtol=0, atol=tol)
    np.testing.assert_allclose(G0, z["G0_%d" % k], rtol=0, atol=tol)


@pytest.mark.parametrize("deg,lev", [(2, 2), (2, 3), (4, 3), (5, 5)])
def test_native_fmwt_matches_gold(deg, lev):
    t = np.load(os.path.join(G, "transformations.npz"))
    np.testing.assert_allclose(N.fmwt_matrix(deg, lev), t["operator_two_scale_%d_%d" % (deg, lev)], atol=2e-14)


@pytest.mark.parametrize("deg,lev", [(1, 0), (3, 0), (1, 4), (3, 4), (4, 6)])
def test_native_fmwt_matches_numpy_and_is_orthogonal(deg, lev):
    F = N.fmwt_matrix(deg, lev)
    assert np.abs(F - P.fmwt_matrix(deg, lev)).max() <= 1e-14
    assert np.abs(F @ F.T - np.eye(F.shape[0])).max() <= 1e-13


@pytest.mark.parametrize("name,lev,deg", [("continuity2", 4, 2), ("continuity3", 3, 3), ("diffusion2", 3, 4),
                                          ("continuity2", 3, 4)])
def test_native_term_mats_match_oracle(name, lev, deg):
    prod = getattr(pdes, name)(lev) if name == "diffusion2" else getattr(pdes, name)(lev, -1.0)
    orac = getattr(O, name)(lev) if name == "diffusion2" else getattr(O, name)(lev, LF=-1.0)
    A = prod.term_mats(deg, builder="native")
    B = O.build_term_mats(orac, deg)
    for ra, rb in zip(A, B):
        for a, b in zip(ra, rb):
            assert np.abs(a - b).max() <= 1e-13 * np.abs(b).max()


@pytest.mark.parametrize("deg", [1, 2, 4, 6])
def test_native_unit_mass_factors_are_exact_identities(deg):
    """A unit-coefficient mass term is the LHS mass itself: its factor, and any chain of such
    factors, is exactly the identity (the reference's M_w \\ M_w), so the plan's structure
    detection sees identity dimensions whatever the transform's round-off."""
    for pde in (pdes.continuity2(3, -1.0), pdes.continuity3(2, -1.0), pdes.diffusion2(3)):
        for t_native, t in zip(pde.term_mats(deg), pde.terms):
            for A, pts in zip(t_native, t):
                if all(p.kind == "mass" for p in pts):
                    assert np.array_equal(A, np.eye(A.shape[0]))
    assert np.array_equal(N.term_matrix(deg, 0.0, 1.0, 3, [P.mass_term(), P.mass_term()]), np.eye(deg * 8))


def _g_var(x):
    return 1.5 + np.sin(x)  # a non-constant coefficient, positive on the interval


def _g_sign(x):
    return x - 0.2  # changes sign inside [-1, 1]: exercises the |g| of the flux


@pytest.mark.parametrize("deg", [1, 2, 3, 4, 5])
@pytest.mark.parametrize("lev", [0, 1, 2, 5])
def test_native_term_matrix_matches_numpy_builder(deg, lev):
    """Every partial-term kind, flux and boundary pairing the builder distinguishes, constant
    and variable coefficients, single terms and LDG-style chains, on 1 / 2 / 4 / 32 cells
    (periodic wrap on one and two cells included)."""
    cases = []
    for bcl, bcr in (("P", "P"), ("D", "D"), ("N", "N"), ("D", "N"), ("N", "D")):
        for LF in (0.0, -1.0, 1.0):
            cases.append([P.div_term(None, LF, bcl, bcr)])
            cases.append([P.grad_term(_g_var, LF, bcl, bcr)])
            cases.append([P.div_term(_g_sign, LF, bcl, bcr), P.grad_term(None, LF, bcl, bcr)])
    cases.append([P.mass_term(_g_var)])
    cases.append([P.mass_term(), P.div_term(_g_var, -1.0, "P", "P"), P.mass_term(_g_var)])
    for pts in cases:
        a = P.term_matrix(deg, -1.0, 1.0, lev, pts)
        b = N.term_matrix(deg, -1.0, 1.0, lev, pts)
        # a periodic single-cell div of a constant cancels to round-off: the floor is the
        # size of its parts (1/h on cells of width 2/2^lev)
        scale = max(np.abs(a).max(), 2.0 ** lev / 2)
        assert np.abs(a - b).max() <= 5e-13 * scale, ([p.kind for p in pts], pts[0].BCL, pts[0].BCR)


def test_native_builder_on_a_shifted_interval():
    pts = [P.div_term(_g_var, -1.0, "D", "N"), P.grad_term(None, -1.0, "D", "N")]
    a = P.term_matrix(3, 0.5, 4.0, 4, pts)
    b = N.term_matrix(3, 0.5, 4.0, 4, pts)
    assert np.abs(a - b).max() <= 5e-13 * np.abs(a).max()


def test_native_builder_rejects_bad_arguments():
    with pytest.raises(AsgError, match="deg=0"):
        N.multiwavelet_filters(0)
    with pytest.raises(AsgError, match="lev=-1"):
        N.fmwt_matrix(2, -1)
    with pytest.raises(AsgError, match="deg\\*2\\^lev"):
        N.fmwt_matrix(4, 13)
    with pytest.raises(AsgError, match="lev=70"):
        N.fmwt_matrix(1, 70)
    with pytest.raises(AsgError, match="n=0"):
        N.gauss_legendre(0)
    with pytest.raises(AsgError, match="empty interval"):
        N.term_matrix(2, 1.0, 1.0, 2, [P.mass_term()])
    bad = P.div_term(None, 0.0, "X", "P")
    with pytest.raises(AsgError, match="boundary types"):
        N.term_matrix(2, 0.0, 1.0, 2, [bad])
    bad = P.mass_term()
    bad.kind = "curl"
    with pytest.raises(KeyError):
        N.term_matrix(2, 0.0, 1.0, 2, [bad])
    with pytest.raises(ValueError, match="at least one"):
        N.term_matrix(2, 0.0, 1.0, 2, [])
    with pytest.raises(ValueError, match="builder"):
        pdes.continuity2(2, -1.0).term_mats(2, builder="fortran")


@pytest.mark.parametrize("name,pdename,lev,deg", [("continuity2_sg_l4_d3", "continuity2", 4, 3),
                                                  ("continuity3_sg_l4_d3", "continuity3", 4, 3)])
def test_native_operators_reproduce_gold_rk3(name, pdename, lev, deg):
    """Five RK3 steps (the oracle's stepper and apply loop) on the native builder's operators,
    built at max_lev 8 as the gold was, reproduce gold/generated-inputs/time_advance."""
    opde = getattr(O, pdename)(lev, LF=0.0)
    lv, cl, _ = O.hash_table_sparse_nd([d.lev for d in opde.dims], 8, "SG")
    idx = O.element_idx1d(lv, cl)
    _, blocks = O.operator_two_scale(deg, 8)
    mats = getattr(pdes, pdename)(lev, 0.0).term_mats(deg, construction_level=8)
    f = O.md_eval(opde, deg, opde.ic, idx, blocks, 0.0)
    dt = opde.dt_fn(opde, 0.01)
    ta = np.load(os.path.join(G, "time_advance.npz"))
    for i in range(5):
        f = O.rk3_step(lambda v: O.apply_A_rows(mats, idx, deg, v), f, i * dt, dt,
                       lambda t: O.md_eval(opde, deg, opde.sources, idx, blocks, t))
        g = ta["%s_t%d" % (name, i)]
        assert np.linalg.norm(f - g) <= 1e-14 * np.linalg.norm(g), i


def test_native_builder_scalar_coefficients_and_null_arguments():
    import ctypes as C

    from asgkron._lib import ASG_ERR_INVALID, lib

    pts = [P.div_term(lambda x: 2.0, -1.0, "N", "D"), P.grad_term(lambda x: -0.5, 0.0, "D", "N")]
    a = P.term_matrix(3, -2.0, 1.0, 3, pts)
    b = N.term_matrix(3, -2.0, 1.0, 3, pts)
    assert np.abs(a - b).max() <= 5e-13 * np.abs(a).max()
    out = np.empty((8, 8))
    ptr = out.ctypes.data_as(C.POINTER(C.c_double))
    assert lib().asg_coeff_matrix_f64(2, 2, 0.0, 1.0, 1, None, ptr) == ASG_ERR_INVALID
    assert lib().asg_fmwt_matrix_f64(2, 2, None) == ASG_ERR_INVALID
    assert lib().asg_gauss_legendre_f64(4, 0.0, 1.0, None, ptr) == ASG_ERR_INVALID
    assert lib().asg_multiwavelet_filters_f64(2, ptr, None) == ASG_ERR_INVALID


@pytest.mark.parametrize("name,levels,deg", [("continuity2", [4, 4], 3), ("continuity3", [2, 3, 2], 4),
                                             ("continuity6", [2] * 6, 4), ("diffusion2", [2, 3], 5)])
@pytest.mark.parametrize("builder", ["native", "numpy", "rechain"])
def test_operators_match_reference_coefficient_gold(name, levels, deg, builder):
    """pde.terms{t}.terms_1D{d}.mat of every term and dimension against
    gold/generated-inputs/coefficients (gold_coefficients.m: central flux, max_lev_coeffs, so
    chained terms are rechained at each dimension's level).  Tolerance: the transform's
    orthogonality round-off, which grows with the degree (2.3e-13 at deg 5)."""
    z = np.load(os.path.join(G, "coefficients.npz"))
    pde = pdes.diffusion2(levels, case="reference") if name == "diffusion2" else getattr(pdes, name)(levels, 0.0)
    if builder == "rechain":
        mats = pde.rechain_term_mats(deg, levels, max_lev=8)
    else:
        mats = pde.term_mats(deg, builder=builder)
    tol = 5e-13 if deg >= 5 else 1e-13
    stem = "%s_coefficients_l%s_d%d" % (name, "_".join("%d" % v for v in levels), deg)
    for t in range(len(pde.terms)):
        for d in range(len(levels)):
            want = z["%s_%d_%d" % (stem, t + 1, d + 1)]
            got = mats[t][d]
            assert got.shape == want.shape, (t, d)
            assert np.abs(got - want).max() <= tol * np.abs(want).max(), (t, d)
