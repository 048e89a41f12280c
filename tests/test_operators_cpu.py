"""The product's 1-D operator builder (asgkron.operators / pdes) against the reference's
two-scale data and the oracle's restatement of coeff_matrix.m."""
import os

import numpy as np
import pytest

from asgkron import operators as P
from asgkron import pdes
from oracle import asgard_oracle as O

G = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.mark.parametrize("k", range(1, 9))
def test_multiwavelet_filters_match_reference_mat(k):
    z = np.load(os.path.join(G, "two_scale_rel.npz"))
    H0, G0 = P.multiwavelet_filters(k)
    tol = 1e-14 if k <= 5 else 5e-12  # Gram-Schmidt round-off grows with the degree
    np.testing.assert_allclose(H0, z["H0_%d" % k], rtol=0, atol=tol)
    np.testing.assert_allclose(G0, z["G0_%d" % k], rtol=0, atol=tol)


@pytest.mark.parametrize("deg,lev", [(2, 2), (2, 3), (4, 3), (5, 5)])
def test_fmwt_matches_gold(deg, lev):
    t = np.load(os.path.join(G, "transformations.npz"))
    np.testing.assert_allclose(P.fmwt_matrix(deg, lev), t["operator_two_scale_%d_%d" % (deg, lev)], atol=2e-14)


def test_gauss_legendre_gold():
    q = np.load(os.path.join(G, "quadrature.npz"))
    x, w = P.gauss_legendre(32, -5, 2)
    np.testing.assert_allclose(x, q["lgwt_roots_32_neg5_2"].ravel(), atol=5e-15)
    np.testing.assert_allclose(w, q["lgwt_weights_32_neg5_2"].ravel(), atol=5e-16)


@pytest.mark.parametrize("name,lev,deg", [("continuity2", 4, 2), ("continuity3", 3, 3), ("diffusion2", 3, 4),
                                          ("continuity2", 3, 4)])
def test_term_mats_match_oracle(name, lev, deg):
    prod = getattr(pdes, name)(lev) if name == "diffusion2" else getattr(pdes, name)(lev, -1.0)
    orac = getattr(O, name)(lev) if name == "diffusion2" else getattr(O, name)(lev, LF=-1.0)
    A = prod.term_mats(deg, builder="numpy")
    B = O.build_term_mats(orac, deg)
    for ra, rb in zip(A, B):
        for a, b in zip(ra, rb):
            assert np.abs(a - b).max() <= 1e-13 * np.abs(b).max()


def test_projection_matches_oracle():
    prod = pdes.continuity2(3, 0.0)
    orac = O.continuity2(3, LF=0.0)
    from asgkron import grid
    t = grid.hash_table_sparse_nD([3, 3], 8)
    idx = t.idx1d()
    _, blocks = O.operator_two_scale(3, 8)
    for tt in (0.0, 0.37):
        a = prod.source_vector(3, idx, tt)
        b = O.md_eval(orac, 3, orac.sources, idx.astype(np.int64), blocks, tt)
        np.testing.assert_allclose(a, b, rtol=0, atol=1e-13 * np.abs(b).max())


@pytest.mark.parametrize("lev,deg", [(2, 2), (3, 3), ([4, 5], 2), (4, 4)])
def test_boundary_vector_matches_oracle(lev, deg):
    """boundary_condition_vector.m for diffusion2's Dirichlet data: product vs oracle."""
    import asgkron
    from asgkron import pdes

    pde = pdes.diffusion2(lev, case="reference")
    idx = asgkron.hash_table_sparse_nD(pde.levels, 8).idx1d()
    _, blocks = O.operator_two_scale(deg, 8)
    for t in (0.0, 0.0137):
        got = pde.boundary_vector(deg, idx, t)
        want = O.boundary_condition_vector(O.diffusion2(lev), deg, idx.astype(np.int64), blocks, t)
        assert np.linalg.norm(got - want) <= 1e-14 * np.linalg.norm(want)


@pytest.mark.parametrize("stem,name,lev", [("continuity2", "continuity2", 5), ("continuity_3", "continuity3", 5),
                                           ("continuity_6", "continuity6", 3), ("diffusion_2", "diffusion2", 3)])
def test_pde_specs_match_reference_pde_gold(stem, name, lev):
    """gold/gold_pde.m evaluates each PDE's initial condition, sources (spatial parts at
    x = 0.1..0.5, time factors at t = 5) and dt at CFL 1; the product's PDEs and the oracle's
    agree to round-off.  Exact solutions are compared where the initial-condition functions
    are the solution's (continuity2, diffusion2); continuity3/6 carry no solution."""
    z = np.load(os.path.join(G, "pde.npz"))
    x = np.array([0.1, 0.2, 0.3, 0.4, 0.5])
    T = 5.0
    prod = pdes.diffusion2(lev, case="reference") if name == "diffusion2" else getattr(pdes, name)(lev)
    orac = getattr(O, name)(lev)
    for spec, ic, sources, dt in ((prod, prod.ic, prod.sources, prod.dt(1.0)),
                                  (orac, orac.ic, orac.sources, orac.dt_fn(orac, 1.0))):
        def same(key, got):
            want = z["%s_%s" % (stem, key)].reshape(-1)
            got = np.asarray(got, dtype=np.float64).reshape(-1) * np.ones_like(want)
            assert np.abs(got - want).max() <= 1e-14 * max(1.0, np.abs(want).max()), key

        D = len(ic[0]) - 1
        for d in range(D):
            same("initial_dim%d" % d, ic[0][d](x, 0.0))
            if name in ("continuity2", "diffusion2"):
                same("exact_dim%d" % d, ic[0][d](x, T))
        if name in ("continuity2", "diffusion2"):
            same("exact_time", ic[0][-1](T))
        assert len(sources) == sum(1 for k in z.files if k.startswith(stem + "_source") and k.endswith("_time"))
        for s, src in enumerate(sources):
            for d in range(D):
                same("source%d_dim%d" % (s, d), src[d](x, T))
            same("source%d_time" % s, src[-1](T))
        same("dt", dt)
