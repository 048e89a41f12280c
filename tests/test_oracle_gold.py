"""Pin the CPU oracle against the reference's own gold files (packed by golden/make_golden.py).

Integer/index structures are compared bit-exactly; floating-point quantities to the stated
tolerances.  The RK3 trajectories were generated with central flux (LF=0) and before
md_eval_function.m gained its mass solve, which is how they are replayed here.
"""
import os

import numpy as np
import pytest

from oracle import asgard_oracle as O

G = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _npz(name):
    return np.load(os.path.join(G, name))


# ---------------------------------------------------------------- quadrature / basis
@pytest.mark.parametrize("lev,deg", [(2, 2), (2, 5), (5, 2), (5, 5)])
def test_transform_blocks_gold(lev, deg):
    """OperatorTwoScale_wavelet2.m's blocks (the per-level pieces md_eval transforms with)
    against gold/generated-inputs/basis/transform_blocks_l<lev>_d<deg>_<b>."""
    z = _npz("basis.npz")
    _, blocks = O.operator_two_scale(deg, lev)
    assert len(blocks) == 2 * lev
    for b, blk in enumerate(blocks):
        want = z["transform_blocks_l%d_d%d_%d" % (lev, deg, b + 1)].reshape(blk.shape)
        np.testing.assert_allclose(blk, want, rtol=0, atol=1e-15)


def test_lgwt_gold():
    q = _npz("quadrature.npz")
    for (n, a, b, tag) in ((10, -1, 1, "10_neg1_1"), (32, -5, 2, "32_neg5_2")):
        x, w = O.lgwt(n, a, b)
        np.testing.assert_allclose(x, q["lgwt_roots_" + tag].ravel(), rtol=0, atol=1e-15 * max(1, abs(a), abs(b)))
        np.testing.assert_allclose(w, q["lgwt_weights_" + tag].ravel(), rtol=0, atol=1e-15)


def test_legendre_at_minus_one_gold():
    q = _npz("quadrature.npz")
    np.testing.assert_allclose(O.lin_legendre(-1.0, 2), q["legendre_poly_neg1_2"], atol=1e-15)
    np.testing.assert_allclose(O.lin_dlegendre(-1.0, 2), q["legendre_deriv_neg1_2"], atol=1e-15)


@pytest.mark.parametrize("deg,lev", [(2, 2), (2, 3), (4, 3), (5, 5)])
def test_two_scale_operator_gold(deg, lev):
    t = _npz("transformations.npz")
    F, _ = O.operator_two_scale(deg, lev)
    np.testing.assert_allclose(F, t["operator_two_scale_%d_%d" % (deg, lev)], atol=2e-14)


def test_combine_dimensions_gold():
    t = _npz("transformations.npz")
    lv, cl, _ = O.hash_table_sparse_nd([3, 3], 8, "SG")
    idx = O.element_idx1d(lv, cl)
    got = O.combine_dimensions(2, [np.arange(1, 17.0), np.arange(17, 33.0)], 2.0, idx)
    np.testing.assert_array_equal(got, t["combine_dim_dim2_deg2_lev3_sg"].ravel())
    lv, cl, _ = O.hash_table_sparse_nd([2, 2, 2], 8, "FG")
    idx = O.element_idx1d(lv, cl)
    got = O.combine_dimensions(3, [np.arange(1, 13.0), np.arange(13, 25.0), np.arange(25, 37.0)], 2.5, idx)
    np.testing.assert_array_equal(got, t["combine_dim_dim3_deg3_lev2_fg"].ravel())


# ---------------------------------------------------------------- element tables
@pytest.mark.parametrize("levels", [[7], [5, 2], [3, 2, 3]])
@pytest.mark.parametrize("grid", ["SG", "FG"])
def test_element_table_gold(levels, grid):
    e = _npz("element_table.npz")
    d = len(levels)
    lv, cl, ids = O.hash_table_sparse_nd(levels, 7, grid)
    table = np.concatenate([lv, cl], axis=1)
    np.testing.assert_array_equal(table, e["table_%dd_%s" % (d, grid)].astype(np.int64))
    np.testing.assert_array_equal(ids.astype(np.int64) - 1, e["ids_%dd_%s" % (d, grid)].ravel().astype(np.int64))


def test_1d_index_gold():
    e = _npz("element_table.npz")
    for k in e.files:
        if k.startswith("1d_index_"):
            lev, cell = (int(v) for v in k.split("_")[2:4])
            assert int(O.lev_cell_to_1d_index(lev, cell)) == int(e[k].ravel()[0]), k


# ---------------------------------------------------------------- permutations
def _tuples(arr):
    return [tuple(int(v) for v in row) for row in np.atleast_2d(arr)]


@pytest.mark.parametrize("dims,n,ordr", [(1, 1, 0), (2, 4, 1), (4, 6, 0), (6, 8, 1)])
def test_perm_leq_eq_max_gold(dims, n, ordr):
    p = _npz("permutations.npz")
    tag = "%d_%d_%d" % (dims, n, ordr)
    assert O.perm_leq(dims, n, bool(ordr)) == _tuples(p["perm_leq_" + tag])
    assert len(O.perm_leq(dims, n)) == int(p["perm_leq_%s_count" % tag].ravel()[0])
    assert O.perm_eq(dims, n, bool(ordr)) == _tuples(p["perm_eq_" + tag])
    if "perm_max_" + tag in p.files:
        assert O.perm_max(dims, [n] * dims, bool(ordr)) == _tuples(p["perm_max_" + tag])
    assert (n + 1) ** dims == int(p["perm_max_%s_count" % tag].ravel()[0])


@pytest.mark.parametrize("levels,srt", [([3, 3], 1), ([1, 4], 0), ([1, 5, 8], 1), ([10, 6, 9, 10], 0),
                                        ([2, 10, 1, 5, 4, 7], 1)])
def test_perm_d_gold(levels, srt):
    p = _npz("permutations.npz")
    d = len(levels)
    tag = "%d_%d" % (d, srt)
    got = O.perm_leq_d(d, levels, max(levels), bool(srt))
    assert got == _tuples(p["perm_leq_d_" + tag])
    assert len(got) == O.perm_leq_d_count(d, levels, max(levels)) == int(p["perm_leq_d_%s_count" % tag].ravel()[0])
    got = O.perm_eq_d(d, levels, max(levels), bool(srt))
    assert got == _tuples(p["perm_eq_d_" + tag])
    assert O.perm_eq_d_count(d, levels, max(levels)) == int(p["perm_eq_d_%s_count" % tag].ravel()[0])
    assert O.perm_max(d, levels, bool(srt)) == _tuples(p["perm_max_d_" + tag])


def test_index_leq_max_gold():
    p = _npz("permutations.npz")
    lists = [np.arange(2, 4), np.arange(0, 5), np.arange(0, 4), np.arange(1, 6)]
    got = [tuple(v + 1 for v in t) for t in O.index_leq_max(4, lists, 10, 4)]
    assert got == _tuples(p["index_leq_max_4d_10s_4m"])
    assert len(got) == int(p["index_leq_max_4d_10s_4m_count"].ravel()[0])


# ---------------------------------------------------------------- connectivity
@pytest.mark.parametrize("lev", [2, 3, 8])
def test_connect_1d_gold(lev):
    c = _npz("connectivity.npz")
    np.testing.assert_array_equal(O.connect_1d(lev), c["connect_1_%d" % lev].astype(np.int64))


@pytest.mark.parametrize("d,lev,grid,levsum,levmax", [(2, 3, "FG", 6, 3), (3, 4, "SG", 4, 4)])
def test_connect_nd_gold(d, lev, grid, levsum, levmax):
    c = _npz("connectivity.npz")
    lv, cl = O.hash_table_nd(lev, d, grid)
    conn = O.connect_nd(d, lv, cl, levsum, levmax, "SG")
    assert len(conn) == lv.shape[0]
    for i, row in enumerate(conn):
        np.testing.assert_array_equal(row, c["connect_n_%d_%d_%s_%d" % (d, lev, grid, i + 1)].ravel().astype(np.int64))


# ---------------------------------------------------------------- kron chain
def test_kron_multd_matches_krond():
    rng = np.random.default_rng(7)
    for n in range(1, 7):
        mats = [rng.standard_normal((rng.integers(2, 4), rng.integers(2, 4))) for _ in range(n)]
        nc = int(np.prod([m.shape[1] for m in mats]))
        X = rng.standard_normal((nc, 3))
        np.testing.assert_allclose(O.kron_multd(n, mats, X), O.krond(mats) @ X, rtol=1e-12, atol=1e-12)


def test_kronmult_batch_matches_krond():
    """Kronmult/test1_batch.m: kronmultN_batch vs explicit kron, tol 1e-7*numel; the same
    A1..A6 shapes (2x3, 3x4, 4x5, 5x6, 6x7, 3x2) and nvec=2, seeded here."""
    rng = np.random.default_rng(11)
    shapes = [(2, 3), (3, 4), (4, 5), (5, 6), (6, 7), (3, 2)]
    mats_all = [rng.random(s) for s in shapes]
    for n in range(1, 7):
        mats = mats_all[:n] if n < 6 else mats_all
        nc = int(np.prod([m.shape[1] for m in mats]))
        X = rng.random((nc, 2))
        lists = [O.BatchList() for _ in range(n)]
        Y = O.kronmult_batch(mats, X, lists)
        Yok = O.krond(mats) @ X
        assert np.max(np.abs(Y - Yok)) < 1e-7 * Yok.size
        # replaying the recorded lists through gemm_vbatched reproduces every C
        for bl in lists:
            if bl.nbatch == 0:
                continue
            ent = bl.entries
            for tA in "NT":
                sel = [e for e in ent]
                Cs = O.gemm_vbatched(sel[0]["transA"], sel[0]["transB"], [e["m"] for e in sel], [e["n"] for e in sel],
                                     [e["k"] for e in sel], 1.0, [e["A"] for e in sel], [e["B"] for e in sel], 0.0,
                                     [e["C"] for e in sel]) if all(e["transB"] == sel[0]["transB"] for e in sel) else None
                if Cs is not None:
                    for e, C in zip(sel, Cs):
                        ref = O.gemm(e["transA"], e["transB"], e["m"], e["n"], e["k"], 1.0, e["A"], e["B"], 0.0, e["C"])
                        np.testing.assert_allclose(C, ref, rtol=1e-14, atol=1e-14)
                break


# ---------------------------------------------------------------- apply_A + RK3 trajectories
def _replay(name, pdefn, lev, deg, grid="SG"):
    pde = pdefn(lev, LF=0.0)
    lev_vec = [d.lev for d in pde.dims]
    max_lev = 4 if len(lev_vec) > 3 else 8
    lv, cl, _ = O.hash_table_sparse_nd(lev_vec, max_lev, grid)
    idx = O.element_idx1d(lv, cl)
    _, blocks = O.operator_two_scale(deg, max_lev)
    mats = O.build_term_mats(pde, deg, coeff_level=max_lev)
    f = O.md_eval(pde, deg, pde.ic, idx, blocks, 0.0)
    dt = pde.dt_fn(pde, 0.01)
    ta = _npz("time_advance.npz")
    worst = 0.0
    for i in range(5):
        f = O.rk3_step(lambda v: O.apply_A_rows(mats, idx, deg, v), f, i * dt, dt,
                       lambda t: O.md_eval(pde, deg, pde.sources, idx, blocks, t))
        g = ta["%s_t%d" % (name, i)]
        ng = np.linalg.norm(g)
        # (a gold state can be exactly zero: deg-2 projections of continuity6's sources vanish)
        worst = max(worst, np.linalg.norm(f - g) / ng if ng > 0 else np.linalg.norm(f))
    return worst


@pytest.mark.parametrize("name,pdefn,lev,deg,grid", [
    ("continuity1_sg_l2_d2", O.continuity1, 2, 2, "SG"),
    ("continuity1_sg_l4_d3", O.continuity1, 4, 3, "SG"),
    ("continuity1_fg_l2_d2", O.continuity1, 2, 2, "FG"),
    ("continuity2_sg_l2_d2", O.continuity2, 2, 2, "SG"),
    ("continuity2_sg_l4_d3", O.continuity2, 4, 3, "SG"),
    ("continuity2_fg_l2_d2", O.continuity2, 2, 2, "FG"),
    ("continuity3_sg_l2_d2", O.continuity3, 2, 2, "SG"),
    ("continuity3_sg_l4_d3", O.continuity3, 4, 3, "SG"),
    ("continuity2_fg_l3_4_d3", O.continuity2, [3, 4], 3, "FG"),
    ("continuity3_sg_l3_4_2_d4", O.continuity3, [3, 4, 2], 4, "SG"),
    ("continuity6_sg_l2_d2", O.continuity6, 2, 2, "SG"),
    ("continuity6_sg_l2_d3", O.continuity6, 2, 3, "SG"),
    ("continuity6_sg_l2_3_2_3_3_2_d2", O.continuity6, [2, 3, 2, 3, 3, 2], 2, "SG"),
])
def test_rk3_trajectory_gold(name, pdefn, lev, deg, grid):
    assert _replay(name, pdefn, lev, deg, grid) < 1e-14


def _replay_be(name, pdefn, lev, deg, grid="SG"):
    """Backward Euler (time_advance.m:267-349: (I - dt A) f1 = f0 + dt s(t + dt), direct
    solve) from the projected initial condition, against the gold trajectory."""
    pde = pdefn(lev, LF=0.0)
    lev_vec = [d.lev for d in pde.dims]
    max_lev = 4 if len(lev_vec) > 3 else 8
    lv, cl, _ = O.hash_table_sparse_nd(lev_vec, max_lev, grid)
    idx = O.element_idx1d(lv, cl)
    _, blocks = O.operator_two_scale(deg, max_lev)
    mats = O.build_term_mats(pde, deg, coeff_level=max_lev)
    f = O.md_eval(pde, deg, pde.ic, idx, blocks, 0.0)
    _, A = O.apply_A_loop(mats, idx, deg, f, build_A=True)
    dt = pde.dt_fn(pde, 0.01)
    ta = _npz("time_advance.npz")
    worst = 0.0
    for i in range(5):
        f = O.backward_euler_step(A, f, dt, O.md_eval(pde, deg, pde.sources, idx, blocks, (i + 1) * dt))
        g = ta["%s_t%d" % (name, i)]
        worst = max(worst, np.linalg.norm(f - g) / np.linalg.norm(g))
    return worst


@pytest.mark.parametrize("name,pdefn,lev,deg,grid", [
    ("continuity1_implicit_l2_d2", O.continuity1, 2, 2, "SG"),
    ("continuity1_implicit_l4_d3", O.continuity1, 4, 3, "SG"),
    ("continuity2_implicit_l2_d2", O.continuity2, 2, 2, "SG"),
    ("continuity2_implicit_l4_d3", O.continuity2, 4, 3, "SG"),
    ("continuity2_implicit_fg_l3_4_d3", O.continuity2, [3, 4], 3, "FG"),
])
def test_backward_euler_trajectory_gold(name, pdefn, lev, deg, grid):
    assert _replay_be(name, pdefn, lev, deg, grid) < 1e-13


def _replay_diffusion2(name, lev, deg, method):
    """diffusion2.m with its Dirichlet data: LDG operators chained at each dimension's own
    level, the boundary vector added to the rhs at the stage (RK3) or end (BE) times."""
    pde = O.diffusion2(lev)
    lev_vec = [d.lev for d in pde.dims]
    lv, cl, _ = O.hash_table_sparse_nd(lev_vec, 8, "SG")
    idx = O.element_idx1d(lv, cl)
    _, blocks = O.operator_two_scale(deg, 8)
    mats = O.build_term_mats(pde, deg)
    f = O.md_eval(pde, deg, pde.ic, idx, blocks, 0.0)
    dt = pde.dt_fn(pde, 0.01)
    bc = lambda t: O.boundary_condition_vector(pde, deg, idx, blocks, t)
    if method == "BE":
        _, A = O.apply_A_loop(mats, idx, deg, f, build_A=True)
    ta = _npz("time_advance.npz")
    worst = 0.0
    for i in range(5):
        if method == "RK3":
            f = O.rk3_step(lambda v: O.apply_A_rows(mats, idx, deg, v), f, i * dt, dt, bc)
        else:
            f = O.backward_euler_step(A, f, dt, bc((i + 1) * dt))
        g = ta["%s_t%d" % (name, i)]
        worst = max(worst, np.linalg.norm(f - g) / np.linalg.norm(g))
    return worst


@pytest.mark.parametrize("name,lev,deg,method", [
    ("diffusion2_sg_l2_d2", 2, 2, "RK3"), ("diffusion2_sg_l3_d3", 3, 3, "RK3"), ("diffusion2_sg_l4_d4", 4, 4, "RK3"),
    ("diffusion2_sg_l4_5_d2", [4, 5], 2, "RK3"), ("diffusion2_implicit_sg_l3_d3", 3, 3, "BE"),
    ("diffusion2_implicit_sg_l4_d3", 4, 3, "BE"), ("diffusion2_implicit_sg_l5_d3", 5, 3, "BE"),
    ("diffusion2_implicit_sg_l4_5_d2", [4, 5], 2, "BE"),
])
def test_diffusion2_trajectory_gold(name, lev, deg, method):
    # deg 4 at lev 4: the LDG operator's entries are ~1e5 times |A f| (cancellation), so
    # rounding-level differences in A reach ~1e-10 of A f; every other stem agrees to ~1e-14
    tol = 1e-9 if name == "diffusion2_sg_l4_d4" else 1e-13
    assert _replay_diffusion2(name, lev, deg, method) < tol


def test_apply_A_loop_equals_vectorised_and_krond():
    """The faithful loop, the vectorised restatement and the assembled krond matrix agree
    (apply_A.m:170-201), with and without a connectivity list."""
    pde = O.continuity2(2, LF=-1.0)
    lv, cl, _ = O.hash_table_sparse_nd([2, 2], 8, "SG")
    idx = O.element_idx1d(lv, cl)
    mats = O.build_term_mats(pde, 2)
    f = np.random.default_rng(0).standard_normal(idx.shape[0] * 4)
    y1 = O.apply_A_loop(mats, idx, 2, f)
    y2 = O.apply_A_rows(mats, idx, 2, f)
    _, A = O.apply_A_loop(mats, idx, 2, f, build_A=True)
    np.testing.assert_allclose(y1, y2, rtol=1e-13, atol=1e-13)
    np.testing.assert_allclose(y1, A @ f, rtol=1e-13, atol=1e-12)
