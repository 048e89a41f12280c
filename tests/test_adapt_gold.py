"""Adaptivity pinned to the reference's adaptation gold (gold/generated-inputs/adapt: one
coarsening and one refinement of given vectors, bit-exact) and its adaptive gold
trajectories.

The product's host pieces under test: the element rules of ``asgkron.adapt.adapt``
(adapt.m), its element tables (hash_table_sparse_nD order) and the rechained operators of
``PDE.rechain_term_mats`` (get_coeff_mats_rechain.m).  The oracle steps and projects (the
checker), on each adapted table.

* continuity2_ad_sg_l3_d4 follows gold/gold_time_advance.m:21-24, 291-362 exactly: the
  initial condition refined until the table stops growing and re-projected, then coarsened
  and re-projected; every step coarsens, advances (RK3), refines from the advanced values and
  repeats the step on the refined table until no element is added.
* diffusion2_ad_implicit_sg_l3_d4 reproduces with an adapt threshold of 1e-4 (the generator
  script states 0.05) and the initial-condition adaptation alone: its table keeps elements
  far below the coarsening threshold of 0.05 at every step.  So the stem pins the
  initial-condition rules, rechained LDG operators on an adapted table, the Dirichlet data
  projected on it and backward Euler.
"""
import os

import numpy as np
import pytest

from oracle import asgard_oracle as O

G = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
NEW_ELEMENT_VALUE = 1e-15


class Replay:
    def __init__(self, name, lev, deg, thr, method, max_lev=8):
        import asgkron
        from asgkron import pdes

        self.opde = O.continuity2(lev, LF=0.0) if name == "continuity2" else O.diffusion2(lev)
        self.ppde = pdes.continuity2(lev, 0.0) if name == "continuity2" else pdes.diffusion2(lev, case="reference")
        self.name, self.deg, self.thr, self.method, self.max_lev = name, deg, thr, method, max_lev
        self.dt = self.opde.dt_fn(self.opde, 0.01)  # at the starting level, as the driver sets it
        _, self.blocks = O.operator_two_scale(deg, max_lev)
        self.cache = {}
        self.set_table(asgkron.hash_table_sparse_nD([lev, lev], max_lev))

    def set_table(self, table):
        from asgkron.adapt import table_levels

        self.table = table
        self.levels = table_levels(table)
        for dim, lv in zip(self.opde.dims, self.levels):  # adapt.m:417-425
            dim.lev = lv
        self.idx = table.idx1d().astype(np.int64)

    def adapt(self, f, coarsen, refine):
        from asgkron.adapt import adapt

        r = adapt(self.table, f, self.deg, self.max_lev, self.thr, coarsen=coarsen, refine=refine)
        self.set_table(r.table)
        return r

    def ic(self):
        return O.md_eval(self.opde, self.deg, self.opde.ic, self.idx, self.blocks, 0.0)

    def step(self, f, t):
        mats = self.ppde.rechain_term_mats(self.deg, self.levels, self.max_lev, self.cache)
        idx, deg = self.idx, self.deg
        if self.name == "diffusion2":
            src = lambda tt: O.boundary_condition_vector(self.opde, deg, idx, self.blocks, tt)
        else:
            src = lambda tt: O.md_eval(self.opde, deg, self.opde.sources, idx, self.blocks, tt)
        if self.method == "BE":
            _, A = O.apply_A_loop(mats, idx, deg, f, build_A=True)
            return O.backward_euler_step(A, f, self.dt, src(t + self.dt))
        return O.rk3_step(lambda v: O.apply_A_rows(mats, idx, deg, v), f, t, self.dt, src)

    def initial(self):
        f = self.ic()
        while True:  # refine until the table stops growing, re-projecting each time
            n0 = f.size
            r = self.adapt(f, coarsen=False, refine=True)
            f = self.ic()
            if r.fval.size == n0:
                break
        self.adapt(f, coarsen=True, refine=False)
        return self.ic()

    def advance(self, f, t):
        """One driver step with adaptation: coarsen, then advance and refine until stable."""
        f = self.adapt(f, coarsen=True, refine=False).fval
        while True:
            f_un = f
            f = self.step(f_un, t)
            r = self.adapt(f, coarsen=False, refine=True)
            f_un = np.concatenate([f_un, np.full(r.added * self.deg ** 2, NEW_ELEMENT_VALUE)])
            if r.added == 0:
                return self.step(f_un, t)
            f = f_un


def test_adaptive_continuity2_rk3_gold():
    ta = np.load(os.path.join(G, "time_advance.npz"))
    rp = Replay("continuity2", 3, 4, 1e-3, "RK3")
    f = rp.initial()
    for i in range(5):
        f = rp.advance(f, i * rp.dt)
        g = ta["continuity2_ad_sg_l3_d4_t%d" % i]
        assert f.size == g.size, (i, f.size, g.size)
        assert np.linalg.norm(f - g) <= 1e-14 * np.linalg.norm(g), i
    assert rp.table.num_elems == 112


def test_adaptive_diffusion2_backward_euler_gold():
    ta = np.load(os.path.join(G, "time_advance.npz"))
    rp = Replay("diffusion2", 3, 4, 1e-4, "BE")
    f = rp.initial()
    assert rp.table.num_elems == 15
    for i in range(5):
        f = rp.step(f, i * rp.dt)
        g = ta["diffusion2_ad_implicit_sg_l3_d4_t%d" % i]
        assert f.size == g.size
        assert np.linalg.norm(f - g) <= 1e-12 * np.linalg.norm(g), i


@pytest.mark.parametrize("levels", [(0, 0), (0, 3), (2, 1), (5, 5)])
def test_rechained_operators_match_truncated_oracle_chain(levels):
    """PDE.rechain_term_mats (native partial terms at max_lev, truncated, multiplied) against
    the oracle's partial terms at max_lev truncated and multiplied, for diffusion2's LDG terms."""
    from asgkron import pdes

    deg = 3
    ppde = pdes.diffusion2(3, case="reference")
    opde = O.diffusion2(3)
    got = ppde.rechain_term_mats(deg, levels, max_lev=6)
    for ti, term in enumerate(opde.terms):
        for d, dim in enumerate(opde.dims):
            n = deg * 2 ** levels[d]
            want = np.eye(n)
            for pt in term[d]:
                want = want @ O.pterm_matrix(deg, dim, pt, 6)[:n, :n]
            assert got[ti][d].shape == (n, n)
            assert np.abs(got[ti][d] - want).max() <= 1e-11 * max(1.0, np.abs(want).max()), (ti, d)


@pytest.mark.parametrize("stem,lev,deg,d", [("continuity1_l4_d3", 4, 3, 1), ("continuity2_l5_d2", 5, 2, 2),
                                            ("continuity3_l4_d4", 4, 4, 3)])
def test_adapt_matches_reference_adapt_gold(stem, lev, deg, d):
    """gold/gold_adapt.m: one coarsening and one refinement (threshold 1e-4, method 1,
    max_lev 8) of a given vector on the SG table; the tables ([levels, cells] rows in
    element order) and vectors are bit-exact.  That generator's adapt.m coarsened only
    elements whose levels are all >= 1 (min_coarsen_level=1); with the current rule every
    level-0 element below the threshold also goes."""
    import asgkron
    from asgkron.adapt import adapt

    z = np.load(os.path.join(G, "adapt.npz"))
    table = asgkron.hash_table_sparse_nD([lev] * d, 8)
    orig = z[stem + "_orig"].reshape(-1)
    for kind, co, rf in (("coarse", True, False), ("refine", False, True)):
        r = adapt(table, orig, deg, 8, 1e-4, coarsen=co, refine=rf, min_coarsen_level=1)
        got = np.hstack([np.asarray(r.table.levels), np.asarray(r.table.cells)]).astype(np.int64)
        want = z["%s_%s_table" % (stem, kind)].reshape(-1, 2 * d).astype(np.int64)
        assert np.array_equal(got, want), kind
        assert np.array_equal(r.fval, z["%s_%s" % (stem, kind)].reshape(-1)), kind
    # the current rule removes the level-0 elements below the threshold as well
    r = adapt(table, orig, deg, 8, 1e-4, coarsen=True, refine=False)
    lv = np.asarray(table.levels)
    f = orig.reshape(lv.shape[0], -1)
    keep = np.abs(f).max(axis=1) > 0.1 * 1e-4 * np.abs(orig).max()
    assert r.table.num_elems == int(keep.sum())
    assert np.array_equal(r.fval, f[keep].ravel())
