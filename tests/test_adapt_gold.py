"""Adaptivity pinned to the reference's adaptation gold (gold/generated-inputs/adapt: one
coarsening and one refinement of given vectors, bit-exact) and its adaptive gold
trajectories.

The product's host pieces under test: ``asgkron.adapt.AdaptiveRun`` (the driver's adaptive
loop), the element rules of ``adapt`` (adapt.m), the element tables (hash_table_sparse_nD
order), the initial-condition projections on adapted tables and the rechained operators of
``PDE.rechain_term_mats`` (get_coeff_mats_rechain.m).  The oracle takes the time steps (the
checker) on each adapted table.

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


def _run(name, lev, deg, thr):
    """The product's AdaptiveRun on the PDE (product spec) and its starting SG table."""
    import asgkron
    from asgkron import pdes
    from asgkron.adapt import AdaptiveRun

    ppde = pdes.continuity2(lev, 0.0) if name == "continuity2" else pdes.diffusion2(lev, case="reference")
    return AdaptiveRun(ppde, deg, asgkron.hash_table_sparse_nD([lev, lev], 8), thr)


def _oracle_step(name, lev, deg, method):
    """The checker's time step on the run's current table: the oracle's apply loop on the
    run's rechained operators, sources / Dirichlet data projected at the run's levels."""
    opde = O.continuity2(lev, LF=0.0) if name == "continuity2" else O.diffusion2(lev)
    dt = opde.dt_fn(opde, 0.01)  # at the starting level, as the driver sets it
    _, blocks = O.operator_two_scale(deg, 8)

    def step(run, f, t):
        for dim, lv in zip(opde.dims, run.levels):
            dim.lev = lv
        idx = run.idx1d.astype(np.int64)
        mats = run.term_mats()
        if name == "diffusion2":
            src = lambda tt: O.boundary_condition_vector(opde, deg, idx, blocks, tt)
        else:
            src = lambda tt: O.md_eval(opde, deg, opde.sources, idx, blocks, tt)
        if method == "BE":
            _, A = O.apply_A_loop(mats, idx, deg, f, build_A=True)
            return O.backward_euler_step(A, f, dt, src(t + dt))
        return O.rk3_step(lambda v: O.apply_A_rows(mats, idx, deg, v), f, t, dt, src)

    return step, dt


def test_adaptive_continuity2_rk3_gold():
    ta = np.load(os.path.join(G, "time_advance.npz"))
    run = _run("continuity2", 3, 4, 1e-3)
    step, dt = _oracle_step("continuity2", 3, 4, "RK3")
    f = run.initial()
    for i in range(5):
        f = run.advance(f, i * dt, step)
        g = ta["continuity2_ad_sg_l3_d4_t%d" % i]
        assert f.size == g.size, (i, f.size, g.size)
        assert np.linalg.norm(f - g) <= 1e-14 * np.linalg.norm(g), i
    assert run.table.num_elems == 112 and run.pde.levels == run.levels


def test_adaptive_diffusion2_backward_euler_gold():
    ta = np.load(os.path.join(G, "time_advance.npz"))
    run = _run("diffusion2", 3, 4, 1e-4)
    step, dt = _oracle_step("diffusion2", 3, 4, "BE")
    f = run.initial()
    assert run.table.num_elems == 15
    for i in range(5):
        f = step(run, f, i * dt)
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


def test_adaptive_run_edge_cases():
    """A zero vector leaves the table alone (adapt.m's refine_threshold <= 0 guard); a step
    that adds nothing is taken once more from the unstepped values on the same table; the
    PDE's levels follow the table."""
    import asgkron
    from asgkron import pdes
    from asgkron.adapt import AdaptiveRun

    pde = pdes.continuity2(2, 0.0)
    table = asgkron.hash_table_sparse_nD([2, 2], 8)
    run = AdaptiveRun(pde, 2, table, 1e-3)
    n0 = run.table.num_elems
    calls = []

    def step(r, f, t):
        calls.append((r.table.num_elems, f.size, t))
        return np.zeros_like(f)

    f = run.advance(np.zeros(n0 * 4), 0.5, step)
    assert run.table.num_elems == n0 and f.size == n0 * 4
    assert calls == [(n0, n0 * 4, 0.5), (n0, n0 * 4, 0.5)]
    assert pde.levels == run.levels == [2, 2]
    mats = run.term_mats()
    assert [m.shape for m in mats[0]] == [(8, 8), (8, 8)]
