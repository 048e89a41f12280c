"""Adaptive element tables (adapt.m) and the plan rebuild that follows them.

``adapt`` restates adapt.m's element rules on the dense table arrays:

* thresholds (adapt.m:15-18): refine where max|f_e| >= max|f| * rel, coarsen where
  max|f_e| <= 0.1 * that (and nothing happens when max|f| is zero);
* coarsening (adapt.m:92-200): every element below the coarsening threshold is removed
  with its coefficients; the others keep their order.  adapt.m:108-110 admits every level
  ("level must be >= 0 at present"); an earlier version, the one that wrote
  gold/generated-inputs/adapt, coarsened only elements whose levels are all >= 1
  (``min_coarsen_level=1``);
* refinement (adapt.m:252-340): for each remaining element at or above the refinement
  threshold, its daughters (get_child_elements.m, methods 1 and 2) that are not in the
  table yet are appended, in discovery order, with coefficient value 1e-15.

``AdaptiveRun`` drives the reference's adaptive time loop around a caller's time step.
``rebuild_plan`` builds the plan for a new table; ``update_plan`` instead replaces the table
of an existing plan in place when the operators keep their values.  Its operators are the plan's own
(single partial terms are level-independent, so operators built at the maximum level serve
every table) or, for chained partial terms, the ones ``PDE.rechain_term_mats`` forms at the
new table's levels, as adapt.m:417-437 does through get_coeff_mats_rechain.m.  Plan creation
is the whole cost of an adaptation step on the device side: structure analysis, work list,
uploads.
"""
import numpy as np

from .grid import ElementTable, element_idx1d

NEW_ELEMENT_VALUE = 1e-15  # adapt.m:20


def child_elements(lev, pos, max_lev, method=1):
    """Daughters of one element (get_child_elements.m): per dimension d, (lev+1, 2 pos) and,
    when lev_d >= 1, (lev+1, 2 pos + 1), each only while lev_d + 1 < max_lev; method 2 adds the
    combinations of the 1-D daughters across dimensions.  Returns [(lev tuple, pos tuple)]."""
    lev = [int(v) for v in lev]
    pos = [int(v) for v in pos]
    d = len(lev)
    out = []
    new_1d = [[] for _ in range(d)]
    for k in range(d):
        if lev[k] + 1 < max_lev:
            l2, p2 = list(lev), list(pos)
            l2[k] += 1
            p2[k] = 2 * pos[k]
            out.append((tuple(l2), tuple(p2)))
            new_1d[k].append((l2[k], p2[k]))
            if lev[k] >= 1:
                l3, p3 = list(lev), list(pos)
                l3[k] += 1
                p3[k] = 2 * pos[k] + 1
                out.append((tuple(l3), tuple(p3)))
                new_1d[k].append((l3[k], p3[k]))
    if method == 2 and all(new_1d):
        # every combination of the 1-D daughters (the tensor-product children)
        combos = [[]]
        for k in range(d):
            combos = [c + [v] for c in combos for v in new_1d[k]]
        for c in combos:
            out.append((tuple(v[0] for v in c), tuple(v[1] for v in c)))
    return out


def md_keys(levels, cells, max_lev):
    """0-based md keys (md_lev_pos_to_idx.m minus one): sum_d (idx1d_d - 1) * 2^(max_lev d)."""
    idx = element_idx1d(levels, cells).astype(np.uint64) - 1
    key = np.zeros(idx.shape[0], dtype=np.uint64)
    for k in range(idx.shape[1]):
        key += idx[:, k] << np.uint64(max_lev * k)
    return key


class AdaptResult:
    def __init__(self, table, fval, removed, added):
        self.table = table        # the new ElementTable
        self.fval = fval          # coefficients on the new table
        self.removed = removed    # indices (into the old table) of removed elements
        self.added = added        # number of appended elements


def adapt(table, fval, deg, max_lev, rel_threshold, coarsen=True, refine=True, method=1, min_coarsen_level=0):
    """One adaptation step of adapt.m on an element table and its coefficient vector.
    Elements with a level below ``min_coarsen_level`` in some dimension are never removed."""
    levels = np.asarray(table.levels, dtype=np.int32)
    cells = np.asarray(table.cells, dtype=np.int32)
    N, d = levels.shape
    B = deg ** d
    f = np.asarray(fval, dtype=np.float64).reshape(N, B)
    if levels.size and int(levels.max()) > max_lev:
        raise ValueError("adapt: element level above max_lev=%d" % max_lev)
    refine_thr = float(np.abs(f).max()) * rel_threshold if N else 0.0
    coarsen_thr = 0.1 * refine_thr
    if refine_thr <= 0:
        coarsen = refine = False
    emax = np.abs(f).max(axis=1) if N else np.zeros(0)
    removable = (emax <= coarsen_thr) & (levels.min(axis=1, initial=max_lev) >= min_coarsen_level)
    removed = np.nonzero(removable)[0] if coarsen else np.zeros(0, dtype=np.int64)
    keep = np.ones(N, dtype=bool)
    keep[removed] = False
    levels, cells, f, emax = levels[keep], cells[keep], f[keep], emax[keep]
    added_lev, added_pos = [], []
    if refine:
        present = {(tuple(l), tuple(c)) for l, c in zip(levels.tolist(), cells.tolist())}
        for n in np.nonzero(emax >= refine_thr)[0]:
            for child in child_elements(levels[n], cells[n], max_lev, method):
                if child not in present:
                    present.add(child)
                    added_lev.append(child[0])
                    added_pos.append(child[1])
    if added_lev:
        levels = np.vstack([levels, np.array(added_lev, dtype=np.int32)])
        cells = np.vstack([cells, np.array(added_pos, dtype=np.int32)])
        f = np.vstack([f, np.full((len(added_lev), B), NEW_ELEMENT_VALUE)])
    new = ElementTable(np.ascontiguousarray(levels), np.ascontiguousarray(cells),
                       md_keys(levels, cells, max_lev) if levels.shape[0] else np.zeros(0, dtype=np.uint64))
    return AdaptResult(new, f.reshape(-1), removed, len(added_lev))


def table_levels(table):
    """Highest level present in each dimension (adapt.m:417-421)."""
    lv = np.asarray(table.levels)
    return [int(v) for v in lv.max(axis=0)] if lv.size else []


def operator_extent(term_mats, deg):
    """Blocks per side of the operators on each dimension (their full extent: operators built at
    the maximum level cover every table the run can reach)."""
    return [min(int(row[m].shape[0]) for row in term_mats) // deg for m in range(len(term_mats[0]))]


def rebuild_plan(plan, table, pairs=None, term_mats=None, reserve=False, **kw):
    """A new plan for the adapted table with the work model of ``plan`` and its operators, or
    ``term_mats`` (e.g. ``pde.rechain_term_mats(deg, table_levels(table))``).  ``reserve``
    packs the operators' full extent, so that ``update_plan`` can follow later tables."""
    from .api import Plan

    structure = kw.pop("structure", plan.structure)
    mats = plan.term_mats if term_mats is None else term_mats
    ob = operator_extent(mats, plan.deg) if reserve else None
    return Plan.create(mats, table.idx1d(), plan.deg, pairs=pairs, structure=structure, op_blocks=ob, **kw)


def update_plan(plan, table, pairs=None, term_mats=None):
    """The plan for the adapted table on the same operator values (single partial terms: the
    operator of a coarser level is the leading block of a finer one, so values never change,
    only the extent the table reaches): the element table and work list are replaced in place
    (asg_plan_update_elements; the operators' analysis, packing and device copies are kept).
    When the table reaches beyond the plan's packed operators, a new plan is built from
    ``term_mats`` (default: the plan's own), reserving their full extent.  Returns the plan to
    use (``plan`` itself, or the new one; the old one is then closed)."""
    from ._lib import ASG_ERR_CAPACITY, AsgError

    try:
        plan.update_elements(table.idx1d(), pairs)
        return plan
    except AsgError as e:
        if e.status != ASG_ERR_CAPACITY:
            raise
    new = rebuild_plan(plan, table, pairs=pairs, term_mats=term_mats, reserve=True)
    plan.close()
    return new


class AdaptiveRun:
    """The reference's adaptive time loop on the host (gold/gold_time_advance.m:291-362,
    adapt.m): the element table, the PDE's levels and the coefficient vector evolve here;
    the time step is the caller's ``step(run, f, t) -> f`` on ``run.table`` with
    ``run.term_mats()`` (a GPU stepper on a plan rebuilt by ``rebuild_plan``, or any other).

    The PDE object is updated in place: its levels follow the table (adapt.m:417-425), so
    its projections (initial condition, sources, boundary data) cover every element."""

    def __init__(self, pde, deg, table, threshold, max_lev=8, method=1, min_coarsen_level=0):
        self.pde, self.deg, self.threshold, self.max_lev = pde, deg, threshold, max_lev
        self.method, self.min_coarsen_level = method, min_coarsen_level
        self._pterms = {}
        self.set_table(table)

    def set_table(self, table):
        self.table = table
        self.levels = table_levels(table)
        self.pde.levels = list(self.levels)
        self.idx1d = table.idx1d()

    def term_mats(self):
        """The operators for the current table: partial terms rechained at its levels."""
        return self.pde.rechain_term_mats(self.deg, self.levels, self.max_lev, self._pterms)

    def adapt(self, f, coarsen, refine):
        r = adapt(self.table, f, self.deg, self.max_lev, self.threshold, coarsen=coarsen, refine=refine,
                  method=self.method, min_coarsen_level=self.min_coarsen_level)
        self.set_table(r.table)
        return r

    def initial(self, t=0.0):
        """The initial condition on an adapted table: refine and re-project until the table
        stops growing, then coarsen and re-project (gold_time_advance.m:291-313)."""
        f = self.pde.initial_condition(self.deg, self.idx1d, t)
        while True:
            n0 = f.size
            r = self.adapt(f, coarsen=False, refine=True)
            f = self.pde.initial_condition(self.deg, self.idx1d, t)
            if r.fval.size == n0:
                break
        self.adapt(f, coarsen=True, refine=False)
        return self.pde.initial_condition(self.deg, self.idx1d, t)

    def advance(self, f, t, step):
        """One step with adaptation (gold_time_advance.m:318-360): coarsen, advance, refine
        from the advanced values; while elements were added, advance again from the
        unstepped values extended to the refined table (new elements at 1e-15)."""
        f = self.adapt(f, coarsen=True, refine=False).fval
        block = self.deg ** len(self.levels)
        while True:
            f_un = np.asarray(f, dtype=np.float64).reshape(-1)
            f = step(self, f_un, t)
            r = self.adapt(f, coarsen=False, refine=True)
            f_un = np.concatenate([f_un, np.full(r.added * block, NEW_ELEMENT_VALUE)])
            if r.added == 0:
                return step(self, f_un, t)
            f = f_un
