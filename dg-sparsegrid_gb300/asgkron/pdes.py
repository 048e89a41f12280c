"""The PDEs of the benchmark configurations, as term/source specifications.

Each follows the reference's pdes/*.m file it names: domains, per-dimension partial terms
(an empty slot is a mass term, MD_TERM.m:23-28), separable sources and initial conditions.
``lev`` overrides every dimension's level, as PDE.m:69 (set_levels) does with opts.lev.
"""
import numpy as np

from . import coeff as _coeff
from . import grid as _grid
from .operators import (boundary_trace, combine_dimensions, div_term, grad_term, mass_term, project_1d, pterm_matrix,
                        term_matrix)


class PDE:
    """bc: separable Dirichlet boundary data [f_1(x, t), ..., f_d(x, t), c(t)] used on every
    'D' side of every partial term (BCL_fList = BCR_fList, as the configurations' PDEs have it)."""

    def __init__(self, name, bounds, lev, terms, sources=(), ic=(), dt_rule=None, bc=None):
        self.name = name
        self.bounds = list(bounds)
        d = len(self.bounds)
        self.levels = [int(lev)] * d if np.isscalar(lev) else [int(v) for v in lev]
        self.terms = [[(sd if sd is not None else [mass_term()]) for sd in t] for t in terms]
        self.sources = list(sources)
        self.ic = list(ic)
        self.dt_rule = dt_rule
        self.bc = bc

    @property
    def num_dims(self):
        return len(self.bounds)

    @property
    def num_terms(self):
        return len(self.terms)

    def dt(self, cfl):
        return self.dt_rule(self, cfl)

    def element_table(self, max_lev=None, grid_type="SG"):
        ml = max_lev if max_lev is not None else max(8, max(self.levels))
        return _grid.hash_table_sparse_nD(self.levels, ml, grid_type)

    def term_mats(self, deg, construction_level=None, builder="native"):
        """pde.terms{t}.terms_1D{d}.mat for every term (get_coeff_mats.m:29-50).  builder
        "native" runs the C++ builder (asg_coeff_matrix_f64: realspace chain, one rotation);
        "numpy" rotates every partial term and solves the mass in wavelet space as the
        reference does.  The two agree to the transform's orthogonality round-off."""
        if builder not in ("numpy", "native"):
            raise ValueError("builder must be 'numpy' or 'native', not %r" % (builder,))
        cache = {}
        out = []
        for t in self.terms:
            row = []
            for d, pts in enumerate(t):
                lo, hi = self.bounds[d]
                lev = self.levels[d] if construction_level is None else construction_level
                key = (d, lev, tuple((p.kind, p.LF, p.bcl, p.bcr, id(p.g)) for p in pts))
                if key not in cache:
                    build = _coeff.term_matrix if builder == "native" else term_matrix
                    cache[key] = build(deg, lo, hi, lev, pts)
                row.append(cache[key])
            out.append(row)
        return out

    def rechain_term_mats(self, deg, levels, max_lev=8, cache=None):
        """pde.terms{t}.terms_1D{d}.mat after adaptation (get_coeff_mats_rechain.m:7-60, with
        max_lev_coeffs): every partial term is built once at max_lev (M \\ L, the native
        builder), truncated to its leading deg 2^levels[d] rows and columns, and the truncated
        factors are multiplied in order.  For single partial terms this equals building at
        levels[d]; for chained (LDG) terms it is what the reference applies after an
        adaptation step.  ``cache`` (a dict) keeps the max-level partial terms between calls."""
        cache = {} if cache is None else cache
        out = []
        for ti, term in enumerate(self.terms):
            row = []
            for d, pts in enumerate(term):
                lo, hi = self.bounds[d]
                n = deg * 2 ** int(levels[d])
                m = None
                for q, pt in enumerate(pts):
                    key = (ti, d, q, deg, max_lev)
                    if key not in cache:
                        cache[key] = _coeff.term_matrix(deg, lo, hi, max_lev, [pt])
                    f = cache[key][:n, :n]
                    m = f.copy() if m is None else m @ f
                row.append(m)
            out.append(row)
        return out

    def _md(self, deg, funcs, idx1d, t):
        out = np.zeros(idx1d.shape[0] * deg ** self.num_dims)
        for fs in funcs:
            vecs = [project_1d(deg, self.levels[d], self.bounds[d][0], self.bounds[d][1], fs[d], t)
                    for d in range(self.num_dims)]
            out += combine_dimensions(deg, vecs, fs[-1](t), idx1d)
        return out

    def source_vector(self, deg, idx1d, t):
        """source_vector.m / md_eval_function.m (separable sources, no mass solve)."""
        return self._md(deg, self.sources, idx1d, t)

    def source_parts(self, deg, idx1d):
        """Spatial parts of the sources (one vector per source) and their time factors,
        so s(t) = sum_s c_s(t) * v_s can be formed on the device each stage."""
        vs = []
        for fs in self.sources:
            vecs = [project_1d(deg, self.levels[d], self.bounds[d][0], self.bounds[d][1], fs[d], 0.0)
                    for d in range(self.num_dims)]
            vs.append(combine_dimensions(deg, vecs, 1.0, idx1d))
        return vs, [fs[-1] for fs in self.sources]

    def initial_condition(self, deg, idx1d, t=0.0):
        return self._md(deg, self.ic, idx1d, t)

    def boundary_parts(self, deg, idx1d, t=0.0):
        """boundary_condition_vector.m:29-193 as (vectors, time factors): for every partial term
        p of dimension d1 with a Dirichlet side, the d1 factor is the boundary flux passed
        through d1's preceding partial terms; each other dimension d2 carries the projection of
        its boundary function times the g of its own p-th partial term, passed through its
        preceding partial terms (the LHS mass matrices are the identity for these terms).  The
        spatial parts are evaluated at t; bc(t) = sum_k c_k(t) v_k."""
        if self.bc is None:
            return [], []
        D = self.num_dims
        vecs, facs = [], []
        pm = {}

        def pmat(d, tt, q):
            key = (d, tt, q)
            if key not in pm:
                lo, hi = self.bounds[d]
                pm[key] = pterm_matrix(deg, lo, hi, self.levels[d], self.terms[tt][d][q])
            return pm[key]

        for tt, term in enumerate(self.terms):
            for d1 in range(D):
                lo1, hi1 = self.bounds[d1]
                for p, pt in enumerate(term[d1]):
                    if pt.kind not in ("div", "grad"):
                        continue
                    for side, kind in (("L", pt.BCL), ("R", pt.BCR)):
                        if kind != "D":
                            continue
                        parts = []
                        for d2 in range(D):
                            if d2 == d1:
                                v = boundary_trace(deg, lo1, hi1, self.levels[d1], pt, self.bc[d1], t, side)
                                for q in range(p - 1, -1, -1):
                                    v = pmat(d1, tt, q) @ v
                            else:
                                lo2, hi2 = self.bounds[d2]
                                g2 = term[d2][p].g
                                f2 = self.bc[d2]
                                v = project_1d(deg, self.levels[d2], lo2, hi2,
                                               lambda x, tt_, f2=f2, g2=g2: f2(x, tt_) * g2(x), t)
                                for q in range(p):
                                    v = pmat(d2, tt, q) @ v
                            parts.append(v)
                        vecs.append(combine_dimensions(deg, parts, 1.0, idx1d))
                        facs.append(self.bc[D])
        return vecs, facs

    def boundary_vector(self, deg, idx1d, t):
        vecs, facs = self.boundary_parts(deg, idx1d, t)
        out = np.zeros(idx1d.shape[0] * deg ** self.num_dims)
        for v, c in zip(vecs, facs):
            out += c(t) * v
        return out

    def forcing_parts(self, deg, idx1d):
        """Sources and boundary data together (the rhs time_advance.m adds to A f each stage)."""
        sv, sf = self.source_parts(deg, idx1d)
        bv, bf = self.boundary_parts(deg, idx1d)
        return sv + bv, sf + bf


def _neg(v):
    return lambda x: 0 * x - v


def continuity2(lev, LF=-1.0):
    """pdes/continuity2.m: x in [-1,1], y in [-2,2]; d/dx and d/dy with g=-1, periodic."""
    pi = np.pi
    terms = [[[div_term(_neg(1.0), LF, "P", "P")], [mass_term()]], [None, [div_term(_neg(1.0), LF, "P", "P")]]]
    sources = [
        [lambda x, t: np.cos(pi * x), lambda y, t: np.sin(2 * pi * y), lambda t: 2 * np.cos(2 * t)],
        [lambda x, t: np.cos(pi * x), lambda y, t: np.cos(2 * pi * y), lambda t: 2 * pi * np.sin(2 * t)],
        [lambda x, t: np.sin(pi * x), lambda y, t: np.sin(2 * pi * y), lambda t: -pi * np.sin(2 * t)],
    ]
    ic = [[lambda x, t: np.cos(pi * x), lambda y, t: np.sin(2 * pi * y), lambda t: np.sin(2 * t)]]
    return PDE("continuity2", [(-1.0, 1.0), (-2.0, 2.0)], lev, terms, sources, ic,
               lambda p, cfl: (p.bounds[0][1] - p.bounds[0][0]) / 2 ** p.levels[0] * cfl)


def continuity3(lev, LF=-1.0):
    """pdes/continuity3.m: [-1,1] x [-2,2] x [-3,3]; one d/dx_k term per dimension, g=-1."""
    pi = np.pi
    terms = [[[div_term(_neg(1.0), LF, "P", "P")] if k == d else None for d in range(3)] for k in range(3)]
    sources = [
        [lambda x, t: np.cos(pi * x), lambda y, t: np.sin(2 * pi * y), lambda z, t: np.cos(2 * pi * z / 3),
         lambda t: 2 * np.cos(2 * t)],
        [lambda x, t: np.cos(pi * x), lambda y, t: np.cos(2 * pi * y), lambda z, t: np.cos(2 * pi * z / 3),
         lambda t: 2 * pi * np.sin(2 * t)],
        [lambda x, t: np.sin(pi * x), lambda y, t: np.sin(2 * pi * y), lambda z, t: np.cos(2 * pi * z / 3),
         lambda t: -pi * np.sin(2 * t)],
        [lambda x, t: np.cos(pi * x), lambda y, t: np.sin(2 * pi * y), lambda z, t: np.sin(2 * pi * z / 3),
         lambda t: -2.0 / 3.0 * pi * np.sin(2 * t)],
    ]
    ic = [[lambda x, t: 0 * x] * 3 + [lambda t: 1.0]]
    return PDE("continuity3", [(-1.0, 1.0), (-2.0, 2.0), (-3.0, 3.0)], lev, terms, sources, ic,
               lambda p, cfl: (p.bounds[0][1] - p.bounds[0][0]) / 2 ** p.levels[0] * cfl)


def continuity6(lev, LF=-1.0):
    """pdes/continuity6.m: six dimensions, d/dx_k with speeds (1,1,3,4,3,2), periodic; the
    manufactured solution cos(pi x) sin(pi y/2) cos(pi z/3) cos(pi vx/10) sin(pi vy/20)
    cos(pi vz/30) sin(2t) gives seven separable sources (continuity6.m:142-221), zero start."""
    bounds = [(-1.0, 1.0), (-2.0, 2.0), (-3.0, 3.0), (-10.0, 10.0), (-20.0, 20.0), (-30.0, 30.0)]
    speeds = [1.0, 1.0, 3.0, 4.0, 3.0, 2.0]
    terms = [[[div_term(_neg(speeds[k]), LF, "P", "P")] if k == d else None for d in range(6)] for k in range(6)]
    pi = np.pi
    freq = [pi, pi / 2, pi / 3, pi / 10, pi / 20, pi / 30]
    sol_is_cos = [True, False, True, True, False, True]

    def factors(swap):  # the solution's spatial factors, dimension ``swap`` cos <-> sin
        out = []
        for k in range(6):
            use_cos = sol_is_cos[k] != (k == swap)
            out.append((lambda a: (lambda x, t: np.cos(a * x)))(freq[k]) if use_cos else
                       (lambda a: (lambda x, t: np.sin(a * x)))(freq[k]))
        return out

    sources = [factors(-1) + [lambda t: 2 * np.cos(2 * t)],
               factors(1) + [lambda t: 0.5 * pi * np.sin(2 * t)],
               factors(0) + [lambda t: -pi * np.sin(2 * t)],
               factors(2) + [lambda t: -pi * np.sin(2 * t)],
               factors(4) + [lambda t: 3.0 / 20.0 * pi * np.sin(2 * t)],
               factors(3) + [lambda t: -2.0 / 5.0 * pi * np.sin(2 * t)],
               factors(5) + [lambda t: -1.0 / 15.0 * pi * np.sin(2 * t)]]
    ic = [[lambda x, t: 0 * x] * 6 + [lambda t: 1.0]]
    return PDE("continuity6", bounds, lev, terms, sources, ic,
               lambda p, cfl: (p.bounds[0][1] - p.bounds[0][0]) / 2 ** p.levels[0] * cfl)


def diffusion2(lev, case="zero_dirichlet"):
    """pdes/diffusion2.m: LDG d2/dx2 + d2/dy2 on [0,1]^2: DIV(+1, N, N) then GRAD(-1, D, D).

    case "reference": the reference file's data -- initial condition and Dirichlet data from
    the solution cos(pi x) cos(pi y) exp(-2 pi^2 t) (diffusion2.m:41-55).
    case "zero_dirichlet": the implicit benchmark configuration -- homogeneous Dirichlet data
    and sin(pi x) sin(pi y) initially.  The operators are the same in both cases (they depend
    on the boundary types only, coeff_matrix.m:212-263)."""
    one = lambda x: 0 * x + 1
    ldg = [div_term(one, 1.0, "N", "N"), grad_term(one, -1.0, "D", "D")]
    terms = [[ldg, [mass_term(), mass_term()]], [[mass_term(), mass_term()], ldg]]
    pi = np.pi
    if case == "reference":
        soln = [lambda x, t: np.cos(pi * x), lambda y, t: np.cos(pi * y), lambda t: np.exp(-2 * pi ** 2 * t)]
        ic, bc = [soln], soln
    elif case == "zero_dirichlet":
        ic, bc = [[lambda x, t: np.sin(pi * x), lambda y, t: np.sin(pi * y), lambda t: 1.0]], None
    else:
        raise ValueError("diffusion2: case must be 'reference' or 'zero_dirichlet'")
    return PDE("diffusion2", [(0.0, 1.0), (0.0, 1.0)], lev, terms, (), ic,
               lambda p, cfl: cfl * (1.0 / 2 ** p.levels[0]) ** 2, bc=bc)
