"""CPU oracle: a plain numpy restatement of the MATLAB ASGarD prototype's ``apply_A`` path.

TEST INFRASTRUCTURE ONLY.  Nothing in the product (the CUDA library, its C ABI or the Python
host mirror) imports this module; only ``tests/``, ``__graft_entry__.smoke()`` and the CPU
baseline leg of ``bench.py`` may use it, and only as the checker.

Every function cites the reference file:line it follows (paths within project-asgard/
DG-SparseGrid).  Indices follow the reference's 1-based conventions where the reference
exposes them (1-D indices, element ids in connectivity lists) and are converted explicitly
where numpy needs 0-based offsets.

Parity pins (see ``tests/test_oracle_gold.py``): element tables, connectivity and
permutations bit-exact against the gold ``.dat`` files; quadrature/two-scale to round-off;
the RK3 trajectories ``continuity{1,2,3}_sg_*`` to ~1e-14 relative with central flux
(LF=0), which is how those gold files were generated.
"""
import os

import numpy as np

_GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "..", "tests", "golden")
EPS = np.finfo(np.float64).eps


# ------------------------------------------------------------------------------------------
# L0 numerics
# ------------------------------------------------------------------------------------------
def lgwt(N, a, b):
    """Legendre-Gauss nodes/weights by Newton iteration (Quadrature/lgwt.m:1-59)."""
    N = N - 1
    N1, N2 = N + 1, N + 2
    xu = np.linspace(-1.0, 1.0, N1)
    y = np.cos((2 * np.arange(N + 1) + 1) * np.pi / (2 * N + 2)) + (0.27 / N1) * np.sin(np.pi * xu * N / N2)
    L = np.zeros((N1, N2))
    y0 = 2.0
    Lp = None
    while np.max(np.abs(y - y0)) > EPS:
        L[:, 0] = 1.0
        L[:, 1] = y
        for k in range(2, N1 + 1):
            L[:, k] = ((2 * k - 1) * y * L[:, k - 1] - (k - 1) * L[:, k - 2]) / k
        Lp = N1 * (L[:, N1 - 1] - y * L[:, N2 - 1]) / (1 - y ** 2)
        y0 = y
        y = y0 - L[:, N2 - 1] / Lp
    x = (a * (1 - y) + b * (1 + y)) / 2
    w = (b - a) / ((1 - y ** 2) * Lp ** 2)
    return x[::-1].copy(), w[::-1].copy()


def default_quad_number(deg):
    """Quadrature/default_quad_number.m:2."""
    return max(deg + 1, 10)


def _legendre_p(n, x):
    x = np.asarray(x, dtype=np.float64)
    p0 = np.ones_like(x)
    if n == 0:
        return p0
    p1 = x.copy()
    for k in range(2, n + 1):
        p0, p1 = p1, ((2 * k - 1) * x * p1 - (k - 1) * p0) / k
    return p1


def lin_legendre(x, k):
    """Normalised Legendre values sqrt(2n+1)*P_n(x), zero outside [-1,1] (DG_loc/lin_legendre.m:8-13)."""
    x = np.atleast_1d(np.asarray(x, dtype=np.float64)).reshape(-1)
    v = np.zeros((x.size, k))
    for kk in range(k):
        v[:, kk] = _legendre_p(kk, x) * np.sqrt(2 * kk + 1)
    v[x > 1, :] = 0.0
    v[x < -1, :] = 0.0
    return v


def lin_dlegendre(x, k):
    """Derivatives via dP_n = n P_{n-1} + x dP_{n-1} (DG_loc/lin_dlegendre.m:4-20)."""
    x = np.atleast_1d(np.asarray(x, dtype=np.float64)).reshape(-1)

    def dlg(n):
        if n == 0:
            return x * 0.0
        return n * _legendre_p(n - 1, x) + x * dlg(n - 1)

    v = np.zeros((x.size, k))
    for kk in range(k):
        v[:, kk] = dlg(kk) * np.sqrt(2 * kk + 1)
    return v


# ------------------------------------------------------------------------------------------
# Two-scale multiwavelet transform (two_scale/OperatorTwoScale_wavelet2.m)
# ------------------------------------------------------------------------------------------
_TS_CACHE = {}


def two_scale_filters(deg):
    """H0, G0 as loaded from two_scale_rel_<deg>.mat (OperatorTwoScale_wavelet2.m:18-26)."""
    if not _TS_CACHE:
        z = np.load(os.path.join(_GOLD, "two_scale_rel.npz"))
        _TS_CACHE.update({k: z[k] for k in z.files})
    return _TS_CACHE["H0_%d" % deg].copy(), _TS_CACHE["G0_%d" % deg].copy()


def operator_two_scale(deg, nlev):
    """FMWT matrix and its blocks (OperatorTwoScale_wavelet2.m:34-144).

    ``blocks`` is a 0-based list: blocks[b] is MATLAB's blocks{b+1}."""
    if nlev == 0:
        return np.eye(deg), []
    H0, G0 = two_scale_filters(deg)
    tol = 1e4 * EPS
    H0[np.abs(H0) < tol] = 0.0
    G0[np.abs(G0) < tol] = 0.0
    jx = np.arange(1, deg + 1)[:, None]
    jy = np.arange(1, deg + 1)[None, :]
    H1 = ((-1.0) ** (jx + jy - 2)) * H0
    G1 = ((-1.0) ** (deg + jx + jy - 2)) * G0
    n = deg * 2 ** nlev
    Gmat = np.zeros((deg, n))
    Hmat = np.zeros((deg, n))
    Hmat[:, :deg] = np.eye(deg)
    blocks = [None] * (2 * nlev)
    for j in range(nlev - 1, -1, -1):
        ncells = 2 ** j
        isize = n // ncells
        isizeh = isize // 2
        Htmp = Hmat[:, :isizeh].copy()
        Gmat[:, :isizeh] = G0 @ Htmp
        Gmat[:, isizeh:isize] = G1 @ Htmp
        Hmat[:, :isizeh] = H0 @ Htmp
        Hmat[:, isizeh:isize] = H1 @ Htmp
        blocks[(j + 1) * 2 - 1] = Gmat[:, :isize].copy()
        h_cols = n if j == 0 else isize
        blocks[j * 2] = Hmat[:, :h_cols].copy()
    FMWT = np.zeros((n, n))
    FMWT[:deg, :n] = blocks[0]
    irow = deg
    for j in range(nlev):
        ncells = 2 ** j
        isize = n // ncells
        Fmat = blocks[1 + j * 2]
        for icell in range(ncells):
            j1 = icell * isize
            i1 = icell * deg + irow
            FMWT[i1:i1 + deg, j1:j1 + isize] = Fmat[:, :isize]
        irow += deg * ncells
    return FMWT, blocks


def apply_fmwt_blocks(level, blocks, X, side="LN"):
    """Apply the level-``level`` transform from max-level blocks (two_scale/apply_FMWT_blocks.m)."""
    if level == 0:
        return X.copy()
    max_level = len(blocks) // 2
    deg = blocks[0].shape[0]
    n = deg * 2 ** level
    X = np.asarray(X, dtype=np.float64)
    vec = X.ndim == 1
    if vec:
        X = X[:, None]
    left = side in ("LN", "LT")
    trans = side in ("LT", "RT")
    cols = X.shape[1]
    Y = np.zeros((n, cols)) if left else np.zeros((X.shape[0], n))
    first = blocks[(max_level - level) * 2]
    if left:
        if trans:
            Y[:n, :] = first.T @ X[:deg, :]
        else:
            Y[:deg, :] = first @ X[:n, :]
    else:
        if trans:
            Y[:, :deg] = X[:, :n] @ first.T
        else:
            Y[:, :n] = X[:, :deg] @ first
    off = (max_level - level) * 2
    ds = deg
    for i in range(level):
        num_cells = 2 ** i
        cell = n // num_cells
        block = blocks[off + i * 2 + 1]
        for j in range(num_cells):
            cs = j * cell
            if left:
                if trans:
                    Y[cs:cs + cell, :] += block.T @ X[ds:ds + deg, :]
                else:
                    Y[ds:ds + deg, :] += block @ X[cs:cs + cell, :]
            else:
                if trans:
                    Y[:, ds:ds + deg] += X[:, cs:cs + cell] @ block.T
                else:
                    Y[:, cs:cs + cell] += X[:, ds:ds + deg] @ block
            ds += deg
    return Y[:, 0] if vec else Y


# ------------------------------------------------------------------------------------------
# PDE term specification (PARTIAL_SD_TERM.m, DIV.m, GRAD.m, MASS.m, MD_TERM.m)
# ------------------------------------------------------------------------------------------
class PTerm:
    """One partial term: type 'mass' | 'div' | 'grad' with coefficient g(x) and flux/BCs."""

    def __init__(self, ptype, g=None, LF=0.0, BCL="N", BCR="N"):
        self.type = ptype
        self.g = g if g is not None else (lambda x: 0.0 * x + 1.0)
        self.LF = LF
        self.BCL = BCL
        self.BCR = BCR
        self.IBCL, self.IBCR = BCL, BCR
        if ptype == "grad":  # GRAD.m:14-34: flip the flux sign and swap D<->N
            swap = {"D": "N", "N": "D"}
            self.IBCL = swap.get(BCL, BCL)
            self.IBCR = swap.get(BCR, BCR)
            self.LF = -LF


def MASS(g=None):
    return PTerm("mass", g)


def DIV(g, LF, BCL, BCR):
    return PTerm("div", g, LF, BCL, BCR)


def GRAD(g, LF, BCL, BCR):
    return PTerm("grad", g, LF, BCL, BCR)


class Dim:
    def __init__(self, lo, hi, lev=3):
        self.min, self.max, self.lev = lo, hi, lev


class PDESpec:
    """dims: list of Dim; terms: list of per-dim lists of PTerm lists (None -> MASS, MD_TERM.m:23-28)."""

    def __init__(self, dims, terms, sources, ic, dt_fn):
        self.dims = dims
        self.terms = [[(sd if sd is not None else [MASS()]) for sd in t] for t in terms]
        self.sources = sources
        self.ic = ic
        self.dt_fn = dt_fn


# ------------------------------------------------------------------------------------------
# 1-D operators (coeff_matrix.m, pterm_coeff_matrix.m, sd_term_coeff_matrix.m)
# ------------------------------------------------------------------------------------------
def coeff_matrix(deg, dim, pterm, coeff_level, t=0.0):
    """Wavelet-space DG matrix of one partial term (coeff_matrix.m:1-344, dense restatement)."""
    lev = coeff_level
    N = 2 ** lev
    h = (dim.max - dim.min) / N
    dof = deg * N
    qx, qw = lgwt(default_quad_number(deg), -1, 1)
    p_L = lin_legendre(-1.0, deg) / np.sqrt(h)  # 1 x deg
    p_R = lin_legendre(1.0, deg) / np.sqrt(h)
    p_val = lin_legendre(qx, deg) / np.sqrt(h)
    Dp_val = lin_dlegendre(qx, deg) / np.sqrt(h) * 2 / h
    J = h / 2
    mass = np.zeros((dof, dof))
    div = np.zeros((dof, dof))
    LF = pterm.LF
    pLt = (-p_L).T  # deg x 1
    pRt = p_R.T
    for i in range(N):
        xL = dim.min + i * h
        xR = xL + h
        c = np.arange(deg * i, deg * (i + 1))
        qxi = ((qx + 1) / 2 + i) * h + dim.min
        G1 = pterm.g(qxi) * 1.0  # dV = 1 for every term of the configs
        val_mass = p_val.T @ (G1[:, None] * p_val * qw[:, None]) * J
        val_div = -Dp_val.T @ (G1[:, None] * p_val * qw[:, None]) * J
        mass[np.ix_(c, c)] += val_mass
        div[np.ix_(c, c)] += val_div
        if pterm.type in ("div", "grad"):
            FCL = float(pterm.g(np.array([xL]))[0])
            FCR = float(pterm.g(np.array([xR]))[0])
            blk = [
                pLt * FCL @ p_R / 2 + LF * abs(FCL) / 2 * pLt @ p_R,
                pLt * FCL @ p_L / 2 + LF * abs(FCL) / 2 * pLt @ (-p_L),
                pRt * FCR @ p_R / 2 + LF * abs(FCR) / 2 * pRt @ p_R,
                pRt * FCR @ p_L / 2 + LF * abs(FCR) / 2 * pRt @ (-p_L),
            ]
            Z = np.zeros((deg, deg))
            if pterm.IBCL == "D" and i == 0:
                blk[0], blk[1] = Z, Z
            if pterm.IBCR == "D" and i == N - 1:
                blk[2], blk[3] = Z, Z
            if pterm.IBCL == "N" and i == 0:
                blk[0] = Z
                blk[1] = pLt * FCL @ p_L
            if pterm.IBCR == "N" and i == N - 1:
                blk[2] = pRt * FCR @ p_R
                blk[3] = Z
            colblk = [c - deg, c, c, c + deg]
            # coeff_matrix.m:271-283 drops the left neighbour at i == 0 and the right one at
            # i == N - 1; on a single cell both go (the reference's sparse(..., dof_1D, dof_1D)
            # would reject the right one, and with max_lev_coeffs it truncates max-level
            # matrices instead, which equals this single-cell build)
            use = [b for b in (0, 1, 2, 3) if not (b == 0 and i == 0) and not (b == 3 and i == N - 1)]
            if pterm.IBCL == "P" or pterm.IBCR == "P":
                if lev >= 1:
                    if i == 0:
                        colblk[0] = np.arange(deg * (N - 1), deg * N)
                    if i == N - 1:
                        colblk[3] = np.arange(0, deg)
                else:
                    colblk = [c, c, c, c]
                use = [0, 1, 2, 3]
            for b in use:
                div[np.ix_(c, colblk[b])] += blk[b]
    grad = -div.T
    FMWT, _ = operator_two_scale(deg, coeff_level)
    if pterm.type == "div":
        m = div
    elif pterm.type == "grad":
        m = grad
    else:
        m = mass
    return FMWT @ m @ FMWT.T


def pterm_matrix(deg, dim, pterm, coeff_level):
    """LHS-mass-solved partial term ``M \\ L`` (pterm_coeff_matrix.m:6-20)."""
    L = coeff_matrix(deg, dim, pterm, coeff_level)
    M = coeff_matrix(deg, dim, MASS(), coeff_level)
    return np.linalg.solve(M, L)


def sd_term_matrix(deg, dim, pterms, coeff_level):
    """Chain of partial terms ``eye * P1 * P2 ...`` (sd_term_coeff_matrix.m:9-22)."""
    mats = [pterm_matrix(deg, dim, pt, coeff_level) for pt in pterms]
    m = np.eye(mats[0].shape[0])
    for x in mats:
        m = m @ x
    return m


def build_term_mats(pde, deg, coeff_level=None):
    """pde.terms{t}.terms_1D{d}.mat for all terms (get_coeff_mats.m:29-50).

    ``coeff_level=None`` builds each dimension at its own level (``max_lev_coeffs`` off);
    an integer builds every dimension at that level (gold generation sets it)."""
    out = []
    for t in pde.terms:
        row = []
        for d, dim in enumerate(pde.dims):
            lev = dim.lev if coeff_level is None else coeff_level
            row.append(sd_term_matrix(deg, dim, t[d], lev))
        out.append(row)
    return out


# ------------------------------------------------------------------------------------------
# Element tables (hash_table_sparse_nD.m + PERMUTE/*) and 1-D index maps
# ------------------------------------------------------------------------------------------
def perm_eq_d_count(idim, levmax, s):
    """PERMUTE/perm_eq_d_count.m."""
    if idim == 1:
        return 1 if levmax[0] >= s else 0
    return sum(perm_eq_d_count(idim - 1, levmax[:idim - 1], s - il) for il in range(0, min(levmax[idim - 1], s) + 1))


def perm_eq_d(idim, levmax, s, last_index_decreasing=False):
    """Tuples with sum == s and t_i <= levmax[i] (PERMUTE/perm_eq_d.m:45-80)."""
    if idim == 1:
        return [(s,)] if levmax[0] >= s else []
    rng = range(0, min(levmax[idim - 1], s) + 1)
    if last_index_decreasing:
        rng = reversed(list(rng))
    out = []
    for il in rng:
        for tup in perm_eq_d(idim - 1, levmax[:idim - 1], s - il, last_index_decreasing):
            out.append(tup + (il,))
    return out


def perm_leq_d(idim, levmax, summax, increasing_sum_order=False):
    """Tuples with sum <= summax, sums walked downward by default (PERMUTE/perm_leq_d.m:26-45)."""
    sums = range(0, summax + 1) if increasing_sum_order else range(summax, -1, -1)
    out = []
    for s in sums:
        out.extend(perm_eq_d(idim, levmax, s))
    return out


def perm_leq_d_count(idim, levmax, summax):
    return sum(perm_eq_d_count(idim, levmax, s) for s in range(summax + 1))


def perm_max(idim, levmax, last_index_decreasing=False):
    """Full-grid level tuples (PERMUTE/perm_max.m)."""
    if idim == 1:
        r = list(range(levmax[0] + 1))
        return [(v,) for v in (reversed(r) if last_index_decreasing else r)]
    n = levmax[idim - 1]
    inner = perm_max(idim - 1, levmax, last_index_decreasing)
    out = []
    for i in range(n + 1):
        v = n - i if last_index_decreasing else i
        for tup in inner:
            out.append(tup[:idim - 1] + (v,))
    return out


def perm_eq(idim, n, last_index_decreasing=False):
    """PERMUTE/perm_eq.m."""
    if idim == 1:
        return [(n,)]
    out = []
    for i in range(n + 1):
        if last_index_decreasing:
            for tup in perm_eq(idim - 1, i, True):
                out.append(tup + (n - i,))
        else:
            for tup in perm_eq(idim - 1, n - i, False):
                out.append(tup + (i,))
    return out


def perm_leq(idim, n, order_by_n=False):
    """PERMUTE/perm_leq.m (the old hash's increasing order)."""
    if order_by_n:
        out = []
        for i in range(n + 1):
            out.extend(perm_eq(idim, i))
        return out
    if idim == 1:
        return [(v,) for v in range(n + 1)]
    out = []
    for i in range(n + 1):
        for tup in perm_leq(idim - 1, n - i, order_by_n):
            out.append(tup + (i,))
    return out


def lev_cell_to_1d_index(lev, cell):
    """1-based 1-D index 2^(lev-1)+cell+1, or 1 at level 0 (lev_cell_to_1D_index.m:6-9)."""
    lev = np.asarray(lev)
    cell = np.asarray(cell)
    idx = np.where(lev == 0, 1, (2.0 ** (lev - 1)).astype(np.int64) + cell + 1)
    return idx.astype(np.int64)


def lev_cell_index_set(levels):
    """Cell tuples of one level tuple, dim 1 fastest (lev_cell_to_1D_index_set.m:10-30)."""
    sizes = [2 ** max(0, l - 1) for l in levels]
    grids = np.indices(sizes[::-1]).reshape(len(levels), -1)[::-1].T
    return grids  # rows: cell tuples, dim 0 varies fastest


def md_lev_pos_to_idx(levels, cells, max_lev):
    """uint64 element key 1 + sum (idx1D-1) * 2^(max_lev*(d-1)) (md_lev_pos_to_idx.m:10-26)."""
    idx = 1
    stride = 1
    for l, c in zip(levels, cells):
        assert l <= max_lev
        idx += (int(lev_cell_to_1d_index(l, c)) - 1) * stride
        stride *= 2 ** max_lev
    return idx


def hash_table_sparse_nd(lev_vec, max_lev, grid_type="SG"):
    """Element table in the new-hash order (hash_table_sparse_nD.m:35-116).

    Returns (levels[N,d], cells[N,d], ids[N]) with ids the uint64 md-index keys."""
    d = len(lev_vec)
    if grid_type == "SG":
        ptable = perm_leq_d(d, list(lev_vec), max(lev_vec))
    else:
        ptable = perm_max(d, list(lev_vec))
    levs, cells, ids = [], [], []
    for lv in ptable:
        for cs in lev_cell_index_set(lv):
            levs.append(lv)
            cells.append(tuple(int(c) for c in cs))
            ids.append(md_lev_pos_to_idx(lv, cs, max_lev))
    return np.array(levs, dtype=np.int64).reshape(-1, d), np.array(cells, dtype=np.int64).reshape(-1, d), np.array(ids, dtype=np.uint64)


def hash_table_nd(lev, d, grid_type="SG"):
    """Old string-keyed hash order (hash_table_nD.m:29-136): returns (levels, cells)."""
    ptable = perm_leq(d, lev) if grid_type == "SG" else perm_max(d, [lev] * d)
    levs, cells = [], []
    for lv in ptable:
        for cs in lev_cell_index_set(lv):
            levs.append(lv)
            cells.append(tuple(int(c) for c in cs))
    return np.array(levs, dtype=np.int64).reshape(-1, d), np.array(cells, dtype=np.int64).reshape(-1, d)


def element_idx1d(levels, cells):
    """A_data.element_local_index_D{d}: 1-based 1-D index per element and dim (global_matrix.m:31-70)."""
    return lev_cell_to_1d_index(levels, cells)


# ------------------------------------------------------------------------------------------
# Connectivity (connect_1D.m, connect_nD.m, PERMUTE/index_leq_max.m, index_max.m)
# ------------------------------------------------------------------------------------------
def connect_1d(Lev):
    """Dense 2^Lev x 2^Lev 0/1 matrix (connect_1D.m:8-50); indices 1-based in the reference."""
    n = 2 ** Lev
    C = np.zeros((n, n), dtype=np.int64)

    def idx(l, c):
        return int(lev_cell_to_1d_index(l, c)) - 1

    for Lx in range(Lev + 1):
        ncx = 2 ** max(0, Lx - 1)
        for Px in range(ncx):
            I = idx(Lx, Px)
            for q in range(max(Px - 1, 0), min(Px + 1, ncx - 1) + 1):
                J = idx(Lx, q)
                C[I, J] = 1
                C[J, I] = 1
            if Px == 0:
                e = idx(Lx, ncx - 1)
                C[I, e] = 1
                C[e, I] = 1
            elif Px == ncx - 1:
                b = idx(Lx, 0)
                C[I, b] = 1
                C[b, I] = 1
            for Ly in range(Lx + 1, Lev + 1):
                nL = Ly - Lx
                ncy = 2 ** (Ly - 1)
                if Lx > 0:
                    py = list(range(max(2 ** nL * Px - 1, 0), min(2 ** nL * Px + 2 ** nL, ncy - 1) + 1))
                else:
                    py = list(range(max(2 ** (nL - 1) * Px - 1, 0), min(2 ** (nL - 1) * Px + 2 ** (nL - 1), ncy - 1) + 1))
                py = [0] + py + [2 ** max(0, Ly - 1) - 1]
                for q in py:
                    J = idx(Ly, q)
                    C[I, J] = 1
                    C[J, I] = 1
    return C


def index_leq_max(ndim, nmat, levsum, levmax):
    """0-based index tuples (last dim slowest) with sum <= levsum, max <= levmax (index_leq_max.m:15-49)."""
    if ndim == 1:
        v = nmat[0]
        return [(i,) for i in range(len(v)) if v[i] <= levsum and v[i] <= levmax]
    out = []
    v = nmat[ndim - 1]
    for i in range(len(v)):
        if v[i] <= levmax:
            for tup in index_leq_max(ndim - 1, nmat, levsum - v[i], levmax):
                out.append(tup + (i,))
    return out


def index_max(ndim, nmat, levmax):
    """index_max.m."""
    if ndim == 1:
        return [(i,) for i in range(len(nmat[0])) if nmat[0][i] <= levmax]
    inner = index_max(ndim - 1, nmat, levmax)
    out = []
    v = nmat[ndim - 1]
    for i in range(len(v)):
        if v[i] <= levmax:
            out.extend(t + (i,) for t in inner)
    return out


def connect_nd(ndim, levels, cells, levsum, levmax, grid_type="SG"):
    """Per-element sorted 1-based connected element lists (connect_nD.m:34-105).

    ``levels``/``cells`` are the element table (any order); lookups go through a dict in
    place of the reference's string-keyed struct."""
    Lev = max(levsum, levmax)
    c1 = connect_1d(Lev)
    key1d = []
    for Lx in range(Lev + 1):
        for Px in range(2 ** max(0, Lx - 1)):
            key1d.append((Lx, Px))
    key1d = np.array(key1d)
    lookup = {}
    for e in range(levels.shape[0]):
        lookup[tuple(levels[e]) + tuple(cells[e])] = e + 1
    idx1 = element_idx1d(levels, cells)
    conn = []
    for e in range(levels.shape[0]):
        lev_arr, cell_arr = [], []
        for dd in range(ndim):
            js = np.nonzero(c1[idx1[e, dd] - 1, :])[0]
            lev_arr.append(key1d[js, 0])
            cell_arr.append(key1d[js, 1])
        if grid_type == "SG":
            res = index_leq_max(ndim, lev_arr, levsum, levmax)
        else:
            res = index_max(ndim, lev_arr, levmax)
        ids = []
        for tup in res:
            key = tuple(int(lev_arr[dd][tup[dd]]) for dd in range(ndim)) + tuple(int(cell_arr[dd][tup[dd]]) for dd in range(ndim))
            ids.append(lookup[key])
        conn.append(np.sort(np.array(ids, dtype=np.int64)))
    return conn


# ------------------------------------------------------------------------------------------
# Kronecker products (kron_multd.m, Kronmult/kronmult{1..6}.m, krond.m)
# ------------------------------------------------------------------------------------------
def krond(mats):
    """kron(A1, kron(A2, ...)) (krond.m:7-17)."""
    out = mats[0]
    for m in mats[1:]:
        out = np.kron(out, m)
    return out


def kronmult(mats, X):
    """Method-1 mode-product chain of kronmult{n}.m: apply A_n to the fastest index first,
    then A_{n-1}, ..., A_1 (kronmult1.m:17, kronmult2.m:66-139, kronmult3.m:47-88).

    X is a column-major vector (or matrix of nvec columns) of length prod(ncol)."""
    ncol = [m.shape[1] for m in mats]
    nrow = [m.shape[0] for m in mats]
    X = np.asarray(X)
    nvec = X.size // int(np.prod(ncol))
    # column-major view: index (j_n fastest ... j_1, vec slowest)
    T = X.reshape([nvec] + ncol, order="C") if False else X.reshape(tuple(ncol[::-1]) + (nvec,), order="F")
    # axes of T: (j_n, j_{n-1}, ..., j_1, vec)
    n = len(mats)
    for k in range(n - 1, -1, -1):
        ax = n - 1 - k
        T = np.moveaxis(np.tensordot(mats[k], T, axes=([1], [ax])), 0, ax)
    return T.reshape(int(np.prod(nrow)), nvec, order="F")


def kron_multd(nkron, mats, X):
    """kron_multd.m:1-87 (the d>6 recursion computes the same product)."""
    if len(mats) < nkron:
        raise ValueError("kron_multd: invalid nkron=%d, length(Acell)=%d" % (nkron, len(mats)))
    isize = int(np.prod([m.shape[1] for m in mats[:nkron]]))
    if np.asarray(X).size % isize != 0:
        raise ValueError("kron_multd:nkron=%d,prod(size(X))=%g,isizeX=%g" % (nkron, np.asarray(X).size, isize))
    return kronmult(mats[:nkron], X)


# ------------------------------------------------------------------------------------------
# Batched-GEMM planner (Kronmult/kronmult{1..6}_batch.m, gemm_vbatched.m, gemm.m, flops_*.m)
# ------------------------------------------------------------------------------------------
def flops_kron(nr, nc):
    """(flops1, flops2, imethod, imem1, imem2) of Kronmult/flops_kron{1..6}.m."""
    n = len(nr)
    if n == 1:
        f = 2.0 * nr[0] * nc[0]
        return f, f, 1, 0, 0
    if n == 2:
        nrowX, ncolX = nc[1], nc[0]
        f1 = 2.0 * nr[1] * nc[1] * ncolX
        m1 = nr[1] * ncolX
        f1 += 2.0 * nr[1] * nc[0] * nr[0]
        f2 = 2.0 * nrowX * nc[0] * nr[0]
        m2 = nrowX * nr[0]
        f2 += 2.0 * nr[1] * nc[1] * nr[0]
        return f1, f2, (1 if f1 <= f2 else 2), m1, m2
    nrowX = int(np.prod(nc[1:]))
    ncolX = nc[0]
    jf1, jf2, jm, jm1, jm2 = flops_kron(nr[1:], nc[1:])
    f1 = (jf1 if jm == 1 else jf2) * ncolX
    m1 = (jm1 if jm == 1 else jm2) * ncolX
    nrowY = int(np.prod(nr[1:]))
    m1 += nrowY * ncolX
    f1 += 2.0 * nrowY * nc[0] * nr[0]
    f2 = 2.0 * nrowX * nc[0] * nr[0]
    m2 = nrowX * nr[0]
    f2 += (jf1 if jm == 1 else jf2) * nr[0]
    m2 += (jm1 if jm == 1 else jm2) * nr[0]
    return f1, f2, (1 if f1 <= f2 else 2), m1, m2


class BatchList:
    """clear_batch_list.m: per-level list of GEMM records."""

    def __init__(self):
        self.entries = []  # dicts with m,n,k,transA,transB,alpha,beta,A,B,C

    @property
    def nbatch(self):
        return len(self.entries)


def gemm(transA, transB, m, n, k, alpha, A, B, beta, C):
    """Kronmult/gemm.m:1-30."""
    opA = A.T if transA in "Tt" else A
    opB = B.T if transB in "Tt" else B
    C = np.array(C, dtype=np.float64, copy=True)
    C[:m, :n] = 0.0 if beta == 0 else beta * C[:m, :n]
    C[:m, :n] += alpha * (opA[:m, :k] @ opB[:k, :n])
    return C


def gemm_vbatched(transA, transB, mlist, nlist, klist, alpha, Alist, Blist, beta, Clist, reference_bug=False):
    """Kronmult/gemm_vbatched.m.  The reference reads ``kk = nlist(ibatch)`` (line 25);
    ``reference_bug=True`` reproduces that, the default uses klist."""
    nb = len(mlist)
    if not (len(nlist) == nb and len(klist) == nb and len(Alist) == nb and len(Blist) == nb and len(Clist) == nb):
        raise ValueError("gemm_vbatched: mismatch nbatch=%d" % nb)
    out = []
    for i in range(nb):
        kk = nlist[i] if reference_bug else klist[i]
        out.append(gemm(transA, transB, mlist[i], nlist[i], kk, alpha, Alist[i], Blist[i], beta, Clist[i]))
    return out


def kronmult_batch(mats, X, lists):
    """kronmult{n}_batch.m: returns Y and appends GEMM records to lists[0..n-1].

    Method choice follows flops_kron{n} (kronmult2_batch.m:43, kronmult6_batch.m:53-56);
    level-1 records go to lists[0] (kronmult1_batch.m:45-66), the outermost A1 product of
    an n-fold product goes to lists[n-1] (kronmult2_batch.m:86-110, kronmult6_batch.m:90-117)."""
    n = len(mats)
    nr = [m.shape[0] for m in mats]
    nc = [m.shape[1] for m in mats]
    nrowX = int(np.prod(nc))
    X = np.asarray(X, dtype=np.float64)
    if X.size % nrowX != 0:
        raise ValueError("kronmult%d_batch: numel(X)=%g, nrowX=%g" % (n, X.size, nrowX))
    nvec = X.size // nrowX
    nrowY = int(np.prod(nr))

    def rec(lst, mm, nn, kk, tA, tB, A, B, C):
        lst.entries.append(dict(m=mm, n=nn, k=kk, transA=tA, transB=tB, alpha=1.0, beta=0.0, A=A, B=B, C=C))

    if n == 1:
        A1 = mats[0]
        mm, kk, nn = nr[0], nc[0], nvec
        B = X.reshape(kk, nn, order="F")
        C = np.zeros((mm, nn))
        rec(lists[0], mm, nn, kk, "N", "N", A1, B, C)
        return gemm("N", "N", mm, nn, kk, 1.0, A1, B, 0.0, C)
    _, _, imethod, _, _ = flops_kron(nr, nc)
    Y = np.zeros((nrowY, nvec))
    if imethod == 1:
        Ytmp = kronmult_batch(mats[1:], X, lists[:n - 1])
        nrowYtmp = int(np.prod(nr[1:])) * nc[0]
        Ytmp = Ytmp.reshape(nrowYtmp, nvec, order="F")
        for i in range(nvec):
            mm, kk, nn = nrowYtmp // nc[0], nc[0], nr[0]
            A = Ytmp[:mm * kk, i].reshape(mm, kk, order="F")
            C = Y[:mm * nn, i].reshape(mm, nn, order="F")
            rec(lists[n - 1], mm, nn, kk, "N", "T", A, mats[0], C)
            Ci = gemm("N", "T", mm, nn, kk, 1.0, A, mats[0], 0.0, C)
            Y[:, i] = Ci[:mm, :nn].reshape(-1, order="F")
        return Y
    Xr = X.reshape(nrowX, nvec, order="F")
    mm = int(np.prod(nc[1:]))
    Ytmp = np.zeros((mm, nr[0] * nvec))
    for i in range(nvec):
        i1 = i * nr[0]
        A = Xr[:, i].reshape(mm, nc[0], order="F")
        C = Ytmp[:, i1:i1 + nr[0]]
        Ci = gemm("N", "T", mm, nr[0], nc[0], 1.0, A, mats[0], 0.0, C)
        Ytmp[:, i1:i1 + nr[0]] = Ci[:mm, :nr[0]]
        rec(lists[0], mm, nr[0], nc[0], "N", "T", A, mats[0], C)
    if n == 2:
        mm2, nn2, kk2 = nr[1], nr[0] * nvec, nc[1]
        C = gemm("N", "N", mm2, nn2, kk2, 1.0, mats[1][:mm2, :kk2], Ytmp[:kk2, :nn2], 0.0, np.zeros((mm2, nn2)))
        rec(lists[1], mm2, nn2, kk2, "N", "N", mats[1][:mm2, :kk2], Ytmp[:kk2, :nn2], C)
        return C.reshape(nr[1] * nr[0], nvec, order="F")
    Y = kronmult_batch(mats[1:], Ytmp, lists[1:])
    return Y.reshape(nrowY, nvec, order="F")


def flops_batch_list(bl):
    """Kronmult/flops_batch_list.m: (total, max, min) of 2*m*n*k."""
    fl = [2.0 * e["m"] * e["n"] * e["k"] for e in bl.entries]
    if not fl:
        return 0.0, 0.0, 1e18
    return float(sum(fl)), float(max(fl)), float(min(fl))


# ------------------------------------------------------------------------------------------
# apply_A (apply_A.m:102-236)
# ------------------------------------------------------------------------------------------
def apply_A_loop(term_mats, idx1d, deg, f, conn=None, build_A=False):
    """Faithful loop of apply_A.m:102-236: rows x (all or connected) cols x terms.

    term_mats[t][d]: dense 1-D operators; idx1d[N,d]: 1-based 1-D indices; conn: optional
    list of 1-based connected element lists.  Returns ftmp (and dense A when build_A)."""
    N, D = idx1d.shape
    B = deg ** D
    f = np.asarray(f, dtype=np.float64).reshape(-1)
    y = np.zeros(N * B)
    A = np.zeros((N * B, N * B)) if build_A else None
    ar = np.arange(deg)
    for e in range(N):
        II = [(idx1d[e, d] - 1) * deg + ar for d in range(D)]
        cols = (np.asarray(conn[e]) - 1) if conn is not None else range(N)
        for j in cols:
            JJ = [(idx1d[j, d] - 1) * deg + ar for d in range(D)]
            for tm in term_mats:
                blocks = [tm[d][np.ix_(II[d], JJ[d])] for d in range(D)]
                if build_A:
                    A[e * B:(e + 1) * B, j * B:(j + 1) * B] += krond(blocks)
                else:
                    y[e * B:(e + 1) * B] += kron_multd(D, blocks, f[j * B:(j + 1) * B]).reshape(-1)
    return (y, A) if build_A else y


def apply_A_rows(term_mats, idx1d, deg, f, rows=None, conn=None):
    """Vectorised restatement of the same sums (per row, all columns at once); the
    column sum is taken per term in column order, as in apply_A.m:124-201."""
    N, D = idx1d.shape
    B = deg ** D
    f = np.asarray(f, dtype=np.float64).reshape(N, B)
    rows = range(N) if rows is None else rows
    out = np.zeros((len(rows), B))
    ar = np.arange(deg)
    for r, e in enumerate(rows):
        cols = (np.asarray(conn[e]) - 1) if conn is not None else np.arange(N)
        acc = np.zeros(B)
        for tm in term_mats:
            # T axes: (col, j_1, ..., j_D) with j_D fastest (C order == element layout)
            T = f[cols].reshape((len(cols),) + (deg,) * D)
            for d in range(D - 1, -1, -1):
                rI = (idx1d[e, d] - 1) * deg + ar
                cJ = (idx1d[cols, d][:, None] - 1) * deg + ar[None, :]
                blk = tm[d][rI[None, :, None], cJ[:, None, :]]  # (col, deg_out, deg_in)
                T = np.moveaxis(np.einsum("cab,c...b->c...a", blk, np.moveaxis(T, d + 1, -1)), -1, d + 1)
            acc += T.reshape(len(cols), B).sum(axis=0)
        out[r] = acc
    return out.reshape(-1)


def grad_ops_loop(term_mats, idx1d, deg, f, r, conn=None):
    """dL/dA_{t,d} for y = apply_A(f) and dL/dy = r, by differentiating each krond block
    (apply_A.m:170-201): d/dA_k[a,b] of r_i' kron(B_1..B_d) f_j = r_i' kron(.., E_ab, ..) f_j.
    Small cases only (p^2 krond products per pair, term and dimension)."""
    N, D = idx1d.shape
    B = deg ** D
    f = np.asarray(f, dtype=np.float64).reshape(N, B)
    r = np.asarray(r, dtype=np.float64).reshape(N, B)
    G = [[np.zeros_like(m) for m in tm] for tm in term_mats]
    ar = np.arange(deg)
    for e in range(N):
        II = [(idx1d[e, d] - 1) * deg + ar for d in range(D)]
        cols = (np.asarray(conn[e]) - 1) if conn is not None else range(N)
        for j in cols:
            JJ = [(idx1d[j, d] - 1) * deg + ar for d in range(D)]
            for t, tm in enumerate(term_mats):
                blocks = [tm[d][np.ix_(II[d], JJ[d])] for d in range(D)]
                for k in range(D):
                    for a in range(deg):
                        for b in range(deg):
                            E = np.zeros((deg, deg))
                            E[a, b] = 1.0
                            K = krond(blocks[:k] + [E] + blocks[k + 1:])
                            G[t][k][II[k][a], JJ[k][b]] += r[e] @ K @ f[j]
    return G


# ------------------------------------------------------------------------------------------
# Projections, sources and RK3 (md_eval_function.m, forward_wavelet_transform.m,
# combine_dimensions_D.m, time_advance.m:151-204)
# ------------------------------------------------------------------------------------------
def forward_wavelet_transform(deg, lev, lo, hi, fn, blocks, t):
    """forward_wavelet_transform.m:9-55."""
    qx, qw = lgwt(default_quad_number(deg), -1, 1)
    n = 2 ** lev
    h = (hi - lo) / n
    f = np.zeros(deg * n)
    p_val = (lin_legendre(qx, deg) / np.sqrt(h)).T
    for i in range(n):
        x = h * (qx / 2 + 0.5 + i) + lo
        f[i * deg:(i + 1) * deg] = p_val @ (qw * fn(x, t))
    f = f * h / 2
    f = apply_fmwt_blocks(lev, blocks, f, "LN")
    return f * (np.abs(f) > 1e-12)


def combine_dimensions(deg, flist, tmul, idx1d):
    """combine_dimensions_D.m:16-51."""
    N, D = idx1d.shape
    B = deg ** D
    out = np.zeros(N * B)
    for e in range(N):
        pieces = [flist[d][(idx1d[e, d] - 1) * deg:idx1d[e, d] * deg][:, None] for d in range(D)]
        out[e * B:(e + 1) * B] += krond(pieces).reshape(-1) * tmul
    return out


def md_eval(pde, deg, md_funcs, idx1d, blocks, t, mass_mats=None):
    """md_eval_function.m:31-48 (mass solve with the per-dimension mass matrices)."""
    out = np.zeros(idx1d.shape[0] * deg ** idx1d.shape[1])
    for fn in md_funcs:
        fl = []
        for d, dim in enumerate(pde.dims):
            v = forward_wavelet_transform(deg, dim.lev, dim.min, dim.max, fn[d], blocks, t)
            if mass_mats is not None:
                n = v.size
                v = np.linalg.solve(mass_mats[d][:n, :n], v)
            fl.append(v)
        out += combine_dimensions(deg, fl, fn[-1](t), idx1d)
    return out


def rk3_step(apply_fn, f, t, dt, source_fn):
    """RungeKutta3 without LHS mass or BCs (time_advance.m:151-204)."""
    s1, s2, s3 = source_fn(t), source_fn(t + 0.5 * dt), source_fn(t + dt)
    k1 = apply_fn(f) + s1
    y1 = f + dt * 0.5 * k1
    k2 = apply_fn(y1) + s2
    y2 = f + dt * (-1.0 * k1 + 2.0 * k2)
    k3 = apply_fn(y2) + s3
    return f + dt * (k1 / 6 + 2.0 / 3.0 * k2 + k3 / 6)


def backward_euler_step(A, f0, dt, s0):
    """backward_euler direct solve ``(I - dt A) f1 = f0 + dt s0`` (time_advance.m:320-349)."""
    AA = np.eye(A.shape[0]) - dt * A
    return np.linalg.solve(AA, f0 + dt * s0)


# ------------------------------------------------------------------------------------------
# The PDEs the configurations use (pdes/continuity{1,2,3,6}.m, pdes/diffusion2.m)
# ------------------------------------------------------------------------------------------
def continuity1(lev, LF=-1.0):
    """pdes/continuity1.m: 1-D advection d/dx with g=-1 on [-1,1]."""
    pi = np.pi
    dims = [Dim(-1.0, 1.0, lev)]
    terms = [[[DIV(lambda x: 0 * x - 1, LF, "P", "P")]]]
    sources = [
        [lambda x, t: np.cos(2 * pi * x), lambda t: np.cos(t)],
        [lambda x, t: np.sin(2 * pi * x), lambda t: -2 * pi * np.sin(t)],
    ]
    ic = [[lambda x, t: np.cos(2 * pi * x), lambda t: np.sin(t)]]
    return PDESpec(dims, terms, sources, ic, lambda p, cfl: (p.dims[0].max - p.dims[0].min) / 2 ** p.dims[0].lev * cfl)


def continuity2(lev, LF=-1.0):
    """pdes/continuity2.m:27-128."""
    pi = np.pi
    lv = [lev] * 2 if np.isscalar(lev) else list(lev)
    dims = [Dim(-1.0, 1.0, lv[0]), Dim(-2.0, 2.0, lv[1])]
    g = lambda x: 0 * x - 1
    terms = [[[DIV(g, LF, "P", "P")], [MASS()]], [None, [DIV(g, LF, "P", "P")]]]
    sources = [
        [lambda x, t: np.cos(pi * x), lambda y, t: np.sin(2 * pi * y), lambda t: 2 * np.cos(2 * t)],
        [lambda x, t: np.cos(pi * x), lambda y, t: np.cos(2 * pi * y), lambda t: 2 * pi * np.sin(2 * t)],
        [lambda x, t: np.sin(pi * x), lambda y, t: np.sin(2 * pi * y), lambda t: -pi * np.sin(2 * t)],
    ]
    ic = [[lambda x, t: np.cos(pi * x), lambda y, t: np.sin(2 * pi * y), lambda t: np.sin(2 * t)]]
    return PDESpec(dims, terms, sources, ic, lambda p, cfl: (p.dims[0].max - p.dims[0].min) / 2 ** p.dims[0].lev * cfl)


def continuity3(lev, LF=-1.0):
    """pdes/continuity3.m:24-129 (PDE.m:69 overrides the per-dimension levels with opts.lev)."""
    pi = np.pi
    lv = [lev] * 3 if np.isscalar(lev) else list(lev)
    dims = [Dim(-1.0, 1.0, lv[0]), Dim(-2.0, 2.0, lv[1]), Dim(-3.0, 3.0, lv[2])]
    g = lambda x: 0 * x - 1
    terms = [[[DIV(g, LF, "P", "P")], None, None], [None, [DIV(g, LF, "P", "P")], None],
             [None, None, [DIV(g, LF, "P", "P")]]]
    sources = [
        [lambda x, t: np.cos(pi * x), lambda y, t: np.sin(2 * pi * y), lambda z, t: np.cos(2 * pi * z / 3), lambda t: 2 * np.cos(2 * t)],
        [lambda x, t: np.cos(pi * x), lambda y, t: np.cos(2 * pi * y), lambda z, t: np.cos(2 * pi * z / 3), lambda t: 2 * pi * np.sin(2 * t)],
        [lambda x, t: np.sin(pi * x), lambda y, t: np.sin(2 * pi * y), lambda z, t: np.cos(2 * pi * z / 3), lambda t: -pi * np.sin(2 * t)],
        [lambda x, t: np.cos(pi * x), lambda y, t: np.sin(2 * pi * y), lambda z, t: np.sin(2 * pi * z / 3), lambda t: -2.0 / 3.0 * pi * np.sin(2 * t)],
    ]
    ic = [[lambda x, t: 0 * x] * 3 + [lambda t: 1.0]]
    return PDESpec(dims, terms, sources, ic, lambda p, cfl: (p.dims[0].max - p.dims[0].min) / 2 ** p.dims[0].lev * cfl)


def continuity6(lev, LF=-1.0):
    """pdes/continuity6.m:28-221: six advection terms, the seven separable sources, zero
    initial condition."""
    lv = [lev] * 6 if np.isscalar(lev) else list(lev)
    bounds = [(-1.0, 1.0), (-2.0, 2.0), (-3.0, 3.0), (-10.0, 10.0), (-20.0, 20.0), (-30.0, 30.0)]
    dims = [Dim(lo, hi, l) for (lo, hi), l in zip(bounds, lv)]
    speeds = [1.0, 1.0, 3.0, 4.0, 3.0, 2.0]
    terms = []
    for k in range(6):
        row = [None] * 6
        row[k] = [DIV((lambda s: (lambda x: 0 * x - s))(speeds[k]), LF, "P", "P")]
        terms.append(row)
    pi = np.pi
    args = [pi, pi / 2, pi / 3, pi / 10, pi / 20, pi / 30]
    cos_ = lambda a: (lambda x, t: np.cos(a * x))
    sin_ = lambda a: (lambda x, t: np.sin(a * x))
    base = ["c", "s", "c", "c", "s", "c"]  # the solution's factors (continuity6.m:214-221)

    def src(flip, tf):  # the solution's factors with dimension ``flip`` differentiated
        fs = []
        for k in range(6):
            kind = base[k] if k != flip else ("s" if base[k] == "c" else "c")
            fs.append(cos_(args[k]) if kind == "c" else sin_(args[k]))
        return fs + [tf]

    sources = [src(-1, lambda t: 2 * np.cos(2 * t)), src(1, lambda t: 0.5 * pi * np.sin(2 * t)),
               src(0, lambda t: -pi * np.sin(2 * t)), src(2, lambda t: -pi * np.sin(2 * t)),
               src(4, lambda t: 3 / 20 * pi * np.sin(2 * t)), src(3, lambda t: -2 / 5 * pi * np.sin(2 * t)),
               src(5, lambda t: -1 / 15 * pi * np.sin(2 * t))]
    ic = [[(lambda x, t: 0 * x)] * 6 + [lambda t: 1.0]]
    return PDESpec(dims, terms, sources, ic, lambda p, cfl: (p.dims[0].max - p.dims[0].min) / 2 ** p.dims[0].lev * cfl)


def diffusion2(lev):
    """pdes/diffusion2.m:33-108: LDG d2/dx2 + d2/dy2 on [0,1]^2 (DIV(+1,N,N) then GRAD(-1,D,D)),
    analytic solution cos(pi x) cos(pi y) exp(-2 pi^2 t) as initial and Dirichlet boundary
    data (diffusion2.m:41-55)."""
    pi = np.pi
    lv = [lev] * 2 if np.isscalar(lev) else list(lev)
    dims = [Dim(0.0, 1.0, lv[0]), Dim(0.0, 1.0, lv[1])]
    one = lambda x: 0 * x + 1
    ldg = [DIV(one, +1.0, "N", "N"), GRAD(one, -1.0, "D", "D")]
    terms = [[ldg, [MASS(), MASS()]], [[MASS(), MASS()], ldg]]
    soln = [lambda x, t: np.cos(pi * x), lambda y, t: np.cos(pi * y), lambda t: np.exp(-2 * pi ** 2 * t)]
    spec = PDESpec(dims, terms, [], [soln], lambda p, cfl: cfl * (1.0 / 2 ** p.dims[0].lev) ** 2)
    spec.bc = soln  # BCL = BCR = the solution (diffusion2.m:49-52)
    return spec


def compute_boundary_condition(g, lev, deg, lo, hi, fn, t, side):
    """compute_boundary_condition.m:1-55 (dV = 1): the boundary trace -g f v|_lo on the first
    cell or +g f v|_hi on the last, in the Legendre basis."""
    n = 2 ** lev
    h = (hi - lo) / n
    bc = np.zeros(deg * n)
    if side == "L":
        p_L = lin_legendre(-1.0, deg)[0] / np.sqrt(h)
        bc[:deg] = -float(g(np.array([lo]))[0]) * p_L * float(fn(np.array([lo]), t)[0])
    else:
        p_R = lin_legendre(1.0, deg)[0] / np.sqrt(h)
        bc[deg * (n - 1):] = float(g(np.array([hi]))[0]) * p_R * float(fn(np.array([hi]), t)[0])
    return bc


def boundary_condition_vector(pde, deg, idx1d, blocks, t, coeff_level=None):
    """boundary_condition_vector.m:1-197 for Dirichlet partial terms (dV = 1, so every LHS
    mass matrix is the identity).  For partial term p of dimension d1 with a 'D' side: the
    other dimensions carry the projection of the boundary function times the p-th partial
    term's g of that dimension, passed through that dimension's preceding partial terms; d1
    carries the FMWT of the boundary trace passed through d1's preceding partial terms;
    combine_dimensions_D then forms the Kronecker product on the element table, scaled by the
    boundary function's time factor."""
    D = len(pde.dims)
    out = np.zeros(idx1d.shape[0] * deg ** D)
    lv = [d.lev if coeff_level is None else coeff_level for d in pde.dims]
    pmats = [[[pterm_matrix(deg, pde.dims[d], pt, lv[d]) for pt in pde.terms[tt][d]] for d in range(D)]
             for tt in range(len(pde.terms))]
    for tt, term in enumerate(pde.terms):
        for d1 in range(D):
            dim = pde.dims[d1]
            dof = deg * 2 ** dim.lev
            for p, pt in enumerate(term[d1]):
                if pt.type not in ("grad", "div"):
                    continue
                for side, kind in (("L", pt.BCL), ("R", pt.BCR)):
                    if kind != "D":
                        continue
                    fl = []
                    for d2 in range(D):
                        oth = term[d2]
                        n2 = deg * 2 ** pde.dims[d2].lev
                        if d2 == d1:
                            v = compute_boundary_condition(pt.g, dim.lev, deg, dim.min, dim.max, pde.bc[d1], t, side)
                            v = apply_fmwt_blocks(dim.lev, blocks, v, "LN")
                            for q in range(p - 1, -1, -1):
                                v = pmats[tt][d1][q][:dof, :dof] @ v
                        else:
                            mp = oth[p]
                            fn = (lambda f2, g2: (lambda x, tt_: f2(x, tt_) * g2(x)))(pde.bc[d2], mp.g)
                            v = forward_wavelet_transform(deg, pde.dims[d2].lev, pde.dims[d2].min, pde.dims[d2].max,
                                                          fn, blocks, t)
                            for q in range(p):
                                v = pmats[tt][d2][q][:n2, :n2] @ v
                        fl.append(v)
                    out += combine_dimensions(deg, fl, pde.bc[D](t), idx1d)
    return out
