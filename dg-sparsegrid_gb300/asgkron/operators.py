"""Host-side producer of the hot path's inputs: dense wavelet-space 1-D DG operators.

Builds pde.terms{t}.terms_1D{d}.mat the way get_coeff_mats.m -> sd_term_coeff_matrix.m ->
pterm_coeff_matrix.m -> coeff_matrix.m does (DG volume + trace terms with Lax-Friedrichs
flux and P/D/N boundary conditions in realspace, rotated by the multiwavelet transform,
LHS-mass solved, partial terms chained), and the multiwavelet filters the transform needs
(two_scale/MultiwaveletGen.m).  Vectorised numpy; independent of the test oracle.
"""
import numpy as np

# ------------------------------------------------------------------------------------------
# Gauss-Legendre quadrature and normalised Legendre polynomials
# ------------------------------------------------------------------------------------------


def gauss_legendre(n, a=-1.0, b=1.0):
    """n-point Gauss-Legendre rule on [a, b] by Newton iteration on P_n (Quadrature/lgwt.m)."""
    m = n - 1
    xu = np.linspace(-1.0, 1.0, n)
    y = np.cos((2 * np.arange(n) + 1) * np.pi / (2 * m + 2)) + (0.27 / n) * np.sin(np.pi * xu * m / (m + 2))
    prev = np.full_like(y, 2.0)
    while np.max(np.abs(y - prev)) > np.finfo(float).eps:
        p_km1, p_k = np.ones_like(y), y.copy()
        for k in range(2, n + 1):
            p_km1, p_k = p_k, ((2 * k - 1) * y * p_k - (k - 1) * p_km1) / k
        dp = n * (p_km1 - y * p_k) / (1 - y ** 2)  # P_n'
        prev = y
        y = prev - p_k / dp
    x = (a * (1 - y) + b * (1 + y)) / 2
    w = (b - a) / ((1 - y ** 2) * dp ** 2)
    return x[::-1].copy(), w[::-1].copy()


def quad_points(deg):
    """max(deg+1, 10) points (Quadrature/default_quad_number.m:2)."""
    return gauss_legendre(max(deg + 1, 10))


def legendre_values(x, deg):
    """[len(x), deg] values of sqrt(2n+1) P_n(x), zero outside [-1, 1] (DG_loc/lin_legendre.m)."""
    x = np.atleast_1d(np.asarray(x, dtype=np.float64))
    out = np.zeros((x.size, deg))
    p_prev, p = np.zeros_like(x), np.ones_like(x)
    for n in range(deg):
        out[:, n] = p * np.sqrt(2 * n + 1)
        p_prev, p = p, ((2 * n + 1) * x * p - n * p_prev) / (n + 1)
    out[(x > 1) | (x < -1), :] = 0.0
    return out


def legendre_derivs(x, deg):
    """[len(x), deg] derivatives of sqrt(2n+1) P_n via P'_n = n P_{n-1} + x P'_{n-1}."""
    x = np.atleast_1d(np.asarray(x, dtype=np.float64))
    out = np.zeros((x.size, deg))
    p_prev, p = np.zeros_like(x), np.ones_like(x)  # P_{n-1}, P_n
    dp = np.zeros_like(x)
    for n in range(deg):
        if n > 0:
            dp = n * p_prev + x * dp
        out[:, n] = dp * np.sqrt(2 * n + 1)
        p_prev, p = p, ((2 * n + 1) * x * p - n * p_prev) / (n + 1)
    return out


# ------------------------------------------------------------------------------------------
# Multiwavelet two-scale filters (two_scale/MultiwaveletGen.m) and the transform matrix
# ------------------------------------------------------------------------------------------
_FILTER_CACHE = {}


def multiwavelet_filters(k):
    """H0, G0 (k x k) of the Alpert multiwavelets as MultiwaveletGen.m builds them.

    Scaling functions: normalised Legendre polynomials on [-1,1].  Wavelets: piecewise
    polynomials on [-1,0] | [0,1], started from -x^j | +x^j, made orthogonal to the scaling
    functions and to each other by Gram-Schmidt in the order of MultiwaveletGen.m, then
    reversed and sign-alternated.  Inner products use the normalised measure dx/2 and an
    exact Gauss rule; the filters are the projections of the level-0 functions onto the
    level-1 scaling functions of [-1,0]."""
    if k in _FILTER_CACHE:
        return tuple(v.copy() for v in _FILTER_CACHE[k])
    xq, wq = quad_points(k)
    wq = wq / 2
    xl, xr = (xq - 1) / 2, (xq + 1) / 2  # nodes of the two halves
    # scaling functions at the half-interval nodes (same polynomial on both halves)
    S_l, S_r = legendre_values(xl, k), legendre_values(xr, k)
    # wavelet candidates: left piece -x^j, right piece +x^j, j = 0..k-1
    W_l = -np.stack([xl ** j for j in range(k)], axis=1)
    W_r = np.stack([xr ** j for j in range(k)], axis=1)

    def ip(al, ar, bl, br):  # <a, b> with measure dx/2 over [-1,1]
        return (np.sum(al * bl * wq) + np.sum(ar * br * wq)) / 2

    for j in range(k):  # orthogonalise against all scaling functions
        pl, pr = np.zeros(xq.size), np.zeros(xq.size)
        for s in range(k):
            c = ip(W_l[:, j], W_r[:, j], S_l[:, s], S_r[:, s])
            pl += c * S_l[:, s]
            pr += c * S_r[:, s]
        W_l[:, j] -= pl
        W_r[:, j] -= pr
    for j in range(1, k):  # Gram-Schmidt among the wavelets (projections from the old set)
        pl, pr = np.zeros(xq.size), np.zeros(xq.size)
        for i in range(j):
            c = ip(W_l[:, j], W_r[:, j], W_l[:, i], W_r[:, i])
            nrm = ip(W_l[:, i], W_r[:, i], W_l[:, i], W_r[:, i])
            pl += c * W_l[:, i] / nrm
            pr += c * W_r[:, i] / nrm
        W_l[:, j] -= pl
        W_r[:, j] -= pr
    for j in range(k):
        nrm = np.sqrt(ip(W_l[:, j], W_r[:, j], W_l[:, j], W_r[:, j]))
        W_l[:, j] /= nrm
        W_r[:, j] /= nrm
    sign = (-1.0) ** np.arange(k)
    W_l = W_l[:, ::-1] * sign
    # filters: project level-0 functions on [-1,0] onto the level-1 scaling functions there.
    # On [-1,0], with u = 2x+1 in [-1,1]: phi^1_b(x) = sqrt(2) phi_b(u).
    u = xq  # u nodes, x = (u-1)/2 = xl
    Phi_u = legendre_values(u, k)
    H0 = (S_l * wq[:, None]).T @ Phi_u / np.sqrt(2)
    G0 = (W_l * wq[:, None]).T @ Phi_u / np.sqrt(2)
    H0[np.abs(H0) < 1e-5] = 0.0
    G0[np.abs(G0) < 1e-5] = 0.0
    _FILTER_CACHE[k] = (H0, G0)
    return H0.copy(), G0.copy()


def fmwt_matrix(deg, lev):
    """Forward multiwavelet transform (deg*2^lev square): rows ordered level 0 scaling,
    then wavelets level by level, cells left to right (OperatorTwoScale_wavelet2.m:127-144).

    Built by running the cascade s_c = H0 s_2c + H1 s_2c+1, d_c = G0 s_2c + G1 s_2c+1 on the
    identity, finest level first."""
    n = deg * 2 ** lev
    if lev == 0:
        return np.eye(deg)
    H0, G0 = multiwavelet_filters(deg)
    tol = 1e4 * np.finfo(float).eps
    H0[np.abs(H0) < tol] = 0.0
    G0[np.abs(G0) < tol] = 0.0
    a = np.arange(deg)
    sgn = (-1.0) ** (a[:, None] + a[None, :])
    H1 = sgn * H0
    G1 = ((-1.0) ** deg) * sgn * G0
    F = np.zeros((n, n))
    s = np.eye(n).reshape(2 ** lev, deg, n)  # scaling coefficients per finest cell
    for L in range(lev, 0, -1):
        left, right = s[0::2], s[1::2]
        d = np.einsum("ab,cbn->can", G0, left) + np.einsum("ab,cbn->can", G1, right)
        s = np.einsum("ab,cbn->can", H0, left) + np.einsum("ab,cbn->can", H1, right)
        ncell = 2 ** (L - 1)
        r0 = deg * ncell  # wavelets of level L start after deg * 2^(L-1) rows
        F[r0:r0 + deg * ncell] = d.reshape(deg * ncell, n)
    F[:deg] = s.reshape(deg, n)
    return F


# ------------------------------------------------------------------------------------------
# Partial terms and the 1-D operator builder
# ------------------------------------------------------------------------------------------
class PartialTerm:
    """One partial term: kind 'mass' | 'div' | 'grad' with coefficient g(x), flux LF and
    boundary types (PARTIAL_SD_TERM.m, DIV.m, GRAD.m, MASS.m).  For 'grad' the flux sign
    flips and D<->N swap as GRAD.m:14-34 does."""

    def __init__(self, kind, g=None, LF=0.0, BCL="N", BCR="N"):
        self.kind = kind
        self.g = g if g is not None else (lambda x: np.ones_like(x))
        self.LF = -LF if kind == "grad" else LF
        swap = {"D": "N", "N": "D"}
        self.bcl = swap.get(BCL, BCL) if kind == "grad" else BCL
        self.bcr = swap.get(BCR, BCR) if kind == "grad" else BCR
        self.BCL, self.BCR = BCL, BCR  # as given: the boundary-data sides (boundary_condition_vector.m:57-60)


def mass_term(g=None):
    return PartialTerm("mass", g)


def div_term(g, LF, BCL, BCR):
    return PartialTerm("div", g, LF, BCL, BCR)


def grad_term(g, LF, BCL, BCR):
    return PartialTerm("grad", g, LF, BCL, BCR)


def realspace_matrix(deg, lo, hi, lev, pt):
    """Realspace DG matrix of a partial term on 2^lev uniform cells (coeff_matrix.m:105-323)."""
    N = 2 ** lev
    h = (hi - lo) / N
    n = deg * N
    xq, wq = quad_points(deg)
    V = legendre_values(xq, deg) / np.sqrt(h)
    dV = legendre_derivs(xq, deg) / np.sqrt(h) * 2 / h
    pL = legendre_values(-1.0, deg)[0] / np.sqrt(h)
    pR = legendre_values(1.0, deg)[0] / np.sqrt(h)
    M = np.zeros((n, n))
    cells = np.arange(N)
    xcell = ((xq[None, :] + 1) / 2 + cells[:, None]) * h + lo  # [N, nq]
    G = pt.g(xcell) * np.ones_like(xcell)
    J = h / 2
    vol_mass = np.einsum("qa,cq,qb->cab", V, G * wq[None, :], V) * J
    vol_div = -np.einsum("qa,cq,qb->cab", dV, G * wq[None, :], V) * J
    loc = vol_mass if pt.kind == "mass" else vol_div
    for c in range(N):
        M[c * deg:(c + 1) * deg, c * deg:(c + 1) * deg] += loc[c]
    if pt.kind in ("div", "grad"):
        LF = pt.LF
        for c in range(N):
            xL, xR = lo + c * h, lo + (c + 1) * h
            gL = float(np.asarray(pt.g(np.array([xL]))).reshape(-1)[0])
            gR = float(np.asarray(pt.g(np.array([xR]))).reshape(-1)[0])
            # trace blocks coupling cell c with (left nbr, itself @xL, itself @xR, right nbr)
            B0 = np.outer(-pL, pR) * (gL / 2 + LF * abs(gL) / 2)
            B1 = np.outer(-pL, pL) * gL / 2 + LF * abs(gL) / 2 * np.outer(-pL, -pL)
            B2 = np.outer(pR, pR) * gR / 2 + LF * abs(gR) / 2 * np.outer(pR, pR)
            B3 = np.outer(pR, pL) * gR / 2 + LF * abs(gR) / 2 * np.outer(pR, -pL)
            blocks = [B0, B1, B2, B3]
            z = np.zeros((deg, deg))
            if c == 0 and pt.bcl == "D":
                blocks[0] = blocks[1] = z
            if c == N - 1 and pt.bcr == "D":
                blocks[2] = blocks[3] = z
            if c == 0 and pt.bcl == "N":
                blocks[0] = z
                blocks[1] = np.outer(-pL, pL) * gL
            if c == N - 1 and pt.bcr == "N":
                blocks[2] = np.outer(pR, pR) * gR
                blocks[3] = z
            periodic = pt.bcl == "P" or pt.bcr == "P"
            nbr = [c - 1, c, c, c + 1]
            use = [0, 1, 2, 3]
            if periodic:
                if lev >= 1:
                    nbr = [(c - 1) % N, c, c, (c + 1) % N]
                else:
                    nbr = [c, c, c, c]
            else:  # no neighbour outside the domain (a single cell has neither)
                use = [b for b in use if 0 <= nbr[b] < N]
            for b in use:
                M[c * deg:(c + 1) * deg, nbr[b] * deg:(nbr[b] + 1) * deg] += blocks[b]
        if pt.kind == "grad":
            M = -M.T
    return M


def pterm_matrix(deg, lo, hi, lev, pt):
    """One partial term in wavelet space, LHS mass solved: M \\ L (pterm_coeff_matrix.m:6-20)."""
    F = fmwt_matrix(deg, lev)
    Mw = F @ realspace_matrix(deg, lo, hi, lev, mass_term()) @ F.T
    return np.linalg.solve(Mw, F @ realspace_matrix(deg, lo, hi, lev, pt) @ F.T)


def boundary_trace(deg, lo, hi, lev, pt, fn, t, side):
    """Wavelet coefficients of the boundary flux of a Dirichlet side (compute_boundary_condition.m
    + apply_FMWT_blocks): -g(lo) f(lo) v(lo) on the first cell, +g(hi) f(hi) v(hi) on the last."""
    N = 2 ** lev
    h = (hi - lo) / N
    c = np.zeros(deg * N)
    x = np.array([lo if side == "L" else hi])
    gval = float(np.asarray(pt.g(x)).reshape(-1)[0])
    fval = float(np.asarray(fn(x, t)).reshape(-1)[0])
    if side == "L":
        c[:deg] = -gval * fval * legendre_values(-1.0, deg)[0] / np.sqrt(h)
    else:
        c[deg * (N - 1):] = gval * fval * legendre_values(1.0, deg)[0] / np.sqrt(h)
    return fmwt_matrix(deg, lev) @ c


def term_matrix(deg, lo, hi, lev, pterms):
    """Chained 1-D operator eye * (M \\ L_1) * (M \\ L_2) ... in wavelet space
    (sd_term_coeff_matrix.m:9-22, pterm_coeff_matrix.m:6-20)."""
    F = fmwt_matrix(deg, lev)
    Mw = F @ realspace_matrix(deg, lo, hi, lev, mass_term()) @ F.T
    out = np.eye(deg * 2 ** lev)
    for pt in pterms:
        Lw = F @ realspace_matrix(deg, lo, hi, lev, pt) @ F.T
        out = out @ np.linalg.solve(Mw, Lw)
    return out


# ------------------------------------------------------------------------------------------
# Projections (forward_wavelet_transform.m, combine_dimensions_D.m)
# ------------------------------------------------------------------------------------------


def project_1d(deg, lev, lo, hi, fn, t=0.0):
    """Wavelet coefficients of fn(x, t) on [lo, hi] at level lev; |c| <= 1e-12 zeroed."""
    xq, wq = quad_points(deg)
    N = 2 ** lev
    h = (hi - lo) / N
    V = legendre_values(xq, deg) / np.sqrt(h)
    x = h * (xq[None, :] / 2 + 0.5 + np.arange(N)[:, None]) + lo
    vals = fn(x, t) * np.ones_like(x)
    c = (vals * wq[None, :]) @ V * h / 2  # [N, deg]
    w = fmwt_matrix(deg, lev) @ c.reshape(-1)
    return w * (np.abs(w) > 1e-12)


def combine_dimensions(deg, vecs, scale, idx1d):
    """Element blocks kron(v_1[I_1(e)], ..., v_d[I_d(e)]) * scale (1-based idx1d)."""
    N, D = idx1d.shape
    out = np.ones((N, 1))
    for d in range(D):
        rows = (idx1d[:, d:d + 1] - 1) * deg + np.arange(deg)[None, :]
        piece = np.asarray(vecs[d])[rows]  # [N, deg]
        out = (out[:, :, None] * piece[:, None, :]).reshape(N, -1)
    return out.reshape(-1) * scale
