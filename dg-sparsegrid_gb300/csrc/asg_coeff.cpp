// The hot path's operator producer on the host: wavelet-space 1-D DG operators.
//
// Host C++ restatement of the reference's construction of pde.terms{t}.terms_1D{d}.mat:
// Gauss-Legendre rules (Quadrature/lgwt.m), the Alpert multiwavelet filters
// (two_scale/MultiwaveletGen.m), the forward transform matrix
// (OperatorTwoScale_wavelet2.m:127-144), the realspace DG volume and trace matrices with the
// Lax-Friedrichs flux and periodic / Dirichlet / Neumann ends (coeff_matrix.m:105-323),
// the LHS-mass solve and the chaining of partial terms (pterm_coeff_matrix.m:6-20,
// sd_term_coeff_matrix.m:9-22).
//
// The reference rotates every realspace matrix into wavelet space (a dense (p 2^L)^3 triple
// product each), solves M_w \ L_w densely and multiplies the chain densely.  With F the
// orthogonal transform, M_w \ L_w = F (M_r^-1 L_r) F^T and the product of rotated factors is
// the rotation of the product, so this builder chains in realspace, where M_r is
// block-diagonal and each L_r block-tridiagonal, and rotates once, visiting only the
// nonzero column range of each transform row.  The result equals the reference's to the
// transform's orthogonality round-off (|F F^T - I| ~ 6e-14 at deg 4).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <new>
#include <thread>
#include <vector>

#include "asg_internal.h"

namespace {

using asg::fail;

constexpr double kPi = 3.14159265358979323846;

// n-point Gauss-Legendre rule on [a, b]: Newton iteration on P_n from the initial guess of
// lgwt.m, every node iterated until the largest update is at most machine epsilon; nodes
// ascending.
void gauss_legendre(int n, double a, double b, double* x, double* w) {
  const int m = n - 1;
  std::vector<double> y(n), prev(n, 2.0), dp(n, 0.0);
  for (int i = 0; i < n; ++i) {
    const double xu = n > 1 ? -1.0 + 2.0 * i / (n - 1) : -1.0;
    y[i] = std::cos((2 * i + 1) * kPi / (2 * m + 2)) + (0.27 / n) * std::sin(kPi * xu * m / (m + 2));
  }
  for (int iter = 0; iter < 100; ++iter) {
    double step = 0.0;
    for (int i = 0; i < n; ++i) step = std::max(step, std::fabs(y[i] - prev[i]));
    if (step <= 2.220446049250313e-16) break;
    for (int i = 0; i < n; ++i) {
      double p0 = 1.0, p1 = y[i];
      for (int k = 2; k <= n; ++k) {
        const double p2 = ((2 * k - 1) * y[i] * p1 - (k - 1) * p0) / k;
        p0 = p1;
        p1 = p2;
      }
      dp[i] = n * (p0 - y[i] * p1) / (1 - y[i] * y[i]);
      prev[i] = y[i];
      y[i] = prev[i] - p1 / dp[i];
    }
  }
  for (int i = 0; i < n; ++i) {  // descending y -> ascending x
    const int r = n - 1 - i;
    x[r] = (a * (1 - y[i]) + b * (1 + y[i])) / 2;
    w[r] = (b - a) / ((1 - y[i] * y[i]) * dp[i] * dp[i]);
  }
}

int quad_count(int deg) { return std::max(deg + 1, 10); }  // default_quad_number.m:2

// sqrt(2n+1) P_n(x), n < deg; zero outside [-1, 1] (lin_legendre.m)
void legendre_values(double x, int deg, double* out) {
  double p0 = 0.0, p1 = 1.0;
  const bool in = x <= 1.0 && x >= -1.0;
  for (int n = 0; n < deg; ++n) {
    out[n] = in ? p1 * std::sqrt(2.0 * n + 1) : 0.0;
    const double p2 = ((2 * n + 1) * x * p1 - n * p0) / (n + 1);
    p0 = p1;
    p1 = p2;
  }
}

// d/dx of sqrt(2n+1) P_n(x) by P'_n = n P_{n-1} + x P'_{n-1}
void legendre_derivs(double x, int deg, double* out) {
  double p0 = 0.0, p1 = 1.0, d = 0.0;
  for (int n = 0; n < deg; ++n) {
    if (n > 0) d = n * p0 + x * d;
    out[n] = d * std::sqrt(2.0 * n + 1);
    const double p2 = ((2 * n + 1) * x * p1 - n * p0) / (n + 1);
    p0 = p1;
    p1 = p2;
  }
}

// H0, G0 (k x k, row-major) of MultiwaveletGen.m: wavelet candidates -x^j | +x^j on the two
// halves of [-1, 1], orthogonalised against the Legendre scaling functions, then against
// each other (classical Gram-Schmidt in index order), normalised, reversed with alternating
// signs; filters are the projections of the level-0 functions on [-1, 0] onto the level-1
// scaling functions there; entries below 1e-5 in magnitude are zeroed.
void multiwavelet_filters(int k, double* H0, double* G0) {
  const int nq = quad_count(k);
  std::vector<double> xq(nq), wq(nq), xl(nq), xr(nq);
  gauss_legendre(nq, -1.0, 1.0, xq.data(), wq.data());
  for (int q = 0; q < nq; ++q) {
    wq[q] /= 2;
    xl[q] = (xq[q] - 1) / 2;
    xr[q] = (xq[q] + 1) / 2;
  }
  std::vector<double> Sl(nq * k), Sr(nq * k), Wl(nq * k), Wr(nq * k), Phi(nq * k);
  for (int q = 0; q < nq; ++q) {
    legendre_values(xl[q], k, &Sl[q * k]);
    legendre_values(xr[q], k, &Sr[q * k]);
    legendre_values(xq[q], k, &Phi[q * k]);
    for (int j = 0; j < k; ++j) {
      Wl[q * k + j] = -std::pow(xl[q], j);
      Wr[q * k + j] = std::pow(xr[q], j);
    }
  }
  // <a_i, b_j> with the measure dx/2 over [-1, 1]
  auto ip = [&](const std::vector<double>& al, const std::vector<double>& ar, int i, const std::vector<double>& bl,
                const std::vector<double>& br, int j) {
    double sl = 0.0, sr = 0.0;
    for (int q = 0; q < nq; ++q) {
      sl += al[q * k + i] * bl[q * k + j] * wq[q];
      sr += ar[q * k + i] * br[q * k + j] * wq[q];
    }
    return (sl + sr) / 2;
  };
  std::vector<double> pl(nq), pr(nq);
  for (int j = 0; j < k; ++j) {
    std::fill(pl.begin(), pl.end(), 0.0);
    std::fill(pr.begin(), pr.end(), 0.0);
    for (int s = 0; s < k; ++s) {
      const double c = ip(Wl, Wr, j, Sl, Sr, s);
      for (int q = 0; q < nq; ++q) {
        pl[q] += c * Sl[q * k + s];
        pr[q] += c * Sr[q * k + s];
      }
    }
    for (int q = 0; q < nq; ++q) {
      Wl[q * k + j] -= pl[q];
      Wr[q * k + j] -= pr[q];
    }
  }
  for (int j = 1; j < k; ++j) {
    std::fill(pl.begin(), pl.end(), 0.0);
    std::fill(pr.begin(), pr.end(), 0.0);
    for (int i = 0; i < j; ++i) {
      const double c = ip(Wl, Wr, j, Wl, Wr, i), nrm = ip(Wl, Wr, i, Wl, Wr, i);
      for (int q = 0; q < nq; ++q) {
        pl[q] += c * Wl[q * k + i] / nrm;
        pr[q] += c * Wr[q * k + i] / nrm;
      }
    }
    for (int q = 0; q < nq; ++q) {
      Wl[q * k + j] -= pl[q];
      Wr[q * k + j] -= pr[q];
    }
  }
  for (int j = 0; j < k; ++j) {
    const double nrm = std::sqrt(ip(Wl, Wr, j, Wl, Wr, j));
    for (int q = 0; q < nq; ++q) Wl[q * k + j] /= nrm;
  }
  const double r2 = std::sqrt(2.0);
  for (int a = 0; a < k; ++a) {
    const int src = k - 1 - a;  // reversed, sign (-1)^a
    const double sg = (a % 2) ? -1.0 : 1.0;
    for (int b = 0; b < k; ++b) {
      double h = 0.0, g = 0.0;
      for (int q = 0; q < nq; ++q) {
        h += Sl[q * k + a] * wq[q] * Phi[q * k + b];
        g += sg * Wl[q * k + src] * wq[q] * Phi[q * k + b];
      }
      h /= r2;
      g /= r2;
      H0[a * k + b] = std::fabs(h) < 1e-5 ? 0.0 : h;
      G0[a * k + b] = std::fabs(g) < 1e-5 ? 0.0 : g;
    }
  }
}

// Forward transform (n = deg 2^lev, row-major): the cascade s_c = H0 s_2c + H1 s_2c+1,
// d_c = G0 s_2c + G1 s_2c+1 run on the identity, finest level first; rows are the level-0
// scaling functions, then the wavelets level by level, cells left to right.  Row r's
// nonzeros lie in columns [c0[r], c1[r]) (the support of its cell).
void fmwt(int deg, int lev, double* F, int* c0, int* c1) {
  const long long n = static_cast<long long>(deg) << lev;
  std::memset(F, 0, sizeof(double) * n * n);
  if (lev == 0) {
    for (int a = 0; a < deg; ++a) {
      F[a * n + a] = 1.0;
      c0[a] = 0;
      c1[a] = deg;
    }
    return;
  }
  std::vector<double> H0(deg * deg), G0(deg * deg), H1(deg * deg), G1(deg * deg);
  multiwavelet_filters(deg, H0.data(), G0.data());
  for (int a = 0; a < deg; ++a)
    for (int b = 0; b < deg; ++b) {
      const double sg = ((a + b) % 2) ? -1.0 : 1.0;
      H1[a * deg + b] = sg * H0[a * deg + b];
      G1[a * deg + b] = ((deg % 2) ? -1.0 : 1.0) * sg * G0[a * deg + b];
    }
  // s: scaling coefficients of cells of the current level, each row restricted to its
  // cell's support of width w columns (w = deg 2^(lev - L))
  int ncell = 1 << lev, w = deg;
  std::vector<double> s(static_cast<size_t>(n) * deg, 0.0), ns;  // [ncell][deg][w]
  for (int c = 0; c < ncell; ++c)
    for (int a = 0; a < deg; ++a) s[(static_cast<size_t>(c) * deg + a) * w + a] = 1.0;
  for (int L = lev; L >= 1; --L) {
    const int nc = ncell / 2, w2 = 2 * w;
    ns.assign(static_cast<size_t>(nc) * deg * w2, 0.0);
    const long long r0 = static_cast<long long>(deg) * nc;  // first wavelet row of level L
    for (int c = 0; c < nc; ++c) {
      const double* left = &s[static_cast<size_t>(2 * c) * deg * w];
      const double* right = &s[static_cast<size_t>(2 * c + 1) * deg * w];
      for (int a = 0; a < deg; ++a) {
        double* sr = &ns[(static_cast<size_t>(c) * deg + a) * w2];
        const long long row = r0 + static_cast<long long>(c) * deg + a;
        double* dr = F + row * n + static_cast<long long>(c) * w2;
        for (int b = 0; b < deg; ++b) {
          const double h0 = H0[a * deg + b], h1 = H1[a * deg + b], g0 = G0[a * deg + b], g1 = G1[a * deg + b];
          for (int x = 0; x < w; ++x) {
            sr[x] += h0 * left[b * w + x];
            sr[w + x] += h1 * right[b * w + x];
            dr[x] += g0 * left[b * w + x];
            dr[w + x] += g1 * right[b * w + x];
          }
        }
        c0[row] = c * w2;
        c1[row] = (c + 1) * w2;
      }
    }
    s.swap(ns);
    ncell = nc;
    w = w2;
  }
  for (int a = 0; a < deg; ++a) {
    std::memcpy(F + a * n, &s[static_cast<size_t>(a) * w], sizeof(double) * n);
    c0[a] = 0;
    c1[a] = static_cast<int>(n);
  }
}

// A block-sparse realspace matrix: deg x deg blocks (row-major) at (block row, block column)
struct Block {
  int r, c;
  std::vector<double> v;
};

struct Term {
  int kind;  // 0 mass, 1 div, 2 grad
  double LF;
  char bcl, bcr;  // as given
  const double* gq;
  const double* gf;
};

// Realspace matrix of one partial term on 2^lev cells (coeff_matrix.m:105-323): volume
// integrals with nq-point Gauss rules per cell, trace blocks with the Lax-Friedrichs flux,
// Dirichlet / Neumann / periodic ends; GRAD negates the flux, swaps D and N and returns the
// negated transpose (GRAD.m:14-34, coeff_matrix.m:323).
std::vector<Block> realspace(int deg, int lev, double lo, double hi, const Term& t, const double* xq,
                             const double* wq, int nq) {
  const int N = 1 << lev;
  const double h = (hi - lo) / N, J = h / 2, sh = std::sqrt(h);
  std::vector<double> V(nq * deg), dV(nq * deg), pL(deg), pR(deg);
  for (int q = 0; q < nq; ++q) {
    legendre_values(xq[q], deg, &V[q * deg]);
    legendre_derivs(xq[q], deg, &dV[q * deg]);
    for (int a = 0; a < deg; ++a) {
      V[q * deg + a] /= sh;
      dV[q * deg + a] = dV[q * deg + a] / sh * 2 / h;
    }
  }
  legendre_values(-1.0, deg, pL.data());
  legendre_values(1.0, deg, pR.data());
  for (int a = 0; a < deg; ++a) {
    pL[a] /= sh;
    pR[a] /= sh;
  }
  const bool grad = t.kind == 2;
  const double LF = grad ? -t.LF : t.LF;
  auto swap_dn = [&](char c) { return grad ? (c == 'D' ? 'N' : (c == 'N' ? 'D' : c)) : c; };
  const char bcl = swap_dn(t.bcl), bcr = swap_dn(t.bcr);
  std::vector<Block> out;
  out.reserve(static_cast<size_t>(N) * 5);
  const int dd = deg * deg;
  for (int c = 0; c < N; ++c) {
    Block vol{c, c, std::vector<double>(dd, 0.0)};
    for (int a = 0; a < deg; ++a)
      for (int b = 0; b < deg; ++b) {
        double s = 0.0;
        for (int q = 0; q < nq; ++q) {
          const double g = t.gq ? t.gq[static_cast<size_t>(c) * nq + q] : 1.0;
          s += (t.kind == 0 ? V[q * deg + a] : dV[q * deg + a]) * (g * wq[q]) * V[q * deg + b];
        }
        vol.v[a * deg + b] = t.kind == 0 ? s * J : -s * J;
      }
    out.push_back(std::move(vol));
  }
  if (t.kind != 0) {
    const bool periodic = bcl == 'P' || bcr == 'P';
    for (int c = 0; c < N; ++c) {
      const double gL = t.gf ? t.gf[c] : 1.0, gR = t.gf ? t.gf[c + 1] : 1.0;
      const double cL = gL / 2 + LF * std::fabs(gL) / 2, aL = LF * std::fabs(gL) / 2;
      const double aR = LF * std::fabs(gR) / 2;
      std::vector<double> B[4];
      for (auto& x : B) x.assign(dd, 0.0);
      for (int a = 0; a < deg; ++a)
        for (int b = 0; b < deg; ++b) {
          B[0][a * deg + b] = -pL[a] * pR[b] * cL;
          B[1][a * deg + b] = -pL[a] * pL[b] * gL / 2 + aL * (pL[a] * pL[b]);
          B[2][a * deg + b] = pR[a] * pR[b] * gR / 2 + aR * (pR[a] * pR[b]);
          B[3][a * deg + b] = pR[a] * pL[b] * gR / 2 + aR * (-pR[a] * pL[b]);
        }
      if (c == 0 && bcl == 'D') B[0].assign(dd, 0.0), B[1].assign(dd, 0.0);
      if (c == N - 1 && bcr == 'D') B[2].assign(dd, 0.0), B[3].assign(dd, 0.0);
      if (c == 0 && bcl == 'N') {
        B[0].assign(dd, 0.0);
        for (int a = 0; a < deg; ++a)
          for (int b = 0; b < deg; ++b) B[1][a * deg + b] = -pL[a] * pL[b] * gL;
      }
      if (c == N - 1 && bcr == 'N') {
        for (int a = 0; a < deg; ++a)
          for (int b = 0; b < deg; ++b) B[2][a * deg + b] = pR[a] * pR[b] * gR;
        B[3].assign(dd, 0.0);
      }
      int nbr[4] = {c - 1, c, c, c + 1};
      bool use[4] = {true, true, true, true};
      if (periodic) {
        if (lev >= 1) {
          nbr[0] = (c - 1 + N) % N;
          nbr[3] = (c + 1) % N;
        } else {
          nbr[0] = nbr[3] = c;
        }
      } else {
        if (c == 0) use[0] = false;
        if (c == N - 1) use[3] = false;
      }
      for (int k = 0; k < 4; ++k)
        if (use[k]) out.push_back(Block{c, nbr[k], B[k]});
    }
    if (grad)  // -M^T
      for (auto& bl : out) {
        std::swap(bl.r, bl.c);
        std::vector<double> tv(dd);
        for (int a = 0; a < deg; ++a)
          for (int b = 0; b < deg; ++b) tv[a * deg + b] = -bl.v[b * deg + a];
        bl.v.swap(tv);
      }
  }
  return out;
}

// Inverse of a small dense matrix by Gauss-Jordan elimination with partial pivoting.
bool invert(int n, const double* A, double* X) {
  std::vector<double> M(A, A + n * n);
  for (int i = 0; i < n * n; ++i) X[i] = 0.0;
  for (int i = 0; i < n; ++i) X[i * n + i] = 1.0;
  for (int c = 0; c < n; ++c) {
    int p = c;
    for (int r = c + 1; r < n; ++r)
      if (std::fabs(M[r * n + c]) > std::fabs(M[p * n + c])) p = r;
    if (M[p * n + c] == 0.0) return false;
    if (p != c)
      for (int k = 0; k < n; ++k) {
        std::swap(M[p * n + k], M[c * n + k]);
        std::swap(X[p * n + k], X[c * n + k]);
      }
    const double d = M[c * n + c];
    for (int k = 0; k < n; ++k) {
      M[c * n + k] /= d;
      X[c * n + k] /= d;
    }
    for (int r = 0; r < n; ++r) {
      if (r == c) continue;
      const double f = M[r * n + c];
      if (f == 0.0) continue;
      for (int k = 0; k < n; ++k) {
        M[r * n + k] -= f * M[c * n + k];
        X[r * n + k] -= f * X[c * n + k];
      }
    }
  }
  return true;
}

// Runs body(lo, hi) over [0, n) in contiguous chunks on up to 16 host threads; chunks whose
// thread cannot be started run on the calling thread.
template <typename F>
void parallel_rows(long long n, F body) {
  const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
  const int T = static_cast<int>(std::min<long long>(std::min(16u, hw), std::max(1LL, n / 256)));
  std::vector<std::thread> th;
  int k = 1;  // chunk 0 runs here
  try {
    th.reserve(T);
    for (; k < T; ++k) th.emplace_back(body, n * k / T, n * (k + 1) / T);
  } catch (...) {
  }
  body(0LL, n / T);
  for (int r = k; r < T; ++r) body(n * r / T, n * (r + 1) / T);
  for (auto& x : th) x.join();
}

asg_status coeff_matrix(int deg, int lev, double lo, double hi, int nterms, const asg_partial_term* terms,
                        double* out) {
  if (deg < 1 || deg > 16 || lev < 0 || lev > 14 || (static_cast<long long>(deg) << lev) > 16384 || !out)
    return fail(ASG_ERR_INVALID, "coeff_matrix: deg=%d lev=%d (deg 1..16, deg*2^lev <= 16384, non-NULL out)", deg, lev);
  if (!(hi > lo)) return fail(ASG_ERR_INVALID, "coeff_matrix: empty interval [%g, %g]", lo, hi);
  if (nterms < 1 || !terms) return fail(ASG_ERR_INVALID, "coeff_matrix: nterms=%d (>= 1 partial terms)", nterms);
  for (int k = 0; k < nterms; ++k) {
    const asg_partial_term& t = terms[k];
    if (t.kind < 0 || t.kind > 2) return fail(ASG_ERR_INVALID, "coeff_matrix: term %d kind=%d (0 mass, 1 div, 2 grad)", k, t.kind);
    auto ok = [](char c) { return c == 'P' || c == 'D' || c == 'N'; };
    if (!ok(t.bcl) || !ok(t.bcr))
      return fail(ASG_ERR_INVALID, "coeff_matrix: term %d boundary types '%c' '%c' (P, D or N)", k, t.bcl ? t.bcl : '?',
                  t.bcr ? t.bcr : '?');
  }
  const int nq = quad_count(deg), N = 1 << lev, dd = deg * deg;
  const long long n = static_cast<long long>(deg) << lev;
  std::vector<double> xq(nq), wq(nq);
  gauss_legendre(nq, -1.0, 1.0, xq.data(), wq.data());
  // unit LHS mass: block-diagonal, inverted block by block
  const Term unit{0, 0.0, 'P', 'P', nullptr, nullptr};
  std::vector<Block> Mr = realspace(deg, lev, lo, hi, unit, xq.data(), wq.data(), nq);
  std::vector<double> Minv(static_cast<size_t>(N) * dd);
  for (int c = 0; c < N; ++c)
    if (!invert(deg, Mr[c].v.data(), &Minv[static_cast<size_t>(c) * dd]))
      return fail(ASG_ERR_INVALID, "coeff_matrix: singular mass block at cell %d", c);
  // factors M^-1 L_k, grouped by block row.  A mass term with g = 1 at every node has the
  // LHS mass's own matrix, so its factor is exactly the identity (the reference's
  // M_w \ M_w) and is left out; a chain of such terms is exactly the identity.
  std::vector<std::vector<std::vector<Block>>> fac;
  for (int k = 0; k < nterms; ++k) {
    if (terms[k].kind == 0) {
      bool unit_mass = true;
      if (terms[k].g_quad)
        for (long long x = 0; x < static_cast<long long>(N) * nq && unit_mass; ++x) unit_mass = terms[k].g_quad[x] == 1.0;
      if (unit_mass) continue;
    }
    fac.emplace_back();
    const Term t{terms[k].kind, terms[k].LF, terms[k].bcl, terms[k].bcr, terms[k].g_quad, terms[k].g_face};
    std::vector<Block> L = realspace(deg, lev, lo, hi, t, xq.data(), wq.data(), nq);
    fac.back().assign(N, {});
    for (auto& bl : L) {
      const double* mi = &Minv[static_cast<size_t>(bl.r) * dd];
      std::vector<double> v(dd, 0.0);
      for (int a = 0; a < deg; ++a)
        for (int x = 0; x < deg; ++x)
          for (int b = 0; b < deg; ++b) v[a * deg + b] += mi[a * deg + x] * bl.v[x * deg + b];
      fac.back()[bl.r].push_back(Block{bl.r, bl.c, std::move(v)});
    }
  }
  if (fac.empty()) {
    std::memset(out, 0, sizeof(double) * n * n);
    for (long long i = 0; i < n; ++i) out[i * n + i] = 1.0;
    return ASG_OK;
  }
  // Y = F (M^-1 L_1) (M^-1 L_2) ..., each row within its nonzero block range; then out = Y F^T
  std::vector<double> F(static_cast<size_t>(n) * n);
  std::vector<int> c0(n), c1(n);
  fmwt(deg, lev, F.data(), c0.data(), c1.data());
  std::vector<double> Y(F), Z(static_cast<size_t>(n) * n);
  std::vector<int> b0(n), b1(n), nb0(n), nb1(n);
  for (long long r = 0; r < n; ++r) {
    b0[r] = c0[r] / deg;
    b1[r] = (c1[r] + deg - 1) / deg;
  }
  for (size_t k = 0; k < fac.size(); ++k) {
    parallel_rows(n, [&](long long r0, long long r1) {
      for (long long r = r0; r < r1; ++r) {
        double* z = &Z[static_cast<size_t>(r) * n];
        const double* y = &Y[static_cast<size_t>(r) * n];
        std::fill(z, z + n, 0.0);
        int lo_b = N, hi_b = 0;
        for (int rb = b0[r]; rb < b1[r]; ++rb)
          for (const Block& bl : fac[k][rb]) {
            const double* yv = y + static_cast<size_t>(rb) * deg;
            double* zv = z + static_cast<size_t>(bl.c) * deg;
            for (int a = 0; a < deg; ++a) {
              const double ya = yv[a];
              if (ya == 0.0) continue;
              for (int b = 0; b < deg; ++b) zv[b] += ya * bl.v[a * deg + b];
            }
            lo_b = std::min(lo_b, bl.c);
            hi_b = std::max(hi_b, bl.c + 1);
          }
        nb0[r] = lo_b < hi_b ? lo_b : 0;
        nb1[r] = lo_b < hi_b ? hi_b : 0;
      }
    });
    Y.swap(Z);
    b0.swap(nb0);
    b1.swap(nb1);
  }
  parallel_rows(n, [&](long long r0, long long r1) {
    for (long long i = r0; i < r1; ++i) {
      const double* y = &Y[static_cast<size_t>(i) * n];
      const long long lo_c = static_cast<long long>(b0[i]) * deg, hi_c = static_cast<long long>(b1[i]) * deg;
      double* o = out + i * n;
      for (long long j = 0; j < n; ++j) {
        const double* f = &F[static_cast<size_t>(j) * n];
        const long long a0 = std::max<long long>(lo_c, c0[j]), a1 = std::min<long long>(hi_c, c1[j]);
        double s = 0.0;
        for (long long x = a0; x < a1; ++x) s += y[x] * f[x];
        o[j] = s;
      }
    }
  });
  return ASG_OK;
}

}  // namespace

extern "C" {

asg_status asg_gauss_legendre_f64(int n, double a, double b, double* x, double* w) {
  if (n < 1 || n > 4096 || !x || !w) return fail(ASG_ERR_INVALID, "gauss_legendre: n=%d (1..4096) and non-NULL x, w", n);
  if (n == 1) {
    x[0] = (a + b) / 2;
    w[0] = b - a;
    return ASG_OK;
  }
  gauss_legendre(n, a, b, x, w);
  return ASG_OK;
}

asg_status asg_multiwavelet_filters_f64(int deg, double* H0, double* G0) {
  if (deg < 1 || deg > 16 || !H0 || !G0) return fail(ASG_ERR_INVALID, "multiwavelet_filters: deg=%d (1..16) and non-NULL H0, G0", deg);
  multiwavelet_filters(deg, H0, G0);
  return ASG_OK;
}

asg_status asg_fmwt_matrix_f64(int deg, int lev, double* F) {
  if (deg < 1 || deg > 16 || lev < 0 || lev > 14 || (static_cast<long long>(deg) << lev) > 16384 || !F)
    return fail(ASG_ERR_INVALID, "fmwt_matrix: deg=%d lev=%d (deg 1..16, deg*2^lev <= 16384, non-NULL F)", deg, lev);
  const long long n = static_cast<long long>(deg) << lev;
  try {
    std::vector<int> c0(n), c1(n);
    fmwt(deg, lev, F, c0.data(), c1.data());
  } catch (const std::bad_alloc&) {
    return fail(ASG_ERR_NOMEM, "fmwt_matrix: out of host memory");
  }
  return ASG_OK;
}

asg_status asg_coeff_matrix_f64(int deg, int lev, double lo, double hi, int nterms, const asg_partial_term* terms,
                                double* out) {
  try {
    return coeff_matrix(deg, lev, lo, hi, nterms, terms, out);
  } catch (const std::bad_alloc&) {
    return fail(ASG_ERR_NOMEM, "coeff_matrix: out of host memory (three %lld x %lld work matrices)",
                static_cast<long long>(deg) << lev, static_cast<long long>(deg) << lev);
  }
}

}  // extern "C"
