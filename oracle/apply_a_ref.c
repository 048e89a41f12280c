/*
 * CPU oracle in plain C -- TEST INFRASTRUCTURE ONLY (also the timed CPU baseline).
 *
 * Faithful restatement of the reference's operator application loop, FP64:
 *   apply_A.m:102-236  for each row element, for each column (all, or the connectivity
 *                      list), for each term: extract the deg x deg blocks
 *                      A_{t,k}[I_k(row), J_k(col)] (apply_A.m:163-168) and accumulate
 *                      kron_multd(d, blocks, f_col) into the row block (apply_A.m:185-201)
 *   kron_multd.m / Kronmult/kronmult{1..6}.m method 1: apply A_d to the fastest index
 *                      first, then A_{d-1}, ..., A_1 (kronmult1.m:17, kronmult2.m:66-139,
 *                      kronmult3.m:47-88)
 * Rows are independent, so OpenMP splits them across threads; the per-row order of the
 * sums is the reference's (columns in list order, terms in order).
 */
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define MAXD 6

static void mode_product(const double* in, double* out, const double* A, int P, int B, int s) {
  /* out[.., a, ..] = sum_b A[a][b] in[.., b, ..] along the index with stride s */
  const int nf = B / P;
  for (int fi = 0; fi < nf; ++fi) {
    const int hi = fi / s, lo = fi % s;
    const int base = hi * s * P + lo;
    for (int a = 0; a < P; ++a) {
      double acc = 0.0;
      for (int b = 0; b < P; ++b) acc += A[a * P + b] * in[base + b * s];
      out[base + a * s] = acc;
    }
  }
}

/*
 * D, P, T, N: dims, degree, terms, elements.  idx1d[N*D] 0-based 1-D indices.
 * ops[T*D]: column-major operators with leading dimension ld[T*D].
 * row_ptr/cols: CSR pair list (0-based) or row_ptr == NULL for all pairs.
 * rows[nrows]: the row elements to compute; y[nrows*P^D] receives their blocks.
 * Returns 0, or -1 on bad arguments.
 */
int oracle_apply_rows(int D, int P, int T, int N, const int* idx1d, const double* const* ops, const int* ld,
                      const long long* row_ptr, const int* cols, const double* f, const int* rows, int nrows,
                      double* y, int nthreads) {
  if (D < 1 || D > MAXD || P < 1 || T < 1 || N < 0 || nrows < 0) return -1;
  int B = 1;
  for (int k = 0; k < D; ++k) B *= P;
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#else
  (void)nthreads;
#endif
  int bad = 0;
#pragma omp parallel
  {
    double* buf0 = (double*)malloc(sizeof(double) * B);
    double* buf1 = (double*)malloc(sizeof(double) * B);
    double* blk = (double*)malloc(sizeof(double) * MAXD * P * P);
    int stride[MAXD];
    int s = 1;
    for (int m = D - 1; m >= 0; --m) {
      stride[m] = s;
      s *= P;
    }
#pragma omp for schedule(dynamic, 1)
    for (int r = 0; r < nrows; ++r) {
      const int i = rows[r];
      double* yi = y + (size_t)r * B;
      memset(yi, 0, sizeof(double) * B);
      if (i < 0 || i >= N) {
        bad = 1;
        continue;
      }
      const long long q0 = row_ptr ? row_ptr[i] : 0, q1 = row_ptr ? row_ptr[i + 1] : N;
      for (long long q = q0; q < q1; ++q) {
        const int j = row_ptr ? cols[q] : (int)q;
        for (int t = 0; t < T; ++t) {
          for (int m = 0; m < D; ++m) {
            const double* op = ops[t * D + m];
            const int L = ld[t * D + m];
            const int r0 = idx1d[i * D + m] * P, c0 = idx1d[j * D + m] * P;
            for (int a = 0; a < P; ++a)
              for (int b = 0; b < P; ++b) blk[m * P * P + a * P + b] = op[(size_t)(c0 + b) * L + (r0 + a)];
          }
          memcpy(buf0, f + (size_t)j * B, sizeof(double) * B);
          double* in = buf0;
          double* out = buf1;
          for (int m = D - 1; m >= 0; --m) {
            mode_product(in, out, blk + m * P * P, P, B, stride[m]);
            double* tmp = in;
            in = out;
            out = tmp;
          }
          for (int k = 0; k < B; ++k) yi[k] += in[k];
        }
      }
    }
    free(buf0);
    free(buf1);
    free(blk);
  }
  return bad ? -1 : 0;
}
