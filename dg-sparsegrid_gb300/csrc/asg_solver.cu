// Time steppers built on the operator application (time_advance.m):
//   asg_rk3_step_*   RungeKutta3 (time_advance.m:151-204) with fused stage updates
//   asg_be_solve_*   backward Euler (time_advance.m:267-349): the reference assembles A and
//                    solves (I - dt A) f1 = b directly; here the system is solved matrix-free
//                    by restarted GMRES inside iterative refinement.  Mixed mode: FP32
//                    operator application inside GMRES, FP64 for the outer residual, the
//                    solution update and every Arnoldi dot product and norm.
// All reductions are two-pass and fixed-order, so results are bitwise reproducible.
#include <algorithm>
#include <type_traits>
#include <cmath>
#include <vector>

#include "asg_internal.h"
#include "asg_rows.cuh"

namespace asg {
namespace {

constexpr int kRedBlocks = 304;  // most partial sums per reduction (2 per SM)
constexpr int kMaxRestart = 64;  // largest GMRES restart length (Hessenberg staged in shared memory)
constexpr int kRedThreads = 256;
// partial sums for a reduction over n values: one block per 4096 values, at most kRedBlocks
inline int red_blocks(long long n) {
  const long long b = (n + 4095) / 4096;
  return static_cast<int>(b < 1 ? 1 : (b > kRedBlocks ? kRedBlocks : b));
}
// sum of nb partials by one warp: lane-strided sums, then a fixed shuffle tree (lane 0 has it)
__device__ __forceinline__ double warp_sum_partials(const double* __restrict__ p, int nb, int lane) {
  double s = 0.0;
  for (int b = lane; b < nb; b += 32) s += p[b];
  for (int off = 16; off > 0; off >>= 1) s += __shfl_down_sync(0xffffffffu, s, off);
  return s;
}

// ---------------------------------------------------------------------------------------
// RK3 stage updates (time_advance.m:177-204):
//   stage 1: k1 = A f + s1;             y = f + dt/2 k1
//   stage 2: k2 = A y + s2;             y = f + dt (-k1 + 2 k2)
//   stage 3: k3 = A y + s3;             f = f + dt (k1/6 + 2 k2/3 + k3/6)
// ---------------------------------------------------------------------------------------
// The stage sources of an RK3 step: three precomputed vectors (or NULL), or ns device vectors
// combined with the stage's ns device coefficients (coef[3*ns]: t, t + dt/2, t + dt), summed
// in FP64 as asg_lincomb_f64 sums them and rounded once to the step's type.
template <typename T>
struct Rk3Src {
  const T* src[3];
  int ns;
  const double* coef;
  const double* const* vecs;
};
template <typename T>
__device__ __forceinline__ T rk3_source(const Rk3Src<T>& S, int k, long long i) {
  if (S.ns > 0) {
    double acc = 0.0;
    for (int q = 0; q < S.ns; ++q) acc = fma(S.coef[k * S.ns + q], S.vecs[q][i], acc);
    return static_cast<T>(acc);
  }
  return S.src[k] ? S.src[k][i] : T(0);
}

// One value's update after a stage's operator application v (= (A x)_i) with the stage's
// source si: the stage kernel and the fused step both call it, so the two paths round alike.
template <typename T>
__device__ __forceinline__ void rk3_update(int stage, long long i, T v, T dt, T si, T* f, T* y, T* k1, T* k2) {
  if (stage == 1) {
    const T a = v + si;
    k1[i] = a;
    y[i] = f[i] + dt * T(0.5) * a;
  } else if (stage == 2) {
    const T b = v + si;
    k2[i] = b;
    y[i] = f[i] + dt * (T(-1) * k1[i] + T(2) * b);
  } else {
    const T c = v + si;
    f[i] = f[i] + dt * (k1[i] / T(6) + T(2) / T(3) * k2[i] + c / T(6));
  }
}

template <typename T>
__global__ void k_rk3_stage(int stage, long long n, T dt, T* __restrict__ f, T* __restrict__ y, T* __restrict__ k1,
                            T* __restrict__ k2, T* __restrict__ k3, Rk3Src<T> S) {
  const T* kv = stage == 1 ? k1 : (stage == 2 ? k2 : k3);
  for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<long long>(gridDim.x) * blockDim.x)
    rk3_update(stage, i, kv[i], dt, rk3_source(S, stage - 1, i), f, y, k1, k2);
}

// out = sum_s c[s] * v[s]  (sources s(t) = sum_s c_s(t) v_s, c on the device)
template <typename T>
__global__ void k_lincomb(long long n, int ns, const T* __restrict__ c, const T* const* __restrict__ v,
                          T* __restrict__ out) {
  for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<long long>(gridDim.x) * blockDim.x) {
    T acc = T(0);
    for (int q = 0; q < ns; ++q) acc = fma(c[q], v[q][i], acc);
    out[i] = acc;
  }
}

// ---------------------------------------------------------------------------------------
// GMRES helpers.  Basis vectors V (FP32 in mixed mode, FP64 otherwise), FP64 work vectors.
// ---------------------------------------------------------------------------------------
// partial[b] = sum of x^2 over block b's slice
__global__ void __launch_bounds__(kRedThreads) k_norm2(long long n, const double* __restrict__ x,
                                                       double* __restrict__ partial) {
  __shared__ double red[kRedThreads / 32];
  double acc = 0.0;
  for (long long i = blockIdx.x * static_cast<long long>(kRedThreads) + threadIdx.x; i < n;
       i += static_cast<long long>(gridDim.x) * kRedThreads)
    acc = fma(x[i], x[i], acc);
  for (int off = 16; off > 0; off >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, off);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int q = 0; q < kRedThreads / 32; ++q) s += red[q];
    partial[blockIdx.x] = s;
  }
}
// V_j = w * inv  (stored in the basis precision)
template <typename TV>
__global__ void k_store_basis(long long n, double inv, const double* __restrict__ w, TV* __restrict__ vj) {
  for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<long long>(gridDim.x) * blockDim.x)
    vj[i] = static_cast<TV>(w[i] * inv);
}
// r = b - (x - dt * ax)   (FP64 outer residual)
__global__ void k_residual(long long n, double dt, const double* __restrict__ b, const double* __restrict__ x,
                           const double* __restrict__ ax, double* __restrict__ r) {
  for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<long long>(gridDim.x) * blockDim.x)
    r[i] = b[i] - (x[i] - dt * ax[i]);
}
// ---- device-side Arnoldi/Givens state: a cycle runs without a host round trip per step ----
struct GmresState {
  int done;      // cycle finished (converged, breakdown or m steps): later kernels return
  int kdone;     // Arnoldi steps taken
  double resid;  // |g[kdone]|, the residual estimate
  double inv;    // 1 / ||w|| of the last step (scales the next basis vector)
  unsigned bar[3];  // fused solve's grid barrier: arrivals, (unused), timeout flag
  int outer, inner, converged;  // fused solve's result
  double rel;
};
// w = V_j - dt * (A V_j), skipped once the cycle is done
template <typename TV, typename TA>
__global__ void k_shift_g(long long n, double dt, const TV* __restrict__ x, const TA* __restrict__ ax,
                          double* __restrict__ w, const GmresState* __restrict__ st) {
  if (st->done) return;
  for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<long long>(gridDim.x) * blockDim.x)
    w[i] = static_cast<double>(x[i]) - dt * static_cast<double>(ax[i]);
}
// out = x rounded to TA (the operand of an operator application in another precision),
// skipped once the cycle is done
template <typename TV, typename TA>
__global__ void k_round_g(long long n, const TV* __restrict__ x, TA* __restrict__ out,
                          const GmresState* __restrict__ st) {
  if (st->done) return;
  for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<long long>(gridDim.x) * blockDim.x)
    out[i] = static_cast<TA>(x[i]);
}
// partial[j * gridDim.x + b] = block b's share of <w, V_j> (FP64), j = blockIdx.y
template <typename TV>
__global__ void __launch_bounds__(kRedThreads) k_dots_g(long long n, const double* __restrict__ w,
                                                        const TV* __restrict__ V, long long ldv,
                                                        double* __restrict__ partial,
                                                        const GmresState* __restrict__ st) {
  if (st->done) return;
  __shared__ double red[kRedThreads / 32];
  const int j = blockIdx.y;
  const TV* v = V + j * ldv;
  double acc = 0.0;
  for (long long i = blockIdx.x * static_cast<long long>(kRedThreads) + threadIdx.x; i < n;
       i += static_cast<long long>(gridDim.x) * kRedThreads)
    acc = fma(w[i], static_cast<double>(v[i]), acc);
  for (int off = 16; off > 0; off >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, off);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int q = 0; q < kRedThreads / 32; ++q) s += red[q];
    partial[j * static_cast<long long>(gridDim.x) + blockIdx.x] = s;
  }
}
// h[j] = sum_b partial (one warp per j, fixed order); the Hessenberg column accumulates both
// CGS passes
__global__ void k_dots_final_g(int k, int nb, const double* __restrict__ partial, double* __restrict__ h,
                               double* __restrict__ hcol, int pass, const GmresState* __restrict__ st) {
  if (st->done) return;
  const int j = blockIdx.x;
  if (j >= k) return;
  const double s = warp_sum_partials(partial + j * static_cast<long long>(nb), nb, threadIdx.x);
  if (threadIdx.x == 0) {
    h[j] = s;
    hcol[j] = pass ? hcol[j] + s : s;
  }
}
// w -= sum_{j<k} h[j] V_j
template <typename TV>
__global__ void k_orth_update_g(long long n, int k, const double* __restrict__ h, const TV* __restrict__ V,
                                long long ldv, double* __restrict__ w, const GmresState* __restrict__ st) {
  if (st->done) return;
  for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<long long>(gridDim.x) * blockDim.x) {
    double acc = w[i];
    for (int j = 0; j < k; ++j) acc = fma(-h[j], static_cast<double>(V[j * ldv + i]), acc);
    w[i] = acc;
  }
}
__global__ void __launch_bounds__(kRedThreads) k_norm2_g(long long n, const double* __restrict__ x,
                                                         double* __restrict__ partial,
                                                         const GmresState* __restrict__ st) {
  if (st->done) return;
  __shared__ double red[kRedThreads / 32];
  double acc = 0.0;
  for (long long i = blockIdx.x * static_cast<long long>(kRedThreads) + threadIdx.x; i < n;
       i += static_cast<long long>(gridDim.x) * kRedThreads)
    acc = fma(x[i], x[i], acc);
  for (int off = 16; off > 0; off >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, off);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int q = 0; q < kRedThreads / 32; ++q) s += red[q];
    partial[blockIdx.x] = s;
  }
}
// Step j of the Givens QR of the Hessenberg matrix (one thread): ||w|| from the partials,
// the previous rotations on the new column, a new rotation, the residual estimate and the
// stopping decision.
__global__ void k_givens(int j, int m, double target, int nb, const double* __restrict__ partial,
                         double* __restrict__ hcol, double* __restrict__ H, double* __restrict__ cs,
                         double* __restrict__ sn, double* __restrict__ g, GmresState* __restrict__ st) {
  if (st->done) return;
  __shared__ double hc[kMaxRestart + 1], c_s[kMaxRestart], s_s[kMaxRestart];
  const int lane = threadIdx.x;
  const double acc = warp_sum_partials(partial, nb, lane);
  for (int i = lane; i <= j; i += 32) hc[i] = hcol[i];  // the column and rotations, staged once
  for (int i = lane; i < j; i += 32) {
    c_s[i] = cs[i];
    s_s[i] = sn[i];
  }
  __syncwarp();
  if (lane == 0) {
    const double hn = sqrt(acc);
    hc[j + 1] = hn;
    for (int i = 0; i < j; ++i) {
      const double a = c_s[i] * hc[i] + s_s[i] * hc[i + 1];
      hc[i + 1] = -s_s[i] * hc[i] + c_s[i] * hc[i + 1];
      hc[i] = a;
    }
    const double den = hypot(hc[j], hc[j + 1]);
    const double c = den > 0 ? hc[j] / den : 1.0, sv = den > 0 ? hc[j + 1] / den : 0.0;
    cs[j] = c;
    sn[j] = sv;
    hc[j] = den;
    const double gj = g[j];
    g[j + 1] = -sv * gj;
    g[j] = c * gj;
    st->resid = fabs(sv * gj);
    st->inv = hn > 0 ? 1.0 / hn : 0.0;
    st->kdone = j + 1;
    st->done = (st->resid <= target || hn == 0.0 || j + 1 == m) ? 1 : 0;
  }
  __syncwarp();
  for (int i = lane; i <= j; i += 32) H[static_cast<long long>(i) * m + j] = hc[i];
}
// V_{j+1} = w / ||w|| (skipped once the cycle is done)
template <typename TV>
__global__ void k_store_basis_g(long long n, const double* __restrict__ w, TV* __restrict__ vj,
                                const GmresState* __restrict__ st) {
  if (st->done) return;
  const double inv = st->inv;
  for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<long long>(gridDim.x) * blockDim.x)
    vj[i] = static_cast<TV>(w[i] * inv);
}
// y = H(1:k,1:k) \ g(1:k), k = kdone (one thread, upper triangular)
__global__ void k_backsolve(int m, const double* __restrict__ H, const double* __restrict__ g, double* __restrict__ y,
                            const GmresState* __restrict__ st) {
  __shared__ double hs[kMaxRestart * kMaxRestart], ys[kMaxRestart];
  const int k = st->kdone;
  for (int q = threadIdx.x; q < k * k; q += blockDim.x) hs[q] = H[static_cast<long long>(q / k) * m + q % k];
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int i = k - 1; i >= 0; --i) {
      double acc = g[i];
      for (int q = i + 1; q < k; ++q) acc -= hs[i * k + q] * ys[q];
      ys[i] = acc / hs[i * k + i];
    }
  }
  __syncthreads();
  for (int q = threadIdx.x; q < k; q += blockDim.x) y[q] = ys[q];
}
// x += sum_{j < kdone} y[j] V_j  (FP64 solution update)
template <typename TV>
__global__ void k_sol_update_g(long long n, const double* __restrict__ y, const TV* __restrict__ V, long long ldv,
                               double* __restrict__ x, const GmresState* __restrict__ st) {
  const int k = st->kdone;
  for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<long long>(gridDim.x) * blockDim.x) {
    double acc = x[i];
    for (int j = 0; j < k; ++j) acc = fma(y[j], static_cast<double>(V[j * ldv + i]), acc);
    x[i] = acc;
  }
}

// ---------------------------------------------------------------------------------------
// Fused backward-Euler solve for plans on the small-block single-mode kernel: one cooperative
// launch solves (I - dt A) x = b -- the FP64 outer residuals, their norms and the stopping
// test, and every restarted GMRES(m) cycle on the correction (basis and operator in TV).  CTA
// b owns a contiguous range of element rows (balanced by work entries) and keeps its slices
// of the Krylov basis V and of Z = (I - dt A) V in shared memory, so everything but the
// operator applications and the grid-wide sums stays on chip.  A restart: r = b - (x - dt A x)
// in FP64 for the CTA's rows and ||r|| (one grid barrier), the stopping test, v_0 = r / ||r||
// published (one barrier) and Z_0; then per Arnoldi step, with w = Z_j:
//   1. first Gram-Schmidt pass's partial dots <w, v_k>                     -> grid barrier
//   2. h = grid sums, w' = w - V h (published), second pass's partial dots and ||w'||^2
//                                                                          -> grid barrier
//   3. h2 = grid sums, ||w||^2 = ||w'||^2 - ||h2||^2 (an explicit sum, with one more barrier,
//      when ||h2||^2 > 1e-2 ||w'||^2), the Givens step, v_{j+1} = (w' - V h2) / ||w||, and
//      (I - dt A) w' for the CTA's rows (the rows' entries cut into chunks over the warps,
//      chunk sums added per row in a fixed order; w' read from its global copy), giving
//      Z_{j+1} = ((I - dt A) w' - Z h2) / ||w|| without a barrier to publish v_{j+1};
// after the last step R y = g (every CTA holds the same R and g) and x += V y over the CTA's
// slice (one barrier before the next residual).  Every CTA reduces the same partials in the
// same order and runs the same recurrences, so all take the same decisions.  Fixed-order
// reductions: bitwise reproducible.  Grid barrier waits are bounded (~2^31 cycles): on
// expiry the kernel records the timeout and returns.
// ---------------------------------------------------------------------------------------
constexpr int kFzThreads = 512;
constexpr int kFzWarps = kFzThreads / 32;
constexpr int kFzGivensWarps = 2;  // warps that run the Givens step while the others apply the operator

template <typename TV, typename TA>
struct FusedArgs {
  ApplyArgs<TA> a;             // the plan's apply arguments in the application precision (f, y unused)
  ApplyArgs<double> a64;       // and in FP64, for the outer residual
  long long n, ldv;
  double dt, tol, inner_reduction;
  int m, max_outer;
  TA* V;                       // global copy of the vector the operator is applied to (n values)
  double* partial;             // (2m + 2) rows of gridDim.x CTA partials
  const double* rhs;           // b
  double* x;                   // initial guess in, solution out
  GmresState* state;           // zeroed before the launch; bar[] is the grid barrier
  const int* blk_row;          // [G+1] row range of CTA b
  const int* blk_slot;         // [G+1] its partial-sum slots
  const int* row_slot;         // [N+1] slots of each row
  const int* warp_item;        // [G*W+1] items of warp w of CTA b
  const FzItem* items;
  int max_rows, max_slots;
  int withhold;                // test hook: barrier at which CTA 0 does not arrive (-1: none)
};

__host__ __device__ constexpr size_t align16(size_t x) { return (x + 15) / 16 * 16; }

// Dynamic shared memory of the fused solve: the triangular factor R [m][m] and the product of
// the Givens rotations Q^T [m+1][m+1] (TV), slices of the basis V and of Z = (I - dt A) V
// [m+1][S] each (TV), w [S] (TV), r [S]
// (FP64), partial-sum slots [slots][B] (FP64-sized: the residual's operator application uses
// them in FP64, the Arnoldi steps' in TV).
template <typename TV>
__host__ __device__ constexpr size_t fused_smem(int m, int max_rows, int max_slots, int B) {
  return align16(static_cast<size_t>(m) * m * sizeof(TV)) +
         align16(static_cast<size_t>(m + 1) * (m + 1) * sizeof(TV)) +
         2 * align16(static_cast<size_t>(m + 1) * max_rows * B * sizeof(TV)) +
         align16(static_cast<size_t>(max_rows) * B * sizeof(TV)) +
         align16(static_cast<size_t>(max_rows) * B * sizeof(double)) +
         static_cast<size_t>(max_slots) * B * sizeof(double);
}

// Grid-wide barrier for a cooperative launch (all CTAs resident).  bar[0] counts arrivals
// over the whole launch (zeroed before it): thread 0 adds one with release semantics and
// polls, with acquire semantics, until the count reaches (barriers passed) x gridDim.x --
// one atomic per CTA, no reset.  The wait is bounded (~2^31 cycles); a CTA that gives up
// sets bar[2], and every CTA then leaves this and every later barrier with false.
__device__ __forceinline__ unsigned ld_acquire_gpu(const unsigned* p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void red_release_gpu(unsigned* p, unsigned v) {
  asm volatile("red.release.gpu.global.add.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ bool grid_sync(unsigned* bar, unsigned& target, bool withhold = false) {
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    int ok = ld_acquire_gpu(bar + 2) == 0u;
    if (ok) {
      target += gridDim.x;
      if (!withhold) red_release_gpu(bar, 1u);  // withhold: the test hook's missing arrival
      const long long t0 = clock64();
      while (ld_acquire_gpu(bar) < target) {
        if (ld_acquire_gpu(bar + 2) != 0u || clock64() - t0 > (1LL << 31)) {
          atomicExch(bar + 2, 1u);
          ok = 0;
          break;
        }
      }
    }
    s_ok = ok;
  }
  __syncthreads();
  return s_ok != 0;
}

// ---------------------------------------------------------------------------------------
// One RK3 step in one cooperative launch, for plans whose apply is the split fiber kernel
// (small blocks, one applied factor per term).  Each stage applies the operator to its input
// row by row exactly as k_single_fiber_split does (same warps per row, same partial order) and
// updates the row's values at once with rk3_update; two grid barriers separate the stages.
// The stage-2 input (y1) and output (y2) are distinct vectors, so a stage never writes what
// another CTA may still be reading.  Results equal the nine-launch step bitwise.
// ---------------------------------------------------------------------------------------
template <typename T>
struct Rk3Args {
  ApplyArgs<T> a;      // the plan's apply arguments (f and y unused)
  T* f;                // the state, advanced in place
  Rk3Src<T> S;         // the stage sources
  T* k1;
  T* k2;
  T* y1;               // stage-1 output, stage-2 input
  T* y2;               // stage-2 output, stage-3 input
  T dt;
  unsigned* bar;       // grid barrier words, zeroed before the launch
};

template <typename T, int P, int MAXF, bool KAHAN, int WR>
__global__ void __launch_bounds__(32 * WR) k_rk3_fused(Rk3Args<T> r) {
  __shared__ __align__(16) T part[WR][256];
  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
  const ApplyArgs<T>& a = r.a;
  const int B = a.B;
  const FiberLane<MAXF> fl = fiber_lane<T, P, MAXF>(a, lane);
  unsigned target = 0;
  for (int stage = 1; stage <= 3; ++stage) {
    const T* x = stage == 1 ? r.f : (stage == 2 ? r.y1 : r.y2);
    T* yout = stage == 1 ? r.y1 : r.y2;
    for (int row = blockIdx.x; row < a.N; row += gridDim.x) {
      fiber_chunk<T, P, MAXF, KAHAN>(a, x, a.row_ptr[row], a.row_ptr[row + 1], fl, part[warp], warp * fl.Gf,
                                     WR * fl.Gf);
      __syncthreads();
      for (int e = threadIdx.x; e < B; e += 32 * WR) {
        T v = part[0][e];
#pragma unroll
        for (int w = 1; w < WR; ++w) v += part[w][e];
        const long long i = static_cast<long long>(row) * B + e;
        rk3_update(stage, i, v, r.dt, rk3_source(r.S, stage - 1, i), r.f, yout, r.k1, r.k2);
      }
      __syncthreads();
    }
    if (stage < 3 && !grid_sync(r.bar, target)) {
      if (threadIdx.x == 0) atomicExch(a.err, static_cast<int>(ASG_ERR_TIMEOUT));
      return;
    }
  }
}

// CTAs of `kern` (threads per CTA, no dynamic shared memory) a cooperative launch can hold on
// the current device; 0 when cooperative launches are unavailable or a query fails.
template <typename K>
long long coop_resident(K kern, int threads) {
  int dev = 0, nsm = 0, coop = 0, per_sm = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev) != cudaSuccess ||
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, threads, 0) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return coop ? static_cast<long long>(per_sm) * nsm : 0;
}

template <typename T, int P>
cudaError_t launch_rk3_fused_p(const Rk3Args<T>& r, cudaStream_t s) {
  constexpr int WR = sizeof(T) == 4 ? 4 : 2;  // the split fiber kernel's warps per row
  constexpr bool K = sizeof(T) == 4;
  const int Lf = r.a.B / P;
  auto go = [&](auto maxf) -> cudaError_t {
    constexpr int MF = decltype(maxf)::value;
    auto kern = k_rk3_fused<T, P, MF, K, WR>;
    // co-resident CTAs, queried once per instantiation (a thread-safe static); a failed query
    // gives 0, and the step then runs as separate launches
    static const long long resident = coop_resident(kern, 32 * WR);
    const int G = static_cast<int>(std::min<long long>(r.a.N, std::min<long long>(resident, 152 * 16)));
    if (G <= 0) return cudaErrorNotSupported;
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3(G);
    cfg.blockDim = dim3(32 * WR);
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeCooperative;
    at[0].val.cooperative = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kern, r);
  };
  if (Lf <= 32) return go(std::integral_constant<int, 1>{});
  if (Lf <= 64) return go(std::integral_constant<int, 2>{});
  return go(std::integral_constant<int, 4>{});
}

template <typename T>
cudaError_t launch_rk3_fused(const Rk3Args<T>& r, int P, cudaStream_t s) {
  switch (P) {
    case 1: return launch_rk3_fused_p<T, 1>(r, s);
    case 2: return launch_rk3_fused_p<T, 2>(r, s);
    case 3: return launch_rk3_fused_p<T, 3>(r, s);
    case 4: return launch_rk3_fused_p<T, 4>(r, s);
    default: return cudaErrorNotSupported;
  }
}

// Sum over the CTA of one value per thread, fixed order; the result goes to every thread.
template <typename T>
__device__ T fz_block_sum(T v) {
  __shared__ T red[kFzWarps];
  __shared__ T total;
  for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    T s = T(0);
    for (int q = 0; q < kFzWarps; ++q) s += red[q];
    total = s;
  }
  __syncthreads();
  const T r = total;
  __syncthreads();
  return r;
}

// Warp sum, fixed order (every lane gets the total).
template <typename T>
__device__ __forceinline__ T fz_warp_sum(T v) {
  for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
  return v;
}

// s_out[k] = sum over the grid's CTAs of partial[k * G + q], k < nk: warp w takes rows w,
// w + 16, ... (up to four loaded together in FP32), its lanes adding q = lane, lane + 32, ... and a
// shuffle tree adding the lanes; every CTA computes the same values in the same order.
template <typename T>
__device__ void sum_partials(const T* partial, int nk, T* s_out) {
  // rows in flight per warp: four in FP32; one in FP64, where the kernel sits at its register
  // limit and more rows in flight measured slower
  constexpr int U = sizeof(T) == 4 ? 4 : 1;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, G = gridDim.x;
  for (int k0 = warp; k0 < nk; k0 += U * kFzWarps) {  // rows k0, k0 + 16, ... together
    T acc[U];
#pragma unroll
    for (int u = 0; u < U; ++u) acc[u] = T(0);
    for (int q = lane; q < G; q += 32) {
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const int k = k0 + u * kFzWarps;
        if (k < nk) acc[u] += __ldcg(partial + static_cast<long long>(k) * G + q);
      }
    }
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int k = k0 + u * kFzWarps;
      const T v = fz_warp_sum(acc[u]);
      if (lane == 0 && k < nk) s_out[k] = v;
    }
  }
  __syncthreads();
}

__device__ __forceinline__ float fz_rsqrt(float x) { return rsqrtf(x); }
__device__ __forceinline__ double fz_rsqrt(double x) { return rsqrt(x); }

// Barrier of the Givens warps only (named barrier 1).
__device__ __forceinline__ void givens_sync() {
  asm volatile("bar.sync 1, %0;" ::"r"(32 * kFzGivensWarps) : "memory");
}

// A f over the CTA's rows into the partial-sum slots: warp items [it0, it1).  Plain sums (no
// compensation): inside the solver the FP64 outer residual corrects the rounding.
template <typename T, int P, int MAXF>
__device__ __forceinline__ void apply_items(const ApplyArgs<T>& a, const T* f, const FzItem* items, int it0, int it1,
                                            int slot0, T* slots, const FiberLane<MAXF>& fl) {
  for (int it = it0; it < it1; ++it) {
    const FzItem t = items[it];
    fiber_chunk<T, P, MAXF, false>(a, f, t.q0, t.q0 + t.len, fl, slots + (t.slot - slot0) * a.B);
  }
}
template <typename T, int P, int MAXO>
__device__ __forceinline__ void apply_items(const ApplyArgs<T>& a, const T* f, const FzItem* items, int it0, int it1,
                                            int slot0, T* slots, const SmallLane<MAXO>& sl) {
  for (int it = it0; it < it1; ++it) {
    const FzItem t = items[it];
    small_chunk<T, P, MAXO, false>(a, f, t.q0, t.q0 + t.len, sl, slots + (t.slot - slot0) * a.B);
  }
}
// ax[e] = the slots of e's row added at output e % B, for the CTA's S elements: a team of
// `team` lanes per element (a power of two up to 32, larger when the CTA has few elements --
// long rows have many slots), lane k adding slots k, k + team, ..., then a shuffle tree
// inside the team.  Fixed order; ends with a CTA barrier.
template <typename T>
__device__ __forceinline__ void slot_reduce(const T* slots, const int* row_slot, int r0, int slot0, int S, int B,
                                            int team, T* ax) {
  const int lg = __ffs(team) - 1;
  for (int base = 0; base < S * team; base += kFzThreads) {  // the same trip count in every thread
    const int t = base + threadIdx.x, e = t >> lg, k = t & (team - 1);
    T acc = T(0);
    if (e < S) {
      const int r = e / B, o = e - r * B;
      const int s0 = row_slot[r0 + r] - slot0, s1 = row_slot[r0 + r + 1] - slot0;
      for (int q = s0 + k; q < s1; q += team) acc += slots[q * B + o];
    }
    for (int off = team >> 1; off > 0; off >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, off);
    if (e < S && k == 0) ax[e] = acc;
  }
  __syncthreads();
}

// The inner GMRES cycle (w, the dot products and their sums, the orthogonalisation updates,
// the Givens rotations, R y = g and V y) runs in TV, the basis precision, and the operator
// inside it in TA: FP32 / FP32 for the solver with an FP32 inner cycle, on the FP32 pipes (an
// FP32 basis holds the Arnoldi relation to FP32 accuracy only, and the FP64 outer residual
// corrects); FP64 / FP32 for the solver that keeps the Arnoldi dot products, norms and updates
// in FP64 and runs only the operator in FP32; FP64 / FP64 for the FP64 solver.  The outer
// residual, its norm, b and x are FP64 in all three.
template <typename TV, typename TA, int P, int MAXO>
__global__ void __launch_bounds__(kFzThreads, 1) k_be_fused(const __grid_constant__ FusedArgs<TV, TA> c) {
  extern __shared__ __align__(16) unsigned char fz_smem[];
  __shared__ TV s_h[kMaxRestart], s_h2[kMaxRestart + 1];
  __shared__ TV s_g[kMaxRestart + 1], s_hc[kMaxRestart + 1], s_rc[kMaxRestart + 1], s_y[kMaxRestart];
  __shared__ TV s_hn2;
  __shared__ TV s_inv, s_hn, s_c, s_s;
  __shared__ double s_sum;
  __shared__ int s_done, s_need;
  const int G = gridDim.x, b = blockIdx.x, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int B = c.a.B, m = c.m;
  const long long ldv = c.ldv;
  const int r0 = c.blk_row[b], r1 = c.blk_row[b + 1];
  const int S = (r1 - r0) * B;  // this CTA's elements
  const long long i0 = static_cast<long long>(r0) * B;
  const int Smax = c.max_rows * B;
  unsigned char* sp = fz_smem;
  TV* s_R = reinterpret_cast<TV*>(sp);  // [m][m]: R(i, j) at i * m + j, i <= j
  sp += align16(static_cast<size_t>(m) * m * sizeof(TV));
  TV* s_Q = reinterpret_cast<TV*>(sp);  // [m+1][m+1]: Q^T = G_{j-1} ... G_0
  sp += align16(static_cast<size_t>(m + 1) * (m + 1) * sizeof(TV));
  TV* Vs = reinterpret_cast<TV*>(sp);  // [m+1][Smax]
  sp += align16(static_cast<size_t>(m + 1) * Smax * sizeof(TV));
  TV* Zs = reinterpret_cast<TV*>(sp);  // [m+1][Smax]
  sp += align16(static_cast<size_t>(m + 1) * Smax * sizeof(TV));
  TV* ws = reinterpret_cast<TV*>(sp);
  sp += align16(static_cast<size_t>(Smax) * sizeof(TV));
  double* rs = reinterpret_cast<double*>(sp);
  sp += align16(static_cast<size_t>(Smax) * sizeof(double));
  TA* slots = reinterpret_cast<TA*>(sp);
  double* slots64 = reinterpret_cast<double*>(sp);
  const int slot0 = c.blk_slot[b];
  TV* pv = reinterpret_cast<TV*>(c.partial);  // rows of TV partials
  TV* part1 = pv;
  TV* part2 = pv + static_cast<long long>(m) * G;
  TV* partg = pv + (2LL * m + 1) * G;
  double* partn = c.partial + (2LL * m + 1) * G;  // FP64 norms of b and r
  unsigned* bar = c.state->bar;
  unsigned bar_target = 0;  // arrivals expected at the next barrier (thread 0)
  int bar_count = 0;        // barriers entered (the test hook's index)
  auto gsync = [&]() { return grid_sync(bar, bar_target, b == 0 && bar_count++ == c.withhold); };
  const int it0 = c.warp_item[b * kFzWarps + warp], it1 = c.warp_item[b * kFzWarps + warp + 1];
  const TV dtv = static_cast<TV>(c.dt);
  // row routine: fiber rows for FP32, per-output rows for FP64 (the faster of the two in each
  // precision); the FP64 residual uses the same lane layout
  using Lane = typename std::conditional<sizeof(TA) == 4, FiberLane<MAXO>, SmallLane<MAXO>>::type;
  Lane sl;
  if constexpr (sizeof(TA) == 4)
    sl = fiber_lane<TA, P, MAXO>(c.a, lane);
  else
    sl = small_lane<TA, P, MAXO>(c.a, lane);
  int team = 1;  // lanes per element in the slot sums
  while (team < 32 && 2 * team * S <= kFzThreads) team <<= 1;
  TA* axs = reinterpret_cast<TA*>(rs);  // A w' for the CTA's rows (rs is free during a cycle)
  {  // ||b||
    double acc = 0.0;
    for (int e = tid; e < S; e += kFzThreads) acc = fma(c.rhs[i0 + e], c.rhs[i0 + e], acc);
    acc = fz_block_sum(acc);
    if (tid == 0) partn[b] = acc;
  }
  bool ok = gsync();
  double bnorm = 0.0;
  if (ok) {
    sum_partials(partn, 1, &s_sum);
    bnorm = sqrt(s_sum);
  }
  int outer = 0, inner = 0, converged = 0;
  double rel = 1.0;
  for (; ok; ++outer) {
    // ---- r = b - (x - dt A x) in FP64 and ||r|| ----
    apply_items<double, P, MAXO>(c.a64, c.x, c.items, it0, it1, slot0, slots64, sl);
    __syncthreads();
    slot_reduce(slots64, c.row_slot, r0, slot0, S, B, team, rs);
    {
      double acc = 0.0;
      for (int e = tid; e < S; e += kFzThreads) {
        const double rv = c.rhs[i0 + e] - (c.x[i0 + e] - c.dt * rs[e]);
        rs[e] = rv;
        acc = fma(rv, rv, acc);
      }
      acc = fz_block_sum(acc);
      if (tid == 0) partn[b] = acc;
    }
    if (!(ok = gsync())) break;
    sum_partials(partn, 1, &s_sum);
    const double rn = sqrt(s_sum);
    rel = bnorm > 0 ? rn / bnorm : rn;
    if (rn <= c.tol * bnorm || rn == 0.0) {
      converged = 1;
      break;
    }
    if (outer == c.max_outer) break;
    // inner target: a fixed relative reduction (the TV operator limits what is attainable)
    const TV target = static_cast<TV>(fmax(c.tol * bnorm, rn * c.inner_reduction));
    // ---- one GMRES(m) cycle on (I - dt A) delta = r, x += delta ----
    // Zs[k] = (I - dt A) v_k.  The operator is applied to w' (w after the first Gram-Schmidt
    // pass, published before the second barrier), and (I - dt A) v_{j+1} =
    // ((I - dt A) w' - sum_k h2_k Z_k) / ||w|| -- so no barrier only to publish v_{j+1}.
    TA* W = c.V;  // global copy of the vector the operator is applied to next
    {
      const double ib = 1.0 / rn;
      for (int e = tid; e < S; e += kFzThreads) {
        const TV v = static_cast<TV>(rs[e] * ib);
        Vs[e] = v;
        W[i0 + e] = static_cast<TA>(v);
      }
    }
    for (int q = tid; q < (m + 1) * (m + 1); q += kFzThreads) s_Q[q] = q == 0 ? TV(1) : TV(0);
    if (tid == 0) {
      for (int k = 0; k <= m; ++k) s_g[k] = TV(0);
      s_g[0] = static_cast<TV>(rn);
    }
    if (!(ok = gsync())) break;
    apply_items<TA, P, MAXO>(c.a, W, c.items, it0, it1, slot0, slots, sl);
    __syncthreads();
    slot_reduce(slots, c.row_slot, r0, slot0, S, B, team, axs);
    for (int e = tid; e < S; e += kFzThreads) {
      const TV z = fma(-dtv, static_cast<TV>(axs[e]), Vs[e]);
      Zs[e] = z;
      ws[e] = z;
    }
    __syncthreads();
    int kdone = 0;
    for (int j = 0; j < m; ++j) {
      // 1. w = Z_j (in ws): pass-1 partial dots
      for (int k = warp; k <= j; k += kFzWarps) {
        const TV* vk = Vs + k * Smax;
        TV acc = TV(0);
        for (int e = lane; e < S; e += 32) acc = fma(ws[e], vk[e], acc);
        acc = fz_warp_sum(acc);
        if (lane == 0) part1[static_cast<long long>(k) * G + b] = acc;
      }
      if (!(ok = gsync())) break;
      // 2. h; w' = w - V h (published); pass-2 partial dots and ||w'||^2
      sum_partials(part1, j + 1, s_h);
      for (int e = tid; e < S; e += kFzThreads) {
        TV acc = ws[e];
        for (int k = 0; k <= j; ++k) acc = fma(-s_h[k], Vs[k * Smax + e], acc);
        ws[e] = acc;
        W[i0 + e] = static_cast<TA>(acc);
      }
      __syncthreads();
      for (int k = warp; k <= j + 1; k += kFzWarps) {
        TV acc = TV(0);
        if (k <= j) {
          const TV* vk = Vs + k * Smax;
          for (int e = lane; e < S; e += 32) acc = fma(ws[e], vk[e], acc);
        } else {
          for (int e = lane; e < S; e += 32) acc = fma(ws[e], ws[e], acc);
        }
        acc = fz_warp_sum(acc);
        if (lane == 0) part2[static_cast<long long>(k) * G + b] = acc;
      }
      if (!(ok = gsync())) break;
      // 3. the Givens warps: h2, ||w|| and the Givens step; the other warps meanwhile apply
      //    (I - dt A) to w' (read from its global copy) -- the two do not depend on each other
      auto givens = [&]() {  // run by the Givens warps
        const int gt = tid;  // 0 .. 32 * kFzGivensWarps - 1
        // earlier rotations on the new column as one product with Q^T (groups of 8 lanes per
        // row, fixed order): FP64 latency is long here, so no serial chain over the rotations
        const int sub = lane >> 3, l8 = lane & 7;
        for (int i0w = warp * 4; i0w <= j; i0w += kFzGivensWarps * 4) {  // warp-uniform trip count
          const int i = i0w + sub;
          TV acc = TV(0);
          if (i <= j) {
            const TV* qrow = s_Q + i * (m + 1);
            for (int k = l8; k <= j; k += 8) acc = fma(qrow[k], s_hc[k], acc);
          }
          for (int off = 4; off > 0; off >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, off);
          if (l8 == 0 && i <= j) s_rc[i] = acc;
        }
        if (gt == 32 * kFzGivensWarps - 1) {  // ||w|| and 1 / ||w||, alongside
          const TV hn2 = s_hn2 > TV(0) ? s_hn2 : TV(0);
          const TV inv = hn2 > TV(0) ? fz_rsqrt(hn2) : TV(0);
          s_inv = inv;
          s_hn = hn2 * inv;
        }
        givens_sync();
        if (gt == 0) {  // the new rotation from (r_j, ||w||)
          const TV rj = s_rc[j], hn = s_hn;
          const TV den2 = fma(rj, rj, hn * hn);
          const TV rd = den2 > TV(0) ? fz_rsqrt(den2) : TV(0);
          const TV cc = den2 > TV(0) ? rj * rd : TV(1), sv = den2 > TV(0) ? hn * rd : TV(0);
          s_c = cc;
          s_s = sv;
          s_rc[j] = den2 * rd;
          const TV gj = s_g[j];
          s_g[j + 1] = -sv * gj;
          s_g[j] = cc * gj;
          s_done = (fabs(sv * gj) <= target || hn == TV(0) || j + 1 == m) ? 1 : 0;
        }
        givens_sync();
        const TV cc = s_c, sv = s_s;  // R(:, j), and rows j, j+1 of Q^T rotated
        for (int i = gt; i <= j; i += 32 * kFzGivensWarps) s_R[i * m + j] = s_rc[i];
        for (int k = gt; k <= j + 1; k += 32 * kFzGivensWarps) {
          const TV old = k <= j ? s_Q[j * (m + 1) + k] : TV(0);
          const TV e = k == j + 1 ? TV(1) : TV(0);
          s_Q[j * (m + 1) + k] = fma(cc, old, sv * e);
          s_Q[(j + 1) * (m + 1) + k] = fma(-sv, old, cc * e);
        }
      };
      sum_partials(part2, j + 2, s_h2);
      for (int k = tid; k <= j; k += kFzThreads) s_hc[k] = s_h[k] + s_h2[k];
      if (warp == 0) {  // ||w||^2 = ||w'||^2 - ||h2||^2 unless that cancels badly
        TV h2sq = TV(0);
        for (int k = lane; k <= j; k += 32) h2sq = fma(s_h2[k], s_h2[k], h2sq);
        h2sq = fz_warp_sum(h2sq);
        const TV nw2 = s_h2[j + 1];
        if (lane == 0) {
          s_hn2 = nw2 - h2sq;
          s_need = h2sq <= TV(1e-2) * nw2 ? 0 : 1;
        }
      }
      __syncthreads();
      if (warp < kFzGivensWarps) {
        if (!s_need) givens();
      } else {
        apply_items<TA, P, MAXO>(c.a, W, c.items, it0, it1, slot0, slots, sl);
      }
      __syncthreads();
      if (s_need) {  // the same decision in every CTA: explicit ||w' - V h2||^2, then the Givens step
        TV acc = TV(0);
        for (int e = tid; e < S; e += kFzThreads) {
          TV v = ws[e];
          for (int k = 0; k <= j; ++k) v = fma(-s_h2[k], Vs[k * Smax + e], v);
          acc = fma(v, v, acc);
        }
        acc = fz_block_sum(acc);
        if (tid == 0) partg[b] = acc;
        if (!(ok = gsync())) break;
        sum_partials(partg, 1, &s_hn2);
        if (warp < kFzGivensWarps) givens();
        __syncthreads();
      }
      kdone = j + 1;
      if (s_done) break;  // the same decision in every CTA
      slot_reduce(slots, c.row_slot, r0, slot0, S, B, team, axs);
      {
        const TV inv = s_inv;
        TV* Vn = Vs + (j + 1) * Smax;
        TV* Zn = Zs + (j + 1) * Smax;
        for (int e = tid; e < S; e += kFzThreads) {
          const TV wp = ws[e];
          TV v = wp, z = fma(-dtv, static_cast<TV>(axs[e]), wp);
          for (int k = 0; k <= j; ++k) {
            v = fma(-s_h2[k], Vs[k * Smax + e], v);
            z = fma(-s_h2[k], Zs[k * Smax + e], z);
          }
          Vn[e] = v * inv;
          z *= inv;
          Zn[e] = z;
          ws[e] = z;
        }
      }
      __syncthreads();
    }
    if (!ok) break;
    // ---- y = R \ g by warp 0 (column sweep), x += V y over the CTA's slice ----
    __syncthreads();
    if (warp == 0) {
      for (int q = lane; q < kdone; q += 32) {
        s_y[q] = s_g[q];
        s_hc[q] = TV(1) / s_R[q * m + q];
      }
      __syncwarp();
      for (int i = kdone - 1; i >= 0; --i) {
        const TV yi = s_y[i] * s_hc[i];
        __syncwarp();
        for (int q = lane; q < i; q += 32) s_y[q] = fma(-s_R[q * m + i], yi, s_y[q]);
        if (lane == 0) s_y[i] = yi;
        __syncwarp();
      }
    }
    __syncthreads();
    for (int e = tid; e < S; e += kFzThreads) {
      TV d = TV(0);
      for (int k = 0; k < kdone; ++k) d = fma(s_y[k], Vs[k * Smax + e], d);
      c.x[i0 + e] += static_cast<double>(d);
    }
    inner += kdone;
    if (!(ok = gsync())) break;  // x complete before the next residual
  }
  if (b == 0 && tid == 0) {
    c.state->outer = outer;
    c.state->inner = inner;
    c.state->converged = converged;
    c.state->rel = rel;
    c.state->done = 1;
  }
}

inline int grid_for(long long n) {
  const long long g = (n + 255) / 256;
  return static_cast<int>(g < 152LL * 16 ? (g > 0 ? g : 1) : 152LL * 16);
}

}  // namespace
}  // namespace asg

// =======================================================================================
// Host orchestration
// =======================================================================================
using asg::fail;

namespace {

size_t align256(size_t x) { return (x + 255) / 256 * 256; }

struct GmresLayout {
  size_t v, vf, w, r, ax64, axmv, h, y, partial, hcol, hh, cs, sn, g, state, total;
};

// Leading dimension of the Krylov basis: every basis vector starts on a 32-byte boundary (the
// operator application reads it with 16-byte loads, in either precision).
long long basis_ld(long long n) { return (n + 3) / 4 * 4; }

// mode: ASG_GMRES_FP64, ASG_GMRES_FP32_INNER or ASG_GMRES_FP32_MATVEC (asgkron.h)
GmresLayout gmres_layout(long long n, int m, int mode) {
  const bool basis32 = mode == ASG_GMRES_FP32_INNER, apply32 = mode != ASG_GMRES_FP64;
  GmresLayout L{};
  size_t off = 0;
  auto take = [&](size_t bytes) {
    const size_t o = off;
    off += align256(bytes);
    return o;
  };
  L.v = take(static_cast<size_t>(m + 1) * basis_ld(n) * (basis32 ? sizeof(float) : sizeof(double)));
  L.vf = take(apply32 && !basis32 ? basis_ld(n) * sizeof(float) : 0);
  L.w = take(n * sizeof(double));
  L.r = take(n * sizeof(double));
  L.ax64 = take(n * sizeof(double));
  L.axmv = take(n * (apply32 ? sizeof(float) : sizeof(double)));
  L.h = take((m + 1) * sizeof(double));
  L.y = take((m + 1) * sizeof(double));
  L.partial = take(static_cast<size_t>(2 * m + 2) * asg::kRedBlocks * sizeof(double));
  L.hcol = take((m + 1) * sizeof(double));
  L.hh = take(static_cast<size_t>(m + 1) * m * sizeof(double));
  L.cs = take(m * sizeof(double));
  L.sn = take(m * sizeof(double));
  L.g = take((m + 1) * sizeof(double));
  L.state = take(sizeof(asg::GmresState));
  L.total = off;
  return L;
}

double host_norm(const double* d_partial, int nb, cudaStream_t s, asg_status* st) {
  std::vector<double> p(nb);
  cudaError_t e = cudaMemcpyAsync(p.data(), d_partial, p.size() * sizeof(double), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) {
    *st = asg::cuda_fail(e, "norm readback");
    return 0.0;
  }
  double acc = 0.0;
  for (double v : p) acc += v;
  return std::sqrt(acc);
}

// Schedule of the fused solve for a small-block plan, built once per plan: at most G0 CTAs (G0:
// the SM count, the row count and one per 64 work entries, whichever is least), contiguous
// row ranges minimising the largest cost in warp rounds; each CTA's rows are cut into chunks
// of whole rounds, at most max(2, U_b / (2 Wa)) rounds each (U_b: the CTA's rounds, Wa: its
// warps that apply the operator -- all but the Givens warps), and the chunks go to those
// warps longest first, each to the least-loaded one.
asg_status fused_schedule(asg_plan* p, int k) {
  if (p->fz_G[k] > 0) return ASG_OK;
  int dev = 0, nsm = 0;
  ASG_CUDA(cudaGetDevice(&dev));
  ASG_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  const int N = p->N, B = p->B, W = asg::kFzWarps;
  const std::vector<long long>& rp = p->row_ptr;
  const long long E = rp[N];
  const int G0 = static_cast<int>(std::max<long long>(
      1, std::min<long long>({static_cast<long long>(nsm), static_cast<long long>(N), (E + 63) / 64})));
  // A warp retires `unit` entries per round -- FP32 (fiber rows): one per lane group of
  // deg^(d-1) lanes; FP64 (per-output rows): two per lane group of L >= deg^d lanes -- so work
  // is counted in rounds.  Contiguous row ranges with the smallest largest cost (a row costs
  // its rounds plus one for the vector work): bisection on the cap, greedy fill.
  long long unit = 1;
  if (k == 1) {
    const int fibers = B / p->P;
    unit = fibers <= 32 ? 32 / fibers : 1;
  } else {
    int lanes = 1;
    while (lanes < B && lanes < 32) lanes <<= 1;
    unit = 2 * (32 / lanes);
  }
  auto rounds = [&](long long len) { return (len + unit - 1) / unit; };
  std::vector<double> cost(N);
  double lo = 0.0, hi = 0.0;
  for (int r = 0; r < N; ++r) {
    cost[r] = static_cast<double>(rounds(rp[r + 1] - rp[r])) + 1.0;
    lo = std::max(lo, cost[r]);
    hi += cost[r];
  }
  lo = std::max(lo, hi / G0);
  auto fill = [&](double cap, std::vector<int>* starts) {
    int parts = 1;
    double acc = 0.0;
    if (starts) starts->assign(1, 0);
    for (int r = 0; r < N; ++r) {
      if (acc > 0.0 && acc + cost[r] > cap) {
        ++parts;
        acc = 0.0;
        if (starts) starts->push_back(r);
      }
      acc += cost[r];
    }
    return parts;
  };
  for (int it = 0; it < 60 && hi - lo > 0.5; ++it) {
    const double mid = 0.5 * (lo + hi);
    if (fill(mid, nullptr) <= G0)
      hi = mid;
    else
      lo = mid;
  }
  std::vector<int> blk_row;
  fill(hi, &blk_row);
  const int G = static_cast<int>(blk_row.size());
  blk_row.push_back(N);
  std::vector<int> blk_slot(G + 1, 0), row_slot(N + 1, 0), warp_item(static_cast<size_t>(G) * W + 1, 0);
  std::vector<asg::FzItem> items;
  int slot = 0, max_rows = 0, max_slots = 0;
  for (int b = 0; b < G; ++b) {
    const int r0 = blk_row[b], r1 = blk_row[b + 1];
    long long Ub = 0;  // the CTA's rounds
    for (int r = r0; r < r1; ++r) Ub += rounds(rp[r + 1] - rp[r]);
    const long long Wa = W - asg::kFzGivensWarps;  // warps that apply the operator
    const long long ch = std::max<long long>(2, (Ub + 2 * Wa - 1) / (2 * Wa));  // rounds per chunk
    blk_slot[b] = slot;
    std::vector<asg::FzItem> bi;
    for (int r = r0; r < r1; ++r) {
      row_slot[r] = slot;
      const long long er = rp[r + 1] - rp[r], ur = rounds(er);
      const long long nch = (ur + ch - 1) / ch;
      long long q = rp[r], left = er;
      for (long long k = 0; k < nch; ++k) {  // whole rounds per chunk, the last one takes the rest
        const long long uk = ur / nch + (k < ur % nch ? 1 : 0);
        const long long len = std::min(left, uk * unit);
        bi.push_back(asg::FzItem{q, static_cast<int>(len), slot++});
        q += len;
        left -= len;
      }
    }
    max_rows = std::max(max_rows, r1 - r0);
    max_slots = std::max(max_slots, slot - blk_slot[b]);
    // longest first onto the least-loaded warp (ties: lowest warp)
    std::vector<int> order(bi.size());
    for (size_t k = 0; k < order.size(); ++k) order[k] = static_cast<int>(k);
    std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return bi[x].len > bi[y].len; });
    std::vector<long long> load(W, 0);
    std::vector<std::vector<asg::FzItem>> per(W);
    const int w0 = asg::kFzGivensWarps;  // warps 0 .. w0-1 run the Givens step instead
    for (int k : order) {
      const int w = static_cast<int>(std::min_element(load.begin() + w0, load.end()) - load.begin());
      load[w] += rounds(bi[k].len) + 1;
      per[w].push_back(bi[k]);
    }
    for (int w = 0; w < W; ++w) {
      warp_item[static_cast<size_t>(b) * W + w] = static_cast<int>(items.size());
      items.insert(items.end(), per[w].begin(), per[w].end());
    }
  }
  blk_slot[G] = slot;
  row_slot[N] = slot;
  warp_item[static_cast<size_t>(G) * W] = static_cast<int>(items.size());
  std::vector<int> ints;
  ints.insert(ints.end(), blk_row.begin(), blk_row.end());
  ints.insert(ints.end(), blk_slot.begin(), blk_slot.end());
  ints.insert(ints.end(), row_slot.begin(), row_slot.end());
  ints.insert(ints.end(), warp_item.begin(), warp_item.end());
  ASG_CUDA(cudaMalloc(reinterpret_cast<void**>(&p->d_fz_int[k]), ints.size() * sizeof(int)));
  ASG_CUDA(cudaMemcpy(p->d_fz_int[k], ints.data(), ints.size() * sizeof(int), cudaMemcpyHostToDevice));
  if (!items.empty()) {
    ASG_CUDA(cudaMalloc(reinterpret_cast<void**>(&p->d_fz_items[k]), items.size() * sizeof(asg::FzItem)));
    ASG_CUDA(cudaMemcpy(p->d_fz_items[k], items.data(), items.size() * sizeof(asg::FzItem), cudaMemcpyHostToDevice));
  }
  p->fz_max_rows[k] = max_rows;
  p->fz_max_slots[k] = max_slots;
  p->fz_G[k] = G;
  return ASG_OK;
}

// The fused solve (one cooperative launch) for plans on the small-block single-mode kernel
// with deg 2..4 whose per-CTA slices fit in shared memory.
template <typename TV, typename TA, int P, int MAXO>
cudaError_t launch_fused(const asg::FusedArgs<TV, TA>& c, int G, size_t smem, cudaStream_t s) {
  auto kern = asg::k_be_fused<TV, TA, P, MAXO>;
  // the shared-memory limit, co-residency and cooperative-launch support, queried once per
  // instantiation and shared-memory size
  static size_t checked_smem = 0;
  static long long resident = 0;
  cudaError_t e = cudaSuccess;
  if (smem != checked_smem) {
    if ((e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem))) != cudaSuccess)
      return e;
    int dev = 0, nsm = 0, coop = 0, per_sm = 0;
    if ((e = cudaGetDevice(&dev)) != cudaSuccess) return e;
    if ((e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return e;
    if ((e = cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev)) != cudaSuccess) return e;
    if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, asg::kFzThreads, smem)) != cudaSuccess) return e;
    resident = coop ? static_cast<long long>(per_sm) * nsm : 0;
    checked_smem = smem;
  }
  if (resident < G) return cudaErrorNotSupported;
  void* args[] = {const_cast<asg::FusedArgs<TV, TA>*>(&c)};
  return cudaLaunchCooperativeKernel(reinterpret_cast<const void*>(kern), dim3(G), dim3(asg::kFzThreads), args, smem, s);
}

template <typename TV, typename TA, int P>
cudaError_t launch_fused_p(const asg::FusedArgs<TV, TA>& c, int G, size_t smem, cudaStream_t s) {
  // outputs (FP64 operator, per-output rows) or fibers (FP32 operator) per lane
  const int B = c.a.B, Lf = B / P;
  if constexpr (sizeof(TA) == 4) {
    if (Lf <= 32) return launch_fused<TV, TA, P, 1>(c, G, smem, s);
    if (Lf <= 64) return launch_fused<TV, TA, P, 2>(c, G, smem, s);
    return launch_fused<TV, TA, P, 4>(c, G, smem, s);
  } else {
    if (B <= 32) return launch_fused<TV, TA, P, 1>(c, G, smem, s);
    if (B <= 64) return launch_fused<TV, TA, P, 2>(c, G, smem, s);
    if (B <= 128) return launch_fused<TV, TA, P, 4>(c, G, smem, s);
    return launch_fused<TV, TA, P, 8>(c, G, smem, s);
  }
}

constexpr size_t kFusedSmemLimit = 200 * 1024;
int g_withhold = -1;  // asg_debug_withhold_arrival

// The whole solve as one launch when the plan qualifies (*used = true; one synchronisation
// to read the result); *used = false otherwise (the caller runs the host-driven solve).
template <typename TV, typename TA>
asg_status be_solve_fused(asg_plan* plan, long long n, double dt, const double* b, double* x, const asg_gmres_opts* o,
                          asg_gmres_info* info, unsigned char* base, const GmresLayout& L, cudaStream_t s, bool* used) {
  *used = false;
  asg::FusedArgs<TV, TA> c{};
  if (!asg::small_plan_args<TA>(plan, &c.a) || !asg::small_plan_args<double>(plan, &c.a64) || c.a.B > 256) return ASG_OK;
  if ((reinterpret_cast<uintptr_t>(b) | reinterpret_cast<uintptr_t>(x)) & 15) return ASG_OK;  // vector loads of x
  const int P = c.a.D >= 2 ? c.a.stride[c.a.D - 2] : c.a.B;
  if (P < 2 || P > 4) return ASG_OK;
  const int m = o->restart;
  const int k = sizeof(TA) == 4 ? 1 : 0;  // the work schedule follows the operator's lane layout
  asg_status st = fused_schedule(plan, k);
  if (st) return st;
  const int G = plan->fz_G[k];
  const size_t smem = asg::fused_smem<TV>(m, plan->fz_max_rows[k], plan->fz_max_slots[k], c.a.B);
  if (smem > kFusedSmemLimit) return ASG_OK;
  c.n = n;
  c.ldv = basis_ld(n);
  c.dt = dt;
  c.tol = o->tol;
  c.inner_reduction = o->inner_reduction;
  c.m = m;
  c.max_outer = o->max_outer;
  c.V = reinterpret_cast<TA*>(base + L.v);
  c.partial = reinterpret_cast<double*>(base + L.partial);
  c.rhs = b;
  c.x = x;
  c.state = reinterpret_cast<asg::GmresState*>(base + L.state);
  const int* fz = plan->d_fz_int[k];
  c.blk_row = fz;
  c.blk_slot = fz + (G + 1);
  c.row_slot = fz + 2 * (G + 1);
  c.warp_item = fz + 2 * (G + 1) + (plan->N + 1);
  c.items = plan->d_fz_items[k];
  c.max_rows = plan->fz_max_rows[k];
  c.max_slots = plan->fz_max_slots[k];
  c.withhold = g_withhold;
  g_withhold = -1;
  ASG_CUDA(cudaMemsetAsync(c.state, 0, sizeof(asg::GmresState), s));
  cudaError_t e = P == 2 ? launch_fused_p<TV, TA, 2>(c, G, smem, s)
                  : P == 3 ? launch_fused_p<TV, TA, 3>(c, G, smem, s)
                           : launch_fused_p<TV, TA, 4>(c, G, smem, s);
  if (e == cudaErrorNotSupported) {
    cudaGetLastError();
    return ASG_OK;  // the CTAs cannot all be resident: the caller runs the host-driven solve
  }
  if (e != cudaSuccess) return asg::cuda_fail(e, "fused backward-Euler solve");
  *used = true;
  asg::GmresState hs{};
  ASG_CUDA(cudaMemcpyAsync(&hs, c.state, sizeof(hs), cudaMemcpyDeviceToHost, s));
  ASG_CUDA(cudaStreamSynchronize(s));
  if (hs.bar[2]) return fail(ASG_ERR_TIMEOUT, "fused backward-Euler solve: grid barrier wait gave up (%d CTAs)", G);
  if (info) {
    asg_gmres_info inf{};
    inf.outer_iters = hs.outer;
    inf.inner_iters = hs.inner;
    inf.converged = hs.converged;
    inf.rel_residual = hs.rel;
    *info = inf;
  }
  return ASG_OK;
}

// One GMRES(m) cycle on (I - dt A) delta = r0 (r0 FP64, beta = ||r0||), adding delta to x64
// in FP64.  TV is the basis precision, TA the operator application's (a TV basis vector is
// rounded to TA first when they differ).  Stops early when the residual estimate drops to
// rtol_abs.  *iters = Arnoldi steps taken, *resid = final residual estimate.
template <typename TV, typename TA>
asg_status gmres_cycle(asg_plan* plan, long long n, double dt, const double* r0, double beta, double* x64, int m,
                       double rtol_abs, unsigned char* base, const GmresLayout& L, cudaStream_t s, int* iters,
                       double* resid) {
  TV* V = reinterpret_cast<TV*>(base + L.v);
  const long long ldv = basis_ld(n);
  double* w = reinterpret_cast<double*>(base + L.w);
  TA* axmv = reinterpret_cast<TA*>(base + L.axmv);
  TA* vf = reinterpret_cast<TA*>(base + L.vf);  // V_j rounded to TA (TA != TV only)
  double* h_dev = reinterpret_cast<double*>(base + L.h);
  double* y_dev = reinterpret_cast<double*>(base + L.y);
  double* partial = reinterpret_cast<double*>(base + L.partial);
  const int gr = asg::grid_for(n);
  *iters = 0;
  const int nb = asg::red_blocks(n);
  *resid = beta;
  if (beta <= rtol_abs || beta == 0.0) return ASG_OK;
  asg::k_store_basis<TV><<<gr, 256, 0, s>>>(n, 1.0 / beta, r0, V);
  double* hcol = reinterpret_cast<double*>(base + L.hcol);
  double* H = reinterpret_cast<double*>(base + L.hh);
  double* cs = reinterpret_cast<double*>(base + L.cs);
  double* sn = reinterpret_cast<double*>(base + L.sn);
  double* g = reinterpret_cast<double*>(base + L.g);
  asg::GmresState* state = reinterpret_cast<asg::GmresState*>(base + L.state);
  // g = (beta, 0, ...), state cleared: the Arnoldi steps below run without host round trips;
  // the host looks at the state every kChunk steps (steps after the stop are no-ops, except
  // the operator application, which is why the host checks at all)
  std::vector<double> g0(m + 1, 0.0);
  g0[0] = beta;
  ASG_CUDA(cudaMemcpyAsync(g, g0.data(), (m + 1) * sizeof(double), cudaMemcpyHostToDevice, s));
  ASG_CUDA(cudaMemsetAsync(state, 0, sizeof(asg::GmresState), s));
  constexpr int kChunk = 4;
  asg::GmresState hs{};
  for (int j0 = 0; j0 < m; j0 += kChunk) {
    for (int j = j0; j < std::min(m, j0 + kChunk); ++j) {
      // w = V_j - dt * A V_j
      const TA* vin = reinterpret_cast<const TA*>(V + j * ldv);
      if (sizeof(TA) != sizeof(TV)) {
        asg::k_round_g<TV, TA><<<gr, 256, 0, s>>>(n, V + j * ldv, vf, state);
        vin = vf;
      }
      asg_status ast = sizeof(TA) == 4 ? asg_apply_f32(plan, reinterpret_cast<const float*>(vin),
                                                       reinterpret_cast<float*>(axmv), s)
                                       : asg_apply_f64(plan, reinterpret_cast<const double*>(vin),
                                                       reinterpret_cast<double*>(axmv), s);
      if (ast) return ast;
      asg::k_shift_g<TV, TA><<<gr, 256, 0, s>>>(n, dt, V + j * ldv, axmv, w, state);
      for (int pass = 0; pass < 2; ++pass) {  // classical Gram-Schmidt, reorthogonalised (FP64)
        asg::k_dots_g<TV><<<dim3(nb, j + 1), asg::kRedThreads, 0, s>>>(n, w, V, ldv, partial, state);
        asg::k_dots_final_g<<<j + 1, 32, 0, s>>>(j + 1, nb, partial, h_dev, hcol, pass, state);
        asg::k_orth_update_g<TV><<<gr, 256, 0, s>>>(n, j + 1, h_dev, V, ldv, w, state);
      }
      asg::k_norm2_g<<<nb, asg::kRedThreads, 0, s>>>(n, w, partial, state);
      asg::k_givens<<<1, 32, 0, s>>>(j, m, rtol_abs, nb, partial, hcol, H, cs, sn, g, state);
      asg::k_store_basis_g<TV><<<gr, 256, 0, s>>>(n, w, V + (j + 1) * ldv, state);
    }
    ASG_CUDA(cudaMemcpyAsync(&hs, state, sizeof(hs), cudaMemcpyDeviceToHost, s));
    ASG_CUDA(cudaStreamSynchronize(s));
    if (hs.done) break;
  }
  // back substitution H y = g and x += V y (FP64 update), on the device
  asg::k_backsolve<<<1, 256, 0, s>>>(m, H, g, y_dev, state);
  asg::k_sol_update_g<TV><<<gr, 256, 0, s>>>(n, y_dev, V, ldv, x64, state);
  *iters = hs.kdone;
  *resid = hs.resid;
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return asg::cuda_fail(e, "gmres kernels");
  return ASG_OK;
}

template <typename TV, typename TA>
asg_status be_solve(asg_plan* p, double dt, const double* b, double* x, const asg_gmres_opts* o, asg_gmres_info* info,
                    void* work, size_t work_bytes, void* stream) {
  asg_plan_stats ps{};
  asg_plan_stats_get(p, &ps);
  const long long n = ps.dof;
  const int m = o->restart;
  const GmresLayout L = gmres_layout(n, m, o->mixed);
  if (work_bytes < L.total) return fail(ASG_ERR_CAPACITY, "be_solve: workspace needs %zu bytes", L.total);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  unsigned char* base = static_cast<unsigned char*>(work);
  double* r = reinterpret_cast<double*>(base + L.r);
  double* ax64 = reinterpret_cast<double*>(base + L.ax64);
  double* partial = reinterpret_cast<double*>(base + L.partial);
  const int gr = asg::grid_for(n);
  asg_status st = ASG_OK;
  bool used = false;
  if ((st = be_solve_fused<TV, TA>(p, n, dt, b, x, o, info, base, L, s, &used)) || used) return st;
  const int nb = asg::red_blocks(n);
  asg::k_norm2<<<nb, asg::kRedThreads, 0, s>>>(n, b, partial);
  const double bnorm = host_norm(partial, nb, s, &st);
  if (st) return st;
  asg_gmres_info inf{};
  inf.rel_residual = 1.0;
  for (int outer = 0; outer <= o->max_outer; ++outer) {
    // FP64 outer residual r = b - (I - dt A) x
    if ((st = asg_apply_f64(p, x, ax64, s))) return st;
    asg::k_residual<<<gr, 256, 0, s>>>(n, dt, b, x, ax64, r);
    asg::k_norm2<<<nb, asg::kRedThreads, 0, s>>>(n, r, partial);
    const double rn = host_norm(partial, nb, s, &st);
    if (st) return st;
    inf.rel_residual = bnorm > 0 ? rn / bnorm : rn;
    inf.outer_iters = outer;
    if (rn <= o->tol * bnorm || rn == 0.0) {
      inf.converged = 1;
      break;
    }
    if (outer == o->max_outer) break;
    // inner target: a fixed relative reduction (FP32 operator: ~1e-5 is attainable)
    const double target = std::max(o->tol * bnorm, rn * o->inner_reduction);
    int it = 0;
    double est = 0.0;
    if ((st = gmres_cycle<TV, TA>(p, n, dt, r, rn, x, m, target, base, L, s, &it, &est))) return st;
    inf.inner_iters += it;
  }
  if (info) *info = inf;
  return ASG_OK;
}

template <typename T>
asg_status rk3(asg_plan* p, T* f, double dt, const asg::Rk3Src<T>& S, T* work, size_t work_bytes, void* stream) {
  if (!p || !f || !work) return fail(ASG_ERR_INVALID, "rk3_step: NULL argument");
  asg_plan_stats st{};
  asg_plan_stats_get(p, &st);
  const long long n = st.dof;
  // four vectors, each starting on a 16-byte boundary (the operator application needs it)
  const long long per = 16 / static_cast<long long>(sizeof(T));
  const long long np = (n + per - 1) / per * per;
  if (work_bytes < static_cast<size_t>(4 * np) * sizeof(T))
    return fail(ASG_ERR_CAPACITY, "rk3_step: workspace needs %lld bytes", 4 * np * (long long)sizeof(T));
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  T* k1 = work;
  T* k2 = work + np;
  T* k3 = work + 2 * np;
  T* y = work + 3 * np;
  auto apply = [&](const T* in, T* out) {
    return sizeof(T) == 8 ? asg_apply_f64(p, reinterpret_cast<const double*>(in), reinterpret_cast<double*>(out), s)
                          : asg_apply_f32(p, reinterpret_cast<const float*>(in), reinterpret_cast<float*>(out), s);
  };
  const int gr = asg::grid_for(n);
  // plans applied by the split fiber kernel: the whole step in one cooperative launch
  int kind = -1;
  asg_plan_kernel_for(p, sizeof(T) == 4 ? 1 : 0, &kind);
  asg::Rk3Args<T> r{};
  if (kind == asg::KK_SINGLE_SMALL && p->P <= 4 && p->d_bar && asg::small_plan_args<T>(p, &r.a)) {
    r.f = f;
    r.S = S;
    r.k1 = k1;
    r.k2 = k2;
    r.y1 = k3;
    r.y2 = y;
    r.dt = static_cast<T>(dt);
    r.bar = p->d_bar;
    cudaError_t e = cudaMemsetAsync(p->d_bar, 0, 4 * sizeof(unsigned), s);
    if (e != cudaSuccess) return asg::cuda_fail(e, "rk3 barrier reset");
    e = asg::launch_rk3_fused<T>(r, p->P, s);
    if (e == cudaSuccess) return ASG_OK;
    if (e != cudaErrorNotSupported) return asg::cuda_fail(e, "fused rk3 launch");
  }
  asg_status a;
  if ((a = apply(f, k1))) return a;
  asg::k_rk3_stage<T><<<gr, 256, 0, s>>>(1, n, static_cast<T>(dt), f, y, k1, k2, k3, S);
  if ((a = apply(y, k2))) return a;
  asg::k_rk3_stage<T><<<gr, 256, 0, s>>>(2, n, static_cast<T>(dt), f, y, k1, k2, k3, S);
  if ((a = apply(y, k3))) return a;
  asg::k_rk3_stage<T><<<gr, 256, 0, s>>>(3, n, static_cast<T>(dt), f, y, k1, k2, k3, S);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return asg::cuda_fail(e, "rk3 stage launch");
  return ASG_OK;
}

}  // namespace

extern "C" {

asg_status asg_rk3_step_f64(asg_plan* plan, double* d_f, double dt, const double* const* d_src, double* d_work,
                            size_t work_bytes, void* stream) {
  ASG_NOT_SLICE(plan, "rk3_step");
  asg::Rk3Src<double> S{};
  for (int k = 0; k < 3; ++k) S.src[k] = d_src ? d_src[k] : nullptr;
  return rk3<double>(plan, d_f, dt, S, d_work, work_bytes, stream);
}
asg_status asg_rk3_step_f32(asg_plan* plan, float* d_f, double dt, const float* const* d_src, float* d_work,
                            size_t work_bytes, void* stream) {
  ASG_NOT_SLICE(plan, "rk3_step");
  asg::Rk3Src<float> S{};
  for (int k = 0; k < 3; ++k) S.src[k] = d_src ? d_src[k] : nullptr;
  return rk3<float>(plan, d_f, dt, S, d_work, work_bytes, stream);
}

asg_status asg_rk3_step_sources_f64(asg_plan* plan, double* d_f, double dt, int ns, const double* d_coef,
                                    const double* const* d_vecs, double* d_work, size_t work_bytes, void* stream) {
  ASG_NOT_SLICE(plan, "rk3_step_sources");
  if (ns < 0 || (ns > 0 && (!d_coef || !d_vecs))) return fail(ASG_ERR_INVALID, "rk3_step_sources: bad sources");
  asg::Rk3Src<double> S{};
  S.ns = ns;
  S.coef = d_coef;
  S.vecs = d_vecs;
  return rk3<double>(plan, d_f, dt, S, d_work, work_bytes, stream);
}
asg_status asg_rk3_step_sources_f32(asg_plan* plan, float* d_f, double dt, int ns, const double* d_coef,
                                    const double* const* d_vecs, float* d_work, size_t work_bytes, void* stream) {
  ASG_NOT_SLICE(plan, "rk3_step_sources");
  if (ns < 0 || (ns > 0 && (!d_coef || !d_vecs))) return fail(ASG_ERR_INVALID, "rk3_step_sources: bad sources");
  asg::Rk3Src<float> S{};
  S.ns = ns;
  S.coef = d_coef;
  S.vecs = d_vecs;
  return rk3<float>(plan, d_f, dt, S, d_work, work_bytes, stream);
}

asg_status asg_lincomb_f64(long long n, int ns, const double* d_coef, const double* const* d_vecs, double* d_out,
                           void* stream) {
  if (n < 0 || ns < 0 || (ns > 0 && (!d_coef || !d_vecs)) || !d_out) return fail(ASG_ERR_INVALID, "lincomb: bad argument");
  asg::k_lincomb<double><<<asg::grid_for(n), 256, 0, static_cast<cudaStream_t>(stream)>>>(n, ns, d_coef, d_vecs, d_out);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? ASG_OK : asg::cuda_fail(e, "lincomb launch");
}

asg_status asg_be_workspace(const asg_plan* plan, const asg_gmres_opts* opts, size_t* bytes) {
  if (!plan || !opts || !bytes) return fail(ASG_ERR_INVALID, "be_workspace: NULL argument");
  ASG_NOT_SLICE(plan, "be_workspace");
  if (opts->restart < 1 || opts->restart > asg::kMaxRestart) return fail(ASG_ERR_INVALID, "be_workspace: restart=%d", opts->restart);
  asg_plan_stats ps{};
  asg_plan_stats_get(plan, &ps);
  if (opts->mixed < ASG_GMRES_FP64 || opts->mixed > ASG_GMRES_FP32_MATVEC)
    return fail(ASG_ERR_INVALID, "be_workspace: mixed=%d", opts->mixed);
  *bytes = gmres_layout(ps.dof, opts->restart, opts->mixed).total;
  return ASG_OK;
}

asg_status asg_be_solve(asg_plan* plan, double dt, const double* d_b, double* d_x, const asg_gmres_opts* opts,
                        asg_gmres_info* info, void* d_work, size_t work_bytes, void* stream) {
  if (!plan || !d_b || !d_x || !opts || !d_work) return fail(ASG_ERR_INVALID, "be_solve: NULL argument");
  ASG_NOT_SLICE(plan, "be_solve");
  if (opts->restart < 1 || opts->restart > asg::kMaxRestart || opts->max_outer < 0 || !(opts->tol > 0) ||
      !(opts->inner_reduction > 0 && opts->inner_reduction < 1) || opts->mixed < ASG_GMRES_FP64 ||
      opts->mixed > ASG_GMRES_FP32_MATVEC)
    return fail(ASG_ERR_INVALID, "be_solve: bad options");
  switch (opts->mixed) {
    case ASG_GMRES_FP32_INNER:
      return be_solve<float, float>(plan, dt, d_b, d_x, opts, info, d_work, work_bytes, stream);
    case ASG_GMRES_FP32_MATVEC:
      return be_solve<double, float>(plan, dt, d_b, d_x, opts, info, d_work, work_bytes, stream);
    default:
      return be_solve<double, double>(plan, dt, d_b, d_x, opts, info, d_work, work_bytes, stream);
  }
}

asg_status asg_debug_withhold_arrival(int barrier) {
  if (barrier < -1) return fail(ASG_ERR_INVALID, "debug_withhold_arrival: barrier=%d", barrier);
  g_withhold = barrier;
  return ASG_OK;
}

}  // extern "C"
