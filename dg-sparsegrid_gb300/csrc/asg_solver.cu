// Time steppers built on the operator application (time_advance.m):
//   asg_rk3_step_*   RungeKutta3 (time_advance.m:151-204) with fused stage updates
//   asg_be_solve_*   backward Euler (time_advance.m:267-349): the reference assembles A and
//                    solves (I - dt A) f1 = b directly; here the system is solved matrix-free
//                    by restarted GMRES inside iterative refinement.  Mixed mode: FP32
//                    operator application inside GMRES, FP64 for the outer residual, the
//                    solution update and every Arnoldi dot product and norm.
// All reductions are two-pass and fixed-order, so results are bitwise reproducible.
#include <algorithm>
#include <cmath>
#include <vector>

#include "asg_internal.h"

namespace asg {
namespace {

constexpr int kRedBlocks = 304;  // partial sums per reduction (2 per SM)
constexpr int kRedThreads = 256;

// ---------------------------------------------------------------------------------------
// RK3 stage updates (time_advance.m:177-204):
//   stage 1: k1 = A f + s1;             y = f + dt/2 k1
//   stage 2: k2 = A y + s2;             y = f + dt (-k1 + 2 k2)
//   stage 3: k3 = A y + s3;             f = f + dt (k1/6 + 2 k2/3 + k3/6)
// ---------------------------------------------------------------------------------------
template <typename T>
__global__ void k_rk3_stage(int stage, long long n, T dt, T* __restrict__ f, T* __restrict__ y, T* __restrict__ k1,
                            T* __restrict__ k2, T* __restrict__ k3, const T* __restrict__ s) {
  for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<long long>(gridDim.x) * blockDim.x) {
    const T si = s ? s[i] : T(0);
    if (stage == 1) {
      const T a = k1[i] + si;
      k1[i] = a;
      y[i] = f[i] + dt * T(0.5) * a;
    } else if (stage == 2) {
      const T b = k2[i] + si;
      k2[i] = b;
      y[i] = f[i] + dt * (T(-1) * k1[i] + T(2) * b);
    } else {
      const T c = k3[i] + si;
      f[i] = f[i] + dt * (k1[i] / T(6) + T(2) / T(3) * k2[i] + c / T(6));
    }
  }
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
// partial[j * kRedBlocks + b] = sum over block b's slice of w * V_j, j < k (FP64 sums)
template <typename TV>
__global__ void __launch_bounds__(kRedThreads) k_dots(long long n, int k, const double* __restrict__ w,
                                                      const TV* __restrict__ V, long long ldv,
                                                      double* __restrict__ partial) {
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
  (void)k;
}
// out[j] = sum_b partial[j * nb + b] in block order (deterministic second pass)
__global__ void k_dots_final(int k, int nb, const double* __restrict__ partial, double* __restrict__ out) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= k) return;
  double s = 0.0;
  for (int b = 0; b < nb; ++b) s += partial[j * static_cast<long long>(nb) + b];
  out[j] = s;
}
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
// w -= sum_{j<k} h[j] V_j   (h on the device)
template <typename TV>
__global__ void k_orth_update(long long n, int k, const double* __restrict__ h, const TV* __restrict__ V, long long ldv,
                              double* __restrict__ w) {
  for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<long long>(gridDim.x) * blockDim.x) {
    double acc = w[i];
    for (int j = 0; j < k; ++j) acc = fma(-h[j], static_cast<double>(V[j * ldv + i]), acc);
    w[i] = acc;
  }
}
// V_j = w * inv  (stored in the basis precision)
template <typename TV>
__global__ void k_store_basis(long long n, double inv, const double* __restrict__ w, TV* __restrict__ vj) {
  for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<long long>(gridDim.x) * blockDim.x)
    vj[i] = static_cast<TV>(w[i] * inv);
}
// w = x - dt * ax   (the operator I - dt A applied, ax = A x in the matvec precision)
template <typename TV, typename TA>
__global__ void k_shift(long long n, double dt, const TV* __restrict__ x, const TA* __restrict__ ax,
                        double* __restrict__ w) {
  for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<long long>(gridDim.x) * blockDim.x)
    w[i] = static_cast<double>(x[i]) - dt * static_cast<double>(ax[i]);
}
// x += sum_j y[j] V_j  (FP64 solution update; y on the device)
template <typename TV>
__global__ void k_sol_update(long long n, int k, const double* __restrict__ y, const TV* __restrict__ V, long long ldv,
                             double* __restrict__ x) {
  for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<long long>(gridDim.x) * blockDim.x) {
    double acc = x[i];
    for (int j = 0; j < k; ++j) acc = fma(y[j], static_cast<double>(V[j * ldv + i]), acc);
    x[i] = acc;
  }
}
// r = b - (x - dt * ax)   (FP64 outer residual)
__global__ void k_residual(long long n, double dt, const double* __restrict__ b, const double* __restrict__ x,
                           const double* __restrict__ ax, double* __restrict__ r) {
  for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<long long>(gridDim.x) * blockDim.x)
    r[i] = b[i] - (x[i] - dt * ax[i]);
}
__global__ void k_copy_f64(long long n, const double* __restrict__ a, double* __restrict__ b) {
  for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<long long>(gridDim.x) * blockDim.x)
    b[i] = a[i];
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
  size_t v, w, r, ax64, axmv, h, y, partial, total;
};

GmresLayout gmres_layout(long long n, int m, bool mixed) {
  GmresLayout L{};
  size_t off = 0;
  auto take = [&](size_t bytes) {
    const size_t o = off;
    off += align256(bytes);
    return o;
  };
  L.v = take(static_cast<size_t>(m + 1) * n * (mixed ? sizeof(float) : sizeof(double)));
  L.w = take(n * sizeof(double));
  L.r = take(n * sizeof(double));
  L.ax64 = take(n * sizeof(double));
  L.axmv = take(n * (mixed ? sizeof(float) : sizeof(double)));
  L.h = take((m + 1) * sizeof(double));
  L.y = take((m + 1) * sizeof(double));
  L.partial = take(static_cast<size_t>(m + 1) * asg::kRedBlocks * sizeof(double));
  L.total = off;
  return L;
}

double host_norm(const double* d_partial, cudaStream_t s, asg_status* st) {
  std::vector<double> p(asg::kRedBlocks);
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

// One GMRES(m) cycle on (I - dt A) delta = r0 (r0 FP64), adding delta to x64 in FP64.  TV is
// the basis and operator-application precision.  Stops early when the residual estimate
// drops to rtol_abs.  *iters = Arnoldi steps taken, *resid = final residual estimate.
template <typename TV>
asg_status gmres_cycle(asg_plan* plan, long long n, double dt, const double* r0, double* x64, int m, double rtol_abs,
                       unsigned char* base, const GmresLayout& L, cudaStream_t s, int* iters, double* resid) {
  TV* V = reinterpret_cast<TV*>(base + L.v);
  double* w = reinterpret_cast<double*>(base + L.w);
  TV* axmv = reinterpret_cast<TV*>(base + L.axmv);
  double* h_dev = reinterpret_cast<double*>(base + L.h);
  double* y_dev = reinterpret_cast<double*>(base + L.y);
  double* partial = reinterpret_cast<double*>(base + L.partial);
  const int gr = asg::grid_for(n);
  asg_status st = ASG_OK;
  *iters = 0;
  asg::k_norm2<<<asg::kRedBlocks, asg::kRedThreads, 0, s>>>(n, r0, partial);
  const double beta = host_norm(partial, s, &st);
  if (st) return st;
  *resid = beta;
  if (beta <= rtol_abs || beta == 0.0) return ASG_OK;
  asg::k_store_basis<TV><<<gr, 256, 0, s>>>(n, 1.0 / beta, r0, V);
  std::vector<double> H(static_cast<size_t>(m + 1) * m, 0.0), cs(m), sn(m), g(m + 1, 0.0), hcol(m + 1), yv(m);
  g[0] = beta;
  int kdone = 0;
  for (int j = 0; j < m; ++j) {
    // w = V_j - dt * A V_j
    asg_status ast = sizeof(TV) == 4 ? asg_apply_f32(plan, reinterpret_cast<const float*>(V + j * n),
                                                     reinterpret_cast<float*>(axmv), s)
                                     : asg_apply_f64(plan, reinterpret_cast<const double*>(V + j * n),
                                                     reinterpret_cast<double*>(axmv), s);
    if (ast) return ast;
    asg::k_shift<TV, TV><<<gr, 256, 0, s>>>(n, dt, V + j * n, axmv, w);
    std::fill(hcol.begin(), hcol.end(), 0.0);
    std::vector<double> hp(j + 1);
    for (int pass = 0; pass < 2; ++pass) {  // classical Gram-Schmidt, reorthogonalised (FP64)
      asg::k_dots<TV><<<dim3(asg::kRedBlocks, j + 1), asg::kRedThreads, 0, s>>>(n, j + 1, w, V, n, partial);
      asg::k_dots_final<<<1, 64, 0, s>>>(j + 1, asg::kRedBlocks, partial, h_dev);
      asg::k_orth_update<TV><<<gr, 256, 0, s>>>(n, j + 1, h_dev, V, n, w);
      ASG_CUDA(cudaMemcpyAsync(hp.data(), h_dev, (j + 1) * sizeof(double), cudaMemcpyDeviceToHost, s));
      ASG_CUDA(cudaStreamSynchronize(s));
      for (int i = 0; i <= j; ++i) hcol[i] += hp[i];
    }
    asg::k_norm2<<<asg::kRedBlocks, asg::kRedThreads, 0, s>>>(n, w, partial);
    const double hn = host_norm(partial, s, &st);
    if (st) return st;
    hcol[j + 1] = hn;
    // previous Givens rotations, then a new one (FP64, host)
    for (int i = 0; i < j; ++i) {
      const double a = cs[i] * hcol[i] + sn[i] * hcol[i + 1];
      hcol[i + 1] = -sn[i] * hcol[i] + cs[i] * hcol[i + 1];
      hcol[i] = a;
    }
    const double den = std::hypot(hcol[j], hcol[j + 1]);
    cs[j] = den > 0 ? hcol[j] / den : 1.0;
    sn[j] = den > 0 ? hcol[j + 1] / den : 0.0;
    hcol[j] = den;
    g[j + 1] = -sn[j] * g[j];
    g[j] = cs[j] * g[j];
    for (int i = 0; i <= j; ++i) H[static_cast<size_t>(i) * m + j] = hcol[i];
    kdone = j + 1;
    *resid = std::fabs(g[j + 1]);
    if (*resid <= rtol_abs || hn == 0.0) break;
    if (j + 1 < m) asg::k_store_basis<TV><<<gr, 256, 0, s>>>(n, 1.0 / hn, w, V + (j + 1) * n);
  }
  // back substitution H y = g, then x += V y (FP64 update)
  for (int i = kdone - 1; i >= 0; --i) {
    double acc = g[i];
    for (int k = i + 1; k < kdone; ++k) acc -= H[static_cast<size_t>(i) * m + k] * yv[k];
    yv[i] = acc / H[static_cast<size_t>(i) * m + i];
  }
  ASG_CUDA(cudaMemcpyAsync(y_dev, yv.data(), kdone * sizeof(double), cudaMemcpyHostToDevice, s));
  asg::k_sol_update<TV><<<gr, 256, 0, s>>>(n, kdone, y_dev, V, n, x64);
  ASG_CUDA(cudaStreamSynchronize(s));  // yv is host memory read by the copy above
  *iters = kdone;
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return asg::cuda_fail(e, "gmres kernels");
  return ASG_OK;
}

template <typename TV>
asg_status be_solve(asg_plan* p, double dt, const double* b, double* x, const asg_gmres_opts* o, asg_gmres_info* info,
                    void* work, size_t work_bytes, void* stream) {
  asg_plan_stats ps{};
  asg_plan_stats_get(p, &ps);
  const long long n = ps.dof;
  const int m = o->restart;
  const GmresLayout L = gmres_layout(n, m, sizeof(TV) == 4);
  if (work_bytes < L.total) return fail(ASG_ERR_CAPACITY, "be_solve: workspace needs %zu bytes", L.total);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  unsigned char* base = static_cast<unsigned char*>(work);
  double* r = reinterpret_cast<double*>(base + L.r);
  double* ax64 = reinterpret_cast<double*>(base + L.ax64);
  double* partial = reinterpret_cast<double*>(base + L.partial);
  const int gr = asg::grid_for(n);
  asg_status st = ASG_OK;
  asg::k_norm2<<<asg::kRedBlocks, asg::kRedThreads, 0, s>>>(n, b, partial);
  const double bnorm = host_norm(partial, s, &st);
  if (st) return st;
  asg_gmres_info inf{};
  inf.rel_residual = 1.0;
  for (int outer = 0; outer <= o->max_outer; ++outer) {
    // FP64 outer residual r = b - (I - dt A) x
    if ((st = asg_apply_f64(p, x, ax64, s))) return st;
    asg::k_residual<<<gr, 256, 0, s>>>(n, dt, b, x, ax64, r);
    asg::k_norm2<<<asg::kRedBlocks, asg::kRedThreads, 0, s>>>(n, r, partial);
    const double rn = host_norm(partial, s, &st);
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
    if ((st = gmres_cycle<TV>(p, n, dt, r, x, m, target, base, L, s, &it, &est))) return st;
    inf.inner_iters += it;
  }
  if (info) *info = inf;
  return ASG_OK;
}

template <typename T>
asg_status rk3(asg_plan* p, T* f, double dt, const T* const* src, T* work, size_t work_bytes, void* stream) {
  if (!p || !f || !work) return fail(ASG_ERR_INVALID, "rk3_step: NULL argument");
  asg_plan_stats st{};
  asg_plan_stats_get(p, &st);
  const long long n = st.dof;
  if (work_bytes < static_cast<size_t>(4 * n) * sizeof(T))
    return fail(ASG_ERR_CAPACITY, "rk3_step: workspace needs %lld bytes", 4 * n * (long long)sizeof(T));
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  T* k1 = work;
  T* k2 = work + n;
  T* k3 = work + 2 * n;
  T* y = work + 3 * n;
  auto apply = [&](const T* in, T* out) {
    return sizeof(T) == 8 ? asg_apply_f64(p, reinterpret_cast<const double*>(in), reinterpret_cast<double*>(out), s)
                          : asg_apply_f32(p, reinterpret_cast<const float*>(in), reinterpret_cast<float*>(out), s);
  };
  const int gr = asg::grid_for(n);
  const T* s1 = src ? src[0] : nullptr;
  const T* s2 = src ? src[1] : nullptr;
  const T* s3 = src ? src[2] : nullptr;
  asg_status a;
  if ((a = apply(f, k1))) return a;
  asg::k_rk3_stage<T><<<gr, 256, 0, s>>>(1, n, static_cast<T>(dt), f, y, k1, k2, k3, s1);
  if ((a = apply(y, k2))) return a;
  asg::k_rk3_stage<T><<<gr, 256, 0, s>>>(2, n, static_cast<T>(dt), f, y, k1, k2, k3, s2);
  if ((a = apply(y, k3))) return a;
  asg::k_rk3_stage<T><<<gr, 256, 0, s>>>(3, n, static_cast<T>(dt), f, y, k1, k2, k3, s3);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return asg::cuda_fail(e, "rk3 stage launch");
  return ASG_OK;
}

}  // namespace

extern "C" {

asg_status asg_rk3_step_f64(asg_plan* plan, double* d_f, double dt, const double* const* d_src, double* d_work,
                            size_t work_bytes, void* stream) {
  return rk3<double>(plan, d_f, dt, d_src, d_work, work_bytes, stream);
}
asg_status asg_rk3_step_f32(asg_plan* plan, float* d_f, double dt, const float* const* d_src, float* d_work,
                            size_t work_bytes, void* stream) {
  return rk3<float>(plan, d_f, dt, d_src, d_work, work_bytes, stream);
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
  if (opts->restart < 1 || opts->restart > 200) return fail(ASG_ERR_INVALID, "be_workspace: restart=%d", opts->restart);
  asg_plan_stats ps{};
  asg_plan_stats_get(plan, &ps);
  *bytes = gmres_layout(ps.dof, opts->restart, opts->mixed != 0).total;
  return ASG_OK;
}

asg_status asg_be_solve(asg_plan* plan, double dt, const double* d_b, double* d_x, const asg_gmres_opts* opts,
                        asg_gmres_info* info, void* d_work, size_t work_bytes, void* stream) {
  if (!plan || !d_b || !d_x || !opts || !d_work) return fail(ASG_ERR_INVALID, "be_solve: NULL argument");
  if (opts->restart < 1 || opts->restart > 200 || opts->max_outer < 0 || !(opts->tol > 0) ||
      !(opts->inner_reduction > 0 && opts->inner_reduction < 1))
    return fail(ASG_ERR_INVALID, "be_solve: bad options");
  return opts->mixed ? be_solve<float>(plan, dt, d_b, d_x, opts, info, d_work, work_bytes, stream)
                     : be_solve<double>(plan, dt, d_b, d_x, opts, info, d_work, work_bytes, stream);
}

}  // extern "C"
