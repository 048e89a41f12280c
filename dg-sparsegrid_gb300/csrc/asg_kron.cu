// Kronecker products and the batched small-GEMM path:
//   asg_gemm_vbatched_*   Kronmult/gemm_vbatched.m (MAGMA-style variable-size batch)
//   asg_kron_plan_*       Kronmult/kronmult{1..6}_batch.m: per-level GEMM lists of the
//                         recursive product kron(A1,..,An)*X, executed level by level
//   asg_krond_*           krond.m: the explicit Kronecker product
#include <algorithm>
#include <cstring>
#include <mutex>
#include <new>
#include <vector>

#include "asg_internal.h"

namespace asg {
namespace {

constexpr int kMaxKron = 6;

// ---------------------------------------------------------------------------------------
// Small column-major GEMM, one CTA per problem: C = alpha*op(A)*op(B) + beta*C.
// beta == 0 overwrites C without reading it (gemm.m:20-24).
// ---------------------------------------------------------------------------------------
template <typename T>
__device__ __forceinline__ void cta_gemm(char ta, char tb, int m, int n, int k, T alpha, const T* A, int lda,
                                         const T* B, int ldb, T beta, T* C, int ldc) {
  const bool tA = (ta == 'T' || ta == 't' || ta == 'C' || ta == 'c');
  const bool tB = (tb == 'T' || tb == 't' || tb == 'C' || tb == 'c');
  for (int idx = threadIdx.x; idx < m * n; idx += blockDim.x) {
    const int i = idx % m, j = idx / m;
    T acc = T(0);
    for (int l = 0; l < k; ++l) {
      const T a = tA ? A[i * static_cast<long long>(lda) + l] : A[l * static_cast<long long>(lda) + i];
      const T b = tB ? B[l * static_cast<long long>(ldb) + j] : B[j * static_cast<long long>(ldb) + l];
      acc = fma(a, b, acc);
    }
    T* c = C + j * static_cast<long long>(ldc) + i;
    *c = (beta == T(0)) ? alpha * acc : fma(beta, *c, alpha * acc);
  }
}

template <typename T>
__global__ void k_gemm_vbatched(char ta, char tb, const int* m, const int* n, const int* k, T alpha,
                                const T* const* A, const int* lda, const T* const* B, const int* ldb, T beta,
                                T* const* C, const int* ldc, int batch) {
  for (int p = blockIdx.x; p < batch; p += gridDim.x)
    cta_gemm<T>(ta, tb, m[p], n[p], k[p], alpha, A[p], lda[p], B[p], ldb[p], beta, C[p], ldc[p]);
}

// ---------------------------------------------------------------------------------------
// kronmult batch lists.  Operand ids: 0..n-1 the factors A1..An, n = X, n+1 = Y,
// n+2+l = temporary of recursion depth l (all in one workspace).
// ---------------------------------------------------------------------------------------
struct KDesc {
  int level;  // 1-based list the reference appends to (batch_list{level})
  int m, n, k;
  char ta, tb;
  int a_id, b_id, c_id;
  long long a_off, b_off, c_off;
  int lda, ldb, ldc;
};

struct Planner {
  std::vector<KDesc> out;
  std::vector<long long> tmp_elems;  // per temp id (index = id - (n+2))
  int nfac = 0;

  // flops_kron{n}.m: (flops1, flops2, imethod)
  static void flops(const int* nr, const int* nc, int n, double& f1, double& f2, int& meth) {
    if (n == 1) {
      f1 = f2 = 2.0 * nr[0] * nc[0];
      meth = 1;
      return;
    }
    if (n == 2) {
      const double nrowX = nc[1], ncolX = nc[0];
      f1 = 2.0 * nr[1] * nc[1] * ncolX + 2.0 * nr[1] * nc[0] * nr[0];
      f2 = 2.0 * nrowX * nc[0] * nr[0] + 2.0 * nr[1] * nc[1] * nr[0];
      meth = f1 <= f2 ? 1 : 2;
      return;
    }
    double jf1, jf2;
    int jm;
    flops(nr + 1, nc + 1, n - 1, jf1, jf2, jm);
    const double inner = jm == 1 ? jf1 : jf2;
    double nrowX = 1, nrowY = 1;
    for (int i = 1; i < n; ++i) {
      nrowX *= nc[i];
      nrowY *= nr[i];
    }
    f1 = inner * nc[0] + 2.0 * nrowY * nc[0] * nr[0];
    f2 = 2.0 * nrowX * nc[0] * nr[0] + inner * nr[0];
    meth = f1 <= f2 ? 1 : 2;
  }

  int new_tmp(long long elems) {
    tmp_elems.push_back(elems);
    return nfac + 2 + static_cast<int>(tmp_elems.size()) - 1;
  }

  // Records kron(A_first..A_first+n-1) * X  (X: operand xid at xoff, prod(nc) x nvec) into
  // operand yid at yoff; lists offset by lvl0 (the reference passes sub-ranges of the lists).
  void rec(int first, const int* nr, const int* nc, int n, int xid, long long xoff, int yid, long long yoff,
           long long nvec, int lvl0) {
    if (n == 1) {  // kronmult1_batch.m: Y = A1 * reshape(X, ncol1, nvec)
      out.push_back({lvl0 + 1, nr[0], static_cast<int>(nvec), nc[0], 'N', 'N', first, xid, yid, 0, xoff, yoff, nr[0],
                     nc[0], nr[0]});
      return;
    }
    double f1, f2;
    int meth;
    flops(nr, nc, n, f1, f2, meth);
    long long nrowX = 1, nrowY = 1, nrowYin = 1;
    for (int i = 0; i < n; ++i) {
      nrowX *= nc[i];
      nrowY *= nr[i];
    }
    for (int i = 1; i < n; ++i) nrowYin *= nr[i];
    if (meth == 1) {
      // Ytmp = kron(A2..An) * X  (X viewed as prod(nc[1:]) x (nc0*nvec)), then per vector
      // Y_i = reshape(Ytmp_i, [mm, nc0]) * A1^T  (kronmult2_batch.m:86-110)
      const long long tsz = nrowYin * nc[0] * nvec;
      const int t = new_tmp(tsz);
      rec(first + 1, nr + 1, nc + 1, n - 1, xid, xoff, t, 0, nc[0] * nvec, lvl0);
      const int mm = static_cast<int>(nrowYin);
      for (long long i = 0; i < nvec; ++i)
        out.push_back({lvl0 + n, mm, nr[0], nc[0], 'N', 'T', t, first, yid, i * mm * nc[0], 0, yoff + i * nrowY, mm,
                       nr[0], mm});
    } else {
      // Ytmp(:, i*nr0 ..) = reshape(X_i, [prod(nc[1:]), nc0]) * A1^T, then Y = kron(A2..An) * Ytmp
      long long inner = 1;
      for (int i = 1; i < n; ++i) inner *= nc[i];
      const long long tsz = inner * nr[0] * nvec;
      const int t = new_tmp(tsz);
      for (long long i = 0; i < nvec; ++i)
        out.push_back({lvl0 + 1, static_cast<int>(inner), nr[0], nc[0], 'N', 'T', xid, first, t, xoff + i * nrowX, 0,
                       i * inner * nr[0], static_cast<int>(inner), nr[0], static_cast<int>(inner)});
      if (n == 2) {
        out.push_back({lvl0 + 2, nr[1], static_cast<int>(nr[0] * nvec), nc[1], 'N', 'N', first + 1, t, yid, 0, 0, yoff,
                       nr[1], nc[1], nr[1]});
      } else {
        rec(first + 1, nr + 1, nc + 1, n - 1, t, 0, yid, yoff, nr[0] * nvec, lvl0 + 1);
      }
    }
  }
};

struct KDev {  // device-side descriptor with a resolved operand kind
  int m, n, k;
  char ta, tb;
  int a_id, b_id, c_id;
  long long a_off, b_off, c_off;
  int lda, ldb, ldc;
};

template <typename T>
struct KBases {
  const T* fac[kMaxKron];
  const T* x;
  T* y;
  T* work;
  long long tmp_off[kMaxKron + 2];  // element offset of each temporary in the workspace
  int nfac;
};

template <typename T>
__device__ __forceinline__ const T* kop(const KBases<T>& b, int id, long long off) {
  if (id < b.nfac) return b.fac[id] + off;
  if (id == b.nfac) return b.x + off;
  if (id == b.nfac + 1) return b.y + off;
  return b.work + b.tmp_off[id - b.nfac - 2] + off;
}

template <typename T>
__global__ void k_kron_level(const KDev* __restrict__ d, int count, KBases<T> b) {
  for (int p = blockIdx.x; p < count; p += gridDim.x) {
    const KDev e = d[p];
    T* c = const_cast<T*>(kop(b, e.c_id, e.c_off));
    cta_gemm<T>(e.ta, e.tb, e.m, e.n, e.k, T(1), kop(b, e.a_id, e.a_off), e.lda, kop(b, e.b_id, e.b_off), e.ldb, T(0),
                c, e.ldc);
  }
}

struct KDims {
  int nr[kMaxKron], nc[kMaxKron];
};

// krond.m: out(r, c) = prod_i A_i(r_i, c_i), last factor fastest, column-major output.
template <typename T>
__global__ void k_krond(KBases<T> b, int n, KDims dims, long long rows, long long cols, T* out) {
  const long long total = rows * cols;
  for (long long idx = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; idx < total;
       idx += static_cast<long long>(gridDim.x) * blockDim.x) {
    long long r = idx % rows, c = idx / rows;
    T v = T(1);
    for (int i = n - 1; i >= 0; --i) {
      const int nr = dims.nr[i], nc = dims.nc[i];
      const int ri = static_cast<int>(r % nr), ci = static_cast<int>(c % nc);
      r /= nr;
      c /= nc;
      v *= b.fac[i][ci * static_cast<long long>(nr) + ri];
    }
    out[idx] = v;
  }
}

}  // namespace
}  // namespace asg

struct asg_kron_plan {
  int nfac = 0;
  long long nvec = 0;
  int nr[asg::kMaxKron] = {0}, nc[asg::kMaxKron] = {0};
  std::vector<asg::KDesc> descs;              // in list order (level 1..n), recording order within
  std::vector<int> level_start;               // [n+1] offsets of each level in the device table
  std::vector<long long> tmp_off;             // element offset of each temporary
  long long work_elems = 0;
  std::vector<asg::KDev> dev;                 // device-order descriptors (uploaded on first use)
  asg::KDev* d_desc = nullptr;
  std::mutex upload_mu;                       // serialises the first-use upload across host threads
};

using asg::fail;

namespace {

template <typename T>
asg_status kron_exec(const asg_kron_plan* cp, const T* const* A, const T* X, T* Y, T* work, size_t work_bytes,
                     void* stream) {
  if (!cp || !A || !X || !Y) return fail(ASG_ERR_INVALID, "kron_batch: NULL argument");
  asg_kron_plan* p = const_cast<asg_kron_plan*>(cp);
  if (!p->dev.empty()) {  // the first execution uploads the descriptor table, once per plan
    std::lock_guard<std::mutex> lock(p->upload_mu);
    if (!p->d_desc) {
      asg::KDev* d = nullptr;
      ASG_CUDA(cudaMalloc(reinterpret_cast<void**>(&d), p->dev.size() * sizeof(asg::KDev)));
      cudaError_t e = cudaMemcpy(d, p->dev.data(), p->dev.size() * sizeof(asg::KDev), cudaMemcpyHostToDevice);
      if (e != cudaSuccess) {
        cudaFree(d);
        return asg::cuda_fail(e, "kron_batch: descriptor upload");
      }
      p->d_desc = d;  // published only once the table is complete
    }
  }
  if (work_bytes < static_cast<size_t>(p->work_elems) * sizeof(T))
    return fail(ASG_ERR_CAPACITY, "kron_batch: workspace needs %lld bytes", p->work_elems * (long long)sizeof(T));
  if (p->work_elems > 0 && !work) return fail(ASG_ERR_INVALID, "kron_batch: NULL workspace");
  asg::KBases<T> b{};
  for (int i = 0; i < p->nfac; ++i) {
    if (!A[i]) return fail(ASG_ERR_INVALID, "kron_batch: factor %d is NULL", i);
    b.fac[i] = A[i];
  }
  b.x = X;
  b.y = Y;
  b.work = work;
  b.nfac = p->nfac;
  for (size_t i = 0; i < p->tmp_off.size(); ++i) b.tmp_off[i] = p->tmp_off[i];
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  for (int l = 0; l < p->nfac; ++l) {
    const int cnt = p->level_start[l + 1] - p->level_start[l];
    if (cnt == 0) continue;
    const int grid = cnt < 65535 ? cnt : 65535;
    asg::k_kron_level<T><<<grid, 128, 0, s>>>(p->d_desc + p->level_start[l], cnt, b);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return asg::cuda_fail(e, "kron level launch");
  }
  return ASG_OK;
}

template <typename T>
asg_status gemm_vb(char ta, char tb, const int* m, const int* n, const int* k, T alpha, const T* const* A,
                   const int* lda, const T* const* B, const int* ldb, T beta, T* const* C, const int* ldc, int batch,
                   void* stream) {
  if (batch < 0) return fail(ASG_ERR_INVALID, "gemm_vbatched: batch=%d", batch);
  if (batch == 0) return ASG_OK;
  if (!m || !n || !k || !A || !lda || !B || !ldb || !C || !ldc) return fail(ASG_ERR_INVALID, "gemm_vbatched: NULL array");
  const char ok[] = "NnTtCc";
  if (!std::strchr(ok, ta) || !std::strchr(ok, tb) || !ta || !tb)
    return fail(ASG_ERR_INVALID, "gemm_vbatched: trans flags must be N/T/C");
  const int grid = batch < 65535 ? batch : 65535;
  asg::k_gemm_vbatched<T><<<grid, 128, 0, static_cast<cudaStream_t>(stream)>>>(ta, tb, m, n, k, alpha, A, lda, B, ldb,
                                                                               beta, C, ldc, batch);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return asg::cuda_fail(e, "gemm_vbatched launch");
  return ASG_OK;
}

template <typename T>
asg_status krond_exec(int n, const int* nrow, const int* ncol, const T* const* A, T* out, void* stream) {
  asg::KBases<T> b{};
  asg::KDims dims{};
  long long rows = 1, cols = 1;
  for (int i = 0; i < n; ++i) {
    if (!A[i]) return fail(ASG_ERR_INVALID, "krond: factor %d is NULL", i);
    b.fac[i] = A[i];
    dims.nr[i] = nrow[i];
    dims.nc[i] = ncol[i];
    rows *= nrow[i];
    cols *= ncol[i];
  }
  b.nfac = n;
  const long long total = rows * cols;
  const int grid = static_cast<int>(std::min<long long>((total + 255) / 256, 152LL * 16));
  asg::k_krond<T><<<grid > 0 ? grid : 1, 256, 0, static_cast<cudaStream_t>(stream)>>>(b, n, dims, rows, cols, out);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return asg::cuda_fail(e, "krond launch");
  return ASG_OK;
}

asg_status check_kron_dims(int n, const int* nrow, const int* ncol) {
  if (n < 1 || n > asg::kMaxKron) return fail(n < 1 ? ASG_ERR_INVALID : ASG_ERR_UNSUPPORTED, "kron: invalid nkron=%d", n);
  if (!nrow || !ncol) return fail(ASG_ERR_INVALID, "kron: NULL sizes");
  for (int i = 0; i < n; ++i)
    if (nrow[i] < 1 || ncol[i] < 1 || nrow[i] > 65536 || ncol[i] > 65536)
      return fail(ASG_ERR_INVALID, "kron: factor %d has size %dx%d", i, nrow[i], ncol[i]);
  return ASG_OK;
}

}  // namespace

extern "C" {

asg_status asg_gemm_vbatched_f64(char ta, char tb, const int* m, const int* n, const int* k, double alpha,
                                 const double* const* A, const int* lda, const double* const* B, const int* ldb,
                                 double beta, double* const* C, const int* ldc, int batch, void* stream) {
  return gemm_vb<double>(ta, tb, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, batch, stream);
}
asg_status asg_gemm_vbatched_f32(char ta, char tb, const int* m, const int* n, const int* k, float alpha,
                                 const float* const* A, const int* lda, const float* const* B, const int* ldb,
                                 float beta, float* const* C, const int* ldc, int batch, void* stream) {
  return gemm_vb<float>(ta, tb, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, batch, stream);
}

asg_status asg_kron_plan_create(int nkron, const int* nrow, const int* ncol, long long nvec, asg_kron_plan** out) {
  if (!out) return fail(ASG_ERR_INVALID, "kron_plan_create: NULL output");
  *out = nullptr;
  asg_status st = check_kron_dims(nkron, nrow, ncol);
  if (st) return st;
  if (nvec < 1) return fail(ASG_ERR_INVALID, "kron_plan_create: nvec=%lld", nvec);
  asg_kron_plan* p = new (std::nothrow) asg_kron_plan;
  if (!p) return fail(ASG_ERR_NOMEM, "kron_plan_create: out of host memory");
  p->nfac = nkron;
  p->nvec = nvec;
  for (int i = 0; i < nkron; ++i) {
    p->nr[i] = nrow[i];
    p->nc[i] = ncol[i];
  }
  asg::Planner pl;
  pl.nfac = nkron;
  pl.rec(0, p->nr, p->nc, nkron, nkron, 0, nkron + 1, 0, nvec, 0);
  // stable order by level: the lists execute level 1 .. n
  p->level_start.assign(nkron + 1, 0);
  std::vector<asg::KDev>& dev = p->dev;
  for (int l = 1; l <= nkron; ++l) {
    p->level_start[l - 1] = static_cast<int>(dev.size());
    for (const auto& d : pl.out)
      if (d.level == l) {
        p->descs.push_back(d);
        dev.push_back({d.m, d.n, d.k, d.ta, d.tb, d.a_id, d.b_id, d.c_id, d.a_off, d.b_off, d.c_off, d.lda, d.ldb, d.ldc});
      }
  }
  p->level_start[nkron] = static_cast<int>(dev.size());
  long long off = 0;
  for (long long e : pl.tmp_elems) {
    p->tmp_off.push_back(off);
    off += (e + 31) / 32 * 32;
  }
  p->work_elems = off;
  *out = p;
  return ASG_OK;
}

asg_status asg_kron_plan_destroy(asg_kron_plan* p) {
  if (!p) return ASG_OK;
  cudaFree(p->d_desc);
  delete p;
  return ASG_OK;
}

asg_status asg_kron_plan_workspace(const asg_kron_plan* p, size_t* bytes_f64, size_t* bytes_f32) {
  if (!p) return fail(ASG_ERR_INVALID, "kron_plan_workspace: NULL plan");
  if (bytes_f64) *bytes_f64 = static_cast<size_t>(p->work_elems) * sizeof(double);
  if (bytes_f32) *bytes_f32 = static_cast<size_t>(p->work_elems) * sizeof(float);
  return ASG_OK;
}

asg_status asg_kron_plan_lists(const asg_kron_plan* p, asg_gemm_desc* out, int capacity, int* count) {
  if (!p) return fail(ASG_ERR_INVALID, "kron_plan_lists: NULL plan");
  const int n = static_cast<int>(p->descs.size());
  if (count) *count = n;
  if (capacity == 0) return ASG_OK;
  if (!out) return fail(ASG_ERR_INVALID, "kron_plan_lists: NULL output");
  if (capacity < n) return fail(ASG_ERR_CAPACITY, "kron_plan_lists: %d descriptors, capacity %d", n, capacity);
  for (int i = 0; i < n; ++i) {
    const auto& d = p->descs[i];
    asg_gemm_desc& o = out[i];
    o.level = d.level;
    o.m = d.m;
    o.n = d.n;
    o.k = d.k;
    o.trans_a = d.ta;
    o.trans_b = d.tb;
    o.alpha = 1.0;
    o.beta = 0.0;
    // temporaries are reported as offsets into the single workspace operand (nkron + 2)
    auto resolve = [&](int id, long long off, int& oid, long long& ooff) {
      if (id >= p->nfac + 2) {
        oid = p->nfac + 2;
        ooff = p->tmp_off[id - p->nfac - 2] + off;
      } else {
        oid = id;
        ooff = off;
      }
    };
    resolve(d.a_id, d.a_off, o.a_operand, o.a_offset);
    resolve(d.b_id, d.b_off, o.b_operand, o.b_offset);
    resolve(d.c_id, d.c_off, o.c_operand, o.c_offset);
    o.lda = d.lda;
    o.ldb = d.ldb;
    o.ldc = d.ldc;
  }
  return ASG_OK;
}

asg_status asg_kron_batch_f64(const asg_kron_plan* p, const double* const* A, const double* X, double* Y,
                              void* work, size_t work_bytes, void* stream) {
  return kron_exec<double>(p, A, X, Y, static_cast<double*>(work), work_bytes, stream);
}
asg_status asg_kron_batch_f32(const asg_kron_plan* p, const float* const* A, const float* X, float* Y, void* work,
                              size_t work_bytes, void* stream) {
  return kron_exec<float>(p, A, X, Y, static_cast<float*>(work), work_bytes, stream);
}

asg_status asg_krond_f64(int nkron, const int* nrow, const int* ncol, const double* const* A, double* out,
                         void* stream) {
  asg_status st = check_kron_dims(nkron, nrow, ncol);
  if (st) return st;
  if (!A || !out) return fail(ASG_ERR_INVALID, "krond: NULL argument");
  return krond_exec<double>(nkron, nrow, ncol, A, out, stream);
}

}  // extern "C"

// ---------------------------------------------------------------------------------------
// Allocation-free executor: asg_kron_batch_static_f64.
//
// For callers that may not allocate device memory at call time -- code running where
// cudaMalloc is not allowed or not wanted (inside a host callback, under an allocator that
// is being torn down, in a time-critical loop that must not synchronise the device), or a
// caller that owns no allocator at all.  The recursion's temporaries live in one fixed
// device array that this file declares; the GEMM descriptors travel in the launch
// parameters, so nothing is uploaded and nothing is allocated.
//
// Contract:
//  * the first call on each device (that device current) looks up the array's address once;
//    make that first call before any stream capture;
//  * plans whose workspace exceeds ASG_KRON_STATIC_SCRATCH_BYTES are rejected with
//    ASG_ERR_CAPACITY before anything is launched;
//  * every call on a device shares the one array and it keeps the previous call's values.
//    Nothing in it has to start at zero: every temporary element is written (beta = 0
//    GEMMs) before any GEMM reads it.  Calls whose launches overlap on the GPU (different
//    streams, or host threads racing on one device) overwrite each other's temporaries:
//    the caller must order them.
// ---------------------------------------------------------------------------------------
static __device__ __align__(256) double g_kron_scratch[ASG_KRON_STATIC_SCRATCH_BYTES / sizeof(double)];

namespace asg {
namespace {

constexpr int kStaticChunk = 48;  // descriptors per launch, carried by value
constexpr int kStaticMaxDevices = 64;

struct KChunk {
  KDev d[kStaticChunk];
  int count;
};
static_assert(sizeof(KChunk) + sizeof(KBases<double>) <= 4096, "launch parameters exceed 4 KB");

__global__ void k_kron_level_static(const KChunk chunk, KBases<double> b) {
  for (int p = blockIdx.x; p < chunk.count; p += gridDim.x) {
    const KDev e = chunk.d[p];
    double* c = const_cast<double*>(kop(b, e.c_id, e.c_off));
    cta_gemm<double>(e.ta, e.tb, e.m, e.n, e.k, 1.0, kop(b, e.a_id, e.a_off), e.lda, kop(b, e.b_id, e.b_off), e.ldb,
                     0.0, c, e.ldc);
  }
}

std::mutex g_scratch_mu;
double* g_scratch_ptr[kStaticMaxDevices];

// The array's device address for the current device.  Only a successful lookup is cached: a
// failed one (for instance one attempted during a stream capture) is retried on the next call.
asg_status static_scratch(double** out) {
  int dev = 0;
  ASG_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kStaticMaxDevices)
    return fail(ASG_ERR_UNSUPPORTED, "kron_batch_static: device %d beyond the %d supported", dev, kStaticMaxDevices);
  std::lock_guard<std::mutex> lock(g_scratch_mu);
  if (!g_scratch_ptr[dev]) {
    void* ptr = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&ptr, g_kron_scratch);
    if (e != cudaSuccess || !ptr)
      return cuda_fail(e != cudaSuccess ? e : cudaErrorInvalidSymbol, "cudaGetSymbolAddress(kron scratch)");
    g_scratch_ptr[dev] = static_cast<double*>(ptr);
  }
  *out = g_scratch_ptr[dev];
  return ASG_OK;
}

}  // namespace
}  // namespace asg

extern "C" asg_status asg_kron_batch_static_f64(const asg_kron_plan* p, const double* const* A, const double* X,
                                                double* Y, void* stream) {
  if (!p || !A || !X || !Y) return fail(ASG_ERR_INVALID, "kron_batch_static: NULL argument");
  const unsigned long long need = static_cast<unsigned long long>(p->work_elems) * sizeof(double);
  if (need > ASG_KRON_STATIC_SCRATCH_BYTES)
    return fail(ASG_ERR_CAPACITY,
                "kron_batch_static: the plan needs %llu bytes of scratch, the static scratch holds %llu; "
                "use asg_kron_batch_f64 with a caller workspace",
                need, static_cast<unsigned long long>(ASG_KRON_STATIC_SCRATCH_BYTES));
  double* work = nullptr;
  asg_status st = asg::static_scratch(&work);
  if (st) return st;
  asg::KBases<double> b{};
  for (int i = 0; i < p->nfac; ++i) {
    if (!A[i]) return fail(ASG_ERR_INVALID, "kron_batch_static: factor %d is NULL", i);
    b.fac[i] = A[i];
  }
  b.x = X;
  b.y = Y;
  b.work = work;
  b.nfac = p->nfac;
  for (size_t i = 0; i < p->tmp_off.size(); ++i) b.tmp_off[i] = p->tmp_off[i];
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  asg::KChunk chunk;
  for (int l = 0; l < p->nfac; ++l) {  // level by level, each level in chunks of descriptors
    for (int q = p->level_start[l]; q < p->level_start[l + 1]; q += asg::kStaticChunk) {
      const int cnt = std::min(asg::kStaticChunk, p->level_start[l + 1] - q);
      std::memcpy(chunk.d, p->dev.data() + q, cnt * sizeof(asg::KDev));
      chunk.count = cnt;
      // the launch's own return code: an earlier, unrelated error left in the runtime's
      // last-error slot is neither reported nor cleared here
      void* args[] = {&chunk, &b};
      const cudaError_t e = cudaLaunchKernel(reinterpret_cast<const void*>(&asg::k_kron_level_static), dim3(cnt),
                                             dim3(128), args, 0, s);
      if (e != cudaSuccess) return asg::cuda_fail(e, "kron_batch_static launch");
    }
  }
  return ASG_OK;
}
