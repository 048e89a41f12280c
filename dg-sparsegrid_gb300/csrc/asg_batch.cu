// Many independent operator applications in one persistent launch.
//
// A batch is built from existing plans whose element blocks hold at most 256 values.  Its
// packed work list holds (problem, first row) items of `rows_per_item` rows, sorted by
// descending cost (chain flops); persistent warps take items from a device counter (reset
// by a memset in the same stream, so the launch is graph-capturable) and run the warp chain
// algorithm of the single-problem kernel for each row, dispatching on the problem's degree,
// with the operands of the next entries prefetched by asynchronous copies.
// Each row is computed by a fixed set of lanes in a fixed order: results do not depend on
// which warp took the item.  A tuner times (warps per CTA, rows per item) candidates.
#include <algorithm>
#include <new>
#include <vector>

#include "asg_internal.h"

namespace asg {
namespace {

struct BatchProblem {
  const void* f;
  void* y;
  const double* ops64;
  const float* ops32;
  const long long* op_off;
  const int* op_nb;
  const int* idx1d;
  const long long* row_ptr;
  const int* ent;
  const unsigned* active;
  int N, D, B, P, T;
  int stride[kMaxDims];
  int vec;  // f blocks start on 16-byte boundaries: 16-byte asynchronous copies
  int R;    // rows a warp computes side by side (1, 2 or 4; capped by the rows per item)
};

struct BatchItem {
  int prob;
  int row;
};

// Asynchronous 4- or 8-byte global -> shared copy (cp.async, completion tracked per thread by
// commit/wait groups).
template <typename T>
__device__ __forceinline__ void cp_async_elem(T* dst, const T* src) {
  const uint32_t d = static_cast<uint32_t>(__cvta_generic_to_shared(dst));
  if constexpr (sizeof(T) == 8)
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(d), "l"(src) : "memory");
  else
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(d), "l"(src) : "memory");
}
// 16-byte asynchronous global -> shared copy (both addresses 16-byte aligned), L2 only.
template <typename T>
__device__ __forceinline__ void cp_async16(T* dst, const T* src) {
  const uint32_t d = static_cast<uint32_t>(__cvta_generic_to_shared(dst));
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait_pending() { asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory"); }

// ceil(2^16 / 3^k), k = 0..4: the fiber-index reciprocals of deg 3 (at most 81 fibers)
__constant__ unsigned c_recip3[5] = {65536u, 21846u, 7282u, 2428u, 810u};

// Per-warp shared memory of the row kernel: the row's block-base table (8-byte entries), the
// active-factor masks of the stages in flight, then in elements of T kBatchStages stages of
// (column block), two chain buffers and kBatchStages stages of factor blocks.
constexpr int kBatchStages = 2;           // entries in flight per warp (the one computed + 1)
constexpr int kStageVals = 256;           // one element block (deg^d <= 256)
constexpr int kAmatVals = 128;  // every factor block of the entries of the rows side by side
constexpr int kWarpVals = kBatchStages * kStageVals + 2 * kStageVals + kBatchStages * kAmatVals;
constexpr int kWarpHdr = kMaxTerms * kMaxDims * sizeof(long long) + 16 * sizeof(unsigned);
template <typename T>
__host__ __device__ constexpr size_t warp_smem_bytes() {
  return kWarpHdr + kWarpVals * sizeof(T);
}

// R rows of a problem side by side in one warp, each on 32/R lanes with its own slice of every
// buffer (with one row a small deg^d leaves most lanes idle).  For each work entry (column j,
// term t) of a row, the column's block goes through the term's mode-product chain (fastest
// dimension first, kronmult method 1, identity factors skipped) and is added to the row's
// accumulators (Kahan-compensated in FP32), entries in list order -- the single-plan warp
// chain kernel's arithmetic, so results equal it bitwise.  Entries are software-pipelined
// through a ring of kBatchStages shared-memory stages: while entry q is computed, the
// asynchronous copies of entries q+1 .. q+S-1 (column block and every applied factor block)
// are in flight, so an entry's global-memory latency overlaps the arithmetic of the ones
// before it (four stages measured no faster than two on the 256-problem batch).  The rows'
// per-(term, dimension) block bases sit in a shared table; the fiber indexing uses shifts
// for deg 2 and 4 and a multiply by a reciprocal for deg 3 instead of divisions.
template <typename T, int P, int R>
__device__ __forceinline__ void warp_rows(const BatchProblem& pb, int row0, int nrows, unsigned char* wsm, int lane) {
  constexpr int MAXE = 8;
  constexpr bool KAHAN = sizeof(T) == 4;
  constexpr int LG = P == 2 ? 1 : (P == 4 ? 2 : 0);  // log2(P) when P is a power of two
  constexpr int S = kBatchStages;
  constexpr int L = 32 / R;  // lanes per row
  const int sub = lane / L, sl = lane - sub * L;
  const bool on = sub < nrows;  // this lane's row exists
  const int row = row0 + (on ? sub : 0);
  long long* abase = reinterpret_cast<long long*>(wsm);
  unsigned* acts = reinterpret_cast<unsigned*>(wsm + kMaxTerms * kMaxDims * sizeof(long long));  // [S][R]
  T* stage = reinterpret_cast<T*>(wsm + kWarpHdr);  // [S][256]
  T* work = stage + S * kStageVals;                 // [2][256]
  T* amat = work + 2 * kStageVals;                  // [S][kAmatVals]
  const T* f = static_cast<const T*>(pb.f);
  T* y = static_cast<T*>(pb.y);
  const T* ops = sizeof(T) == 8 ? reinterpret_cast<const T*>(pb.ops64) : reinterpret_cast<const T*>(pb.ops32);
  const int B = pb.B, D = pb.D, nt = pb.T, TD = nt * D;
  constexpr int PP = P * P;
  // each row's slices: stage and chain buffers B values apart, factor blocks D*P^2 apart
  const int so = sub * B, ao = sub * D * PP;
  // block base of operator (t, m) at this row's 1-D index: op_off + I_m(row) * nb * P^2
  for (int k = sl; k < TD; k += L) {
    const long long off = pb.op_off[k];
    abase[sub * TD + k] =
        off < 0 ? 0 : off + static_cast<long long>(pb.idx1d[row * D + k % D]) * pb.op_nb[k] * PP;
  }
  __syncwarp();
  // issue the copies of this row's entry q into stage st: the column block and every applied
  // factor block (16-byte pieces where the alignment allows: f blocks when pb.vec, factor
  // blocks for deg 2 and 4, whose P x P blocks are whole 16-byte multiples at aligned offsets)
  auto issue = [&](long long q, int st) {
    const int e = pb.ent[q];
    const int j = e >> 4, t = e & 15;
    const unsigned act = pb.active[t];
    const T* src = f + static_cast<size_t>(j) * B;
    T* dst = stage + st * kStageVals + so;
    constexpr int V = 16 / static_cast<int>(sizeof(T));
    if (pb.vec) {
      for (int k = sl * V; k < B; k += L * V) cp_async16(dst + k, src + k);
    } else {
      for (int k = sl; k < B; k += L) cp_async_elem(dst + k, src + k);
    }
    T* ad = amat + st * kAmatVals + ao;
    const long long* ab = abase + sub * TD + t * D;
    if constexpr (PP % V == 0) {
      constexpr int PV = PP / V;  // 16-byte pieces per factor block
      for (int k = sl; k < D * PV; k += L) {
        const int m = k / PV, r = (k - m * PV) * V;
        if ((act >> m) & 1u) cp_async16(ad + m * PP + r, ops + ab[m] + static_cast<long long>(pb.idx1d[j * D + m]) * PP + r);
      }
    } else {
      for (int k = sl; k < D * PP; k += L) {
        const int m = k / PP, r = k - m * PP;
        if ((act >> m) & 1u) cp_async_elem(ad + m * PP + r, ops + ab[m] + static_cast<long long>(pb.idx1d[j * D + m]) * PP + r);
      }
    }
    return act;
  };
  T acc[MAXE], cmp[MAXE];
#pragma unroll
  for (int k = 0; k < MAXE; ++k) acc[k] = cmp[k] = T(0);
  const long long q0 = on ? pb.row_ptr[row] : 0, q1 = on ? pb.row_ptr[row + 1] : 0;
  // the rows' entry counts may differ: the warp runs to the longest, each row's lanes idle
  // past their own end (the batch's all-pairs rows all have N * T entries)
  long long n = q1 - q0;
  for (int off = L; off < 32; off <<= 1) n = max(n, __shfl_xor_sync(0xffffffffu, n, off));
  // entries q0 .. q0+S-2 in flight first (one commit group each, empty past the row's end)
  for (int k = 0; k < S - 1; ++k) {
    if (q0 + k < q1) {
      const unsigned a0 = issue(q0 + k, k);
      if (sl == 0) acts[k * R + sub] = a0;
    }
    cp_async_commit();
  }
  for (long long kq = 0; kq < n; ++kq) {
    const long long q = q0 + kq;
    const int cur = static_cast<int>(kq % S);
    if (q + S - 1 < q1) {  // refill the stage consumed by entry q-1
      const int nx = (cur + S - 1) % S;
      const unsigned a1 = issue(q + S - 1, nx);
      if (sl == 0) acts[nx * R + sub] = a1;
    }
    cp_async_commit();
    cp_async_wait_pending<S - 1>();  // this lane's copies of entry q have landed
    __syncwarp();                    // ... and every lane's (and acts)
    const bool live = q < q1;        // this row still has entry q
    const unsigned act = live ? acts[cur * R + sub] : 0u;
    const T* in = stage + cur * kStageVals + so;
    const T* Am = amat + cur * kAmatVals + ao;
    int wsel = 0;
    int s = 1, sh = 0;  // stride P^(D-1-m) of dimension m; for P = 2, 4: s = 1 << sh
    for (int m = D - 1; m >= 0; --m, s *= P, sh += LG) {
      const bool applied = (act >> m) & 1u;
      if (!__any_sync(0xffffffffu, applied)) continue;
      T A[PP];
      if constexpr (sizeof(T) == 4 && P == 4) {  // four 16-byte shared loads
#pragma unroll
        for (int r = 0; r < 4; ++r) {
          const float4 v = reinterpret_cast<const float4*>(Am + m * PP)[r];
          A[4 * r] = v.x;
          A[4 * r + 1] = v.y;
          A[4 * r + 2] = v.z;
          A[4 * r + 3] = v.w;
        }
      } else {
#pragma unroll
        for (int r = 0; r < PP; ++r) A[r] = Am[m * PP + r];
      }
      T* out = work + wsel * kStageVals + so;
      // fi / s without a division for deg 3 (s = 3^k): fi * ceil(2^16 / s) >> 16, exact for
      // fi < 256 and s <= 81 (checked exhaustively); deg 1 has s = 1
      const unsigned rs = P == 3 ? c_recip3[D - 1 - m] : 65536u;
      if (applied) {
        for (int fi = sl; fi < B / P; fi += L) {
          int hi, lo;
          if constexpr (LG > 0) {
            hi = fi >> sh;
            lo = fi & (s - 1);
          } else {
            hi = static_cast<int>((static_cast<unsigned>(fi) * rs) >> 16);
            lo = fi - hi * s;
          }
          const int base = hi * s * P + lo;
          T x[P];
#pragma unroll
          for (int b = 0; b < P; ++b) x[b] = in[base + b * s];
#pragma unroll
          for (int a = 0; a < P; ++a) {
            T sum = A[a * P] * x[0];
#pragma unroll
            for (int b = 1; b < P; ++b) sum = fma(A[a * P + b], x[b], sum);
            out[base + a * s] = sum;
          }
        }
      }
      __syncwarp();
      if (applied) {
        in = out;
        wsel ^= 1;
      }
    }
    if (live) {
#pragma unroll
      for (int k = 0; k < MAXE; ++k) {
        const int idx = sl + L * k;
        if (idx < B) {
          if (KAHAN) {
            const T yv = in[idx] - cmp[k];
            const T tt = acc[k] + yv;
            cmp[k] = (tt - acc[k]) - yv;
            acc[k] = tt;
          } else {
            acc[k] += in[idx];
          }
        }
      }
    }
    __syncwarp();  // stage cur is refilled by the next iteration's copies
  }
  if (on) {
    T* yr = y + static_cast<size_t>(row) * B;
#pragma unroll
    for (int k = 0; k < MAXE; ++k) {
      const int idx = sl + L * k;
      if (idx < B) yr[idx] = acc[k];
    }
  }
}

template <typename T, int P>
__device__ __forceinline__ void rows_deg(const BatchProblem& pb, int row, int nr, int R, unsigned char* wsm, int lane) {
  if (R == 4)
    warp_rows<T, P, 4>(pb, row, nr, wsm, lane);
  else if (R == 2)
    warp_rows<T, P, 2>(pb, row, nr, wsm, lane);
  else
    warp_rows<T, P, 1>(pb, row, nr, wsm, lane);
}

template <typename T>
__global__ void k_batch(const BatchProblem* __restrict__ probs, const BatchItem* __restrict__ items, int nitems,
                        int rows_per_item, int* counter) {
  extern __shared__ __align__(16) unsigned char batch_smem[];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  unsigned char* wsm = batch_smem + warp * warp_smem_bytes<T>();
  while (true) {
    int it = 0;
    if (lane == 0) it = atomicAdd(counter, 1);
    it = __shfl_sync(0xffffffffu, it, 0);
    if (it >= nitems) break;
    const BatchItem w = items[it];
    const BatchProblem pb = probs[w.prob];
    const int r1 = min(pb.N, w.row + rows_per_item);
    const int R = min(pb.R, rows_per_item);
    for (int row = w.row; row < r1; row += R) {
      const int nr = min(R, r1 - row);
      switch (pb.P) {
        case 1: rows_deg<T, 1>(pb, row, nr, R, wsm, lane); break;
        case 2: rows_deg<T, 2>(pb, row, nr, R, wsm, lane); break;
        case 3: rows_deg<T, 3>(pb, row, nr, R, wsm, lane); break;
        case 4: rows_deg<T, 4>(pb, row, nr, R, wsm, lane); break;
        default: break;  // rejected at batch creation
      }
    }
  }
}

}  // namespace
}  // namespace asg

struct asg_batch {
  std::vector<asg_plan*> plans;
  std::vector<asg::BatchProblem> probs;  // host copy (pointers filled per precision)
  asg::BatchProblem* d_probs = nullptr;
  asg::BatchItem* d_items[3] = {nullptr, nullptr, nullptr};  // per rows_per_item choice
  int nitems[3] = {0, 0, 0};
  int* d_counter = nullptr;
  int wpb = 4;          // tuned warps per CTA
  int rpi_choice = 0;   // tuned rows per item (index into kRowsPerItem)
  int io_set = 0;       // bit 0: FP64 io set, bit 1: FP32 io set
  std::vector<const void*> f64, f32;
  std::vector<void*> y64, y32;
  double flops = 0;
};

namespace {
constexpr int kRowsPerItem[3] = {1, 2, 4};

asg_status upload_probs(asg_batch* b, bool f32) {
  const size_t es = f32 ? sizeof(float) : sizeof(double);
  for (size_t k = 0; k < b->probs.size(); ++k) {
    b->probs[k].f = f32 ? b->f32[k] : b->f64[k];
    b->probs[k].y = f32 ? b->y32[k] : b->y64[k];
    b->probs[k].vec = (reinterpret_cast<uintptr_t>(b->probs[k].f) % 16 == 0 && (b->probs[k].B * es) % 16 == 0) ? 1 : 0;
  }
  ASG_CUDA(cudaMemcpy(b->d_probs, b->probs.data(), b->probs.size() * sizeof(asg::BatchProblem),
                      cudaMemcpyHostToDevice));
  return ASG_OK;
}
}  // namespace

using asg::fail;

extern "C" {

asg_status asg_batch_create(asg_plan* const* plans, int count, asg_batch** out) {
  if (!plans || !out || count < 1) return fail(ASG_ERR_INVALID, "batch_create: bad arguments");
  *out = nullptr;
  for (int k = 0; k < count; ++k) ASG_NOT_SLICE(plans[k], "batch_create");
  asg_batch* b = new (std::nothrow) asg_batch;
  if (!b) return fail(ASG_ERR_NOMEM, "batch_create: out of host memory");
  struct Cost {
    double c;
    int prob, row;
  };
  std::vector<Cost> rows;
  for (int k = 0; k < count; ++k) {
    asg_plan* p = plans[k];
    if (!p) {
      delete b;
      return fail(ASG_ERR_INVALID, "batch_create: plan %d is NULL", k);
    }
    if (p->B > 256 || p->P > 4) {
      delete b;
      return fail(ASG_ERR_UNSUPPORTED, "batch_create: plan %d has deg^d=%d (batch rows need <= 256, deg <= 4)", k, p->B);
    }
    b->plans.push_back(p);
    asg::BatchProblem pb{};
    pb.ops64 = p->d_ops64;
    pb.ops32 = p->d_ops32;
    pb.op_off = p->d_op_off;
    pb.op_nb = p->d_op_nb;
    pb.idx1d = p->d_idx1d;
    pb.row_ptr = p->d_row_ptr;
    pb.ent = p->d_ent;
    pb.active = p->d_active;
    pb.N = p->N;
    pb.D = p->D;
    pb.B = p->B;
    pb.P = p->P;
    pb.T = p->T;
    // rows side by side: each row's block-base table (T*D), stage (B) and factor blocks
    // (D*deg^2) must fit the warp's buffers, the stages' masks (kBatchStages*R) its header
    pb.R = 1;
    for (int r = 4; r > 1; r /= 2)
      if (r * p->T * p->D <= asg::kMaxTerms * asg::kMaxDims && r * p->B <= asg::kStageVals &&
          r * p->D * p->P * p->P <= asg::kAmatVals && r * asg::kBatchStages <= 16) {
        pb.R = r;
        break;
      }
    int sd = 1;
    for (int m = p->D - 1; m >= 0; --m) {
      pb.stride[m] = sd;
      sd *= p->P;
    }
    b->probs.push_back(pb);
    b->flops += p->flops_exec;
    double pd1 = 1.0;
    for (int q = 0; q <= p->D; ++q) pd1 *= p->P;
    for (int i = 0; i < p->N; ++i) {
      double c = 0;
      for (long long q = p->row_ptr[i]; q < p->row_ptr[i + 1]; ++q)
        c += 2.0 * pd1 * (1 + __builtin_popcount(p->active[p->ent[q] & 15]));
      rows.push_back({c, k, i});
    }
  }
  b->f64.assign(count, nullptr);
  b->f32.assign(count, nullptr);
  b->y64.assign(count, nullptr);
  b->y32.assign(count, nullptr);
  cudaError_t e = cudaMalloc(reinterpret_cast<void**>(&b->d_probs), count * sizeof(asg::BatchProblem));
  if (e == cudaSuccess) e = cudaMalloc(reinterpret_cast<void**>(&b->d_counter), sizeof(int));
  for (int c = 0; c < 3 && e == cudaSuccess; ++c) {
    // items of kRowsPerItem[c] consecutive rows, most expensive first
    std::vector<std::pair<double, asg::BatchItem>> its;
    for (size_t q = 0; q < rows.size();) {
      const int prob = rows[q].prob;
      double cost = 0;
      const int r0 = rows[q].row;
      int n = 0;
      while (q < rows.size() && rows[q].prob == prob && n < kRowsPerItem[c]) {
        cost += rows[q].c;
        ++q;
        ++n;
      }
      its.push_back({cost, {prob, r0}});
    }
    std::stable_sort(its.begin(), its.end(), [](const auto& x, const auto& y) { return x.first > y.first; });
    std::vector<asg::BatchItem> v;
    for (auto& x : its) v.push_back(x.second);
    b->nitems[c] = static_cast<int>(v.size());
    e = cudaMalloc(reinterpret_cast<void**>(&b->d_items[c]), v.size() * sizeof(asg::BatchItem));
    if (e == cudaSuccess) e = cudaMemcpy(b->d_items[c], v.data(), v.size() * sizeof(asg::BatchItem), cudaMemcpyHostToDevice);
  }
  if (e != cudaSuccess) {
    asg_status st = asg::cuda_fail(e, "batch_create upload");
    asg_batch_destroy(b);
    return st;
  }
  *out = b;
  return ASG_OK;
}

asg_status asg_batch_destroy(asg_batch* b) {
  if (!b) return ASG_OK;
  cudaFree(b->d_probs);
  cudaFree(b->d_counter);
  for (auto* p : b->d_items) cudaFree(p);
  delete b;
  return ASG_OK;
}

asg_status asg_batch_set_io_f64(asg_batch* b, const double* const* f, double* const* y) {
  if (!b || !f || !y) return fail(ASG_ERR_INVALID, "batch_set_io: NULL argument");
  for (size_t k = 0; k < b->plans.size(); ++k) {
    if (!f[k] || !y[k] || f[k] == y[k]) return fail(ASG_ERR_INVALID, "batch_set_io: bad buffers for problem %zu", k);
    b->f64[k] = f[k];
    b->y64[k] = y[k];
  }
  b->io_set |= 1;
  return ASG_OK;
}

asg_status asg_batch_set_io_f32(asg_batch* b, const float* const* f, float* const* y) {
  if (!b || !f || !y) return fail(ASG_ERR_INVALID, "batch_set_io: NULL argument");
  for (size_t k = 0; k < b->plans.size(); ++k) {
    if (!f[k] || !y[k] || f[k] == y[k]) return fail(ASG_ERR_INVALID, "batch_set_io: bad buffers for problem %zu", k);
    b->f32[k] = f[k];
    b->y32[k] = y[k];
  }
  b->io_set |= 2;
  return ASG_OK;
}

// Uploads the problem table for the precision (synchronous); apply then only launches.
asg_status asg_batch_prepare(asg_batch* b, int precision) {
  if (!b) return fail(ASG_ERR_INVALID, "batch_prepare: NULL batch");
  const bool f32 = precision == 1;
  if (!(b->io_set & (f32 ? 2 : 1))) return fail(ASG_ERR_INVALID, "batch_prepare: buffers not set for this precision");
  return upload_probs(b, f32);
}

asg_status asg_batch_apply(asg_batch* b, int precision, void* stream) {
  if (!b) return fail(ASG_ERR_INVALID, "batch_apply: NULL batch");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  ASG_CUDA(cudaMemsetAsync(b->d_counter, 0, sizeof(int), s));
  const int c = b->rpi_choice;
  const int grid = 152 * (b->wpb == 4 ? 8 : 4);
  if (precision == 1) {
    static bool done = false;  // opt in once to the largest request (8 warps per CTA)
    if (!done) {
      ASG_CUDA(cudaFuncSetAttribute(asg::k_batch<float>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    static_cast<int>(8 * asg::warp_smem_bytes<float>())));
      done = true;
    }
    asg::k_batch<float><<<grid, b->wpb * 32, b->wpb * asg::warp_smem_bytes<float>(), s>>>(
        b->d_probs, b->d_items[c], b->nitems[c], kRowsPerItem[c], b->d_counter);
  } else {
    static bool done = false;
    if (!done) {
      ASG_CUDA(cudaFuncSetAttribute(asg::k_batch<double>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    static_cast<int>(8 * asg::warp_smem_bytes<double>())));
      done = true;
    }
    asg::k_batch<double><<<grid, b->wpb * 32, b->wpb * asg::warp_smem_bytes<double>(), s>>>(
        b->d_probs, b->d_items[c], b->nitems[c], kRowsPerItem[c], b->d_counter);
  }
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? ASG_OK : asg::cuda_fail(e, "batch launch");
}

asg_status asg_batch_tune(asg_batch* b, int precision, void* stream, float* best_ms) {
  if (!b) return fail(ASG_ERR_INVALID, "batch_tune: NULL batch");
  asg_status st = asg_batch_prepare(b, precision);
  if (st) return st;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  cudaEvent_t e0, e1;
  ASG_CUDA(cudaEventCreate(&e0));
  ASG_CUDA(cudaEventCreate(&e1));
  float best = 1e30f;
  int bw = 4, bc = 0;
  for (int wpb : {4, 8})
    for (int c = 0; c < 3; ++c) {
      b->wpb = wpb;
      b->rpi_choice = c;
      if ((st = asg_batch_apply(b, precision, stream))) return st;  // warm-up
      ASG_CUDA(cudaEventRecord(e0, s));
      for (int r = 0; r < 3; ++r)
        if ((st = asg_batch_apply(b, precision, stream))) return st;
      ASG_CUDA(cudaEventRecord(e1, s));
      ASG_CUDA(cudaEventSynchronize(e1));
      float ms = 0;
      ASG_CUDA(cudaEventElapsedTime(&ms, e0, e1));
      if (ms < best) {
        best = ms;
        bw = wpb;
        bc = c;
      }
    }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  b->wpb = bw;
  b->rpi_choice = bc;
  if (best_ms) *best_ms = best / 3;
  return ASG_OK;
}

asg_status asg_batch_configure(asg_batch* b, int warps_per_cta, int rows_per_item) {
  if (!b) return fail(ASG_ERR_INVALID, "batch_configure: NULL batch");
  if (warps_per_cta != 4 && warps_per_cta != 8)
    return fail(ASG_ERR_INVALID, "batch_configure: warps_per_cta=%d (4 or 8)", warps_per_cta);
  int c = -1;
  for (int k = 0; k < 3; ++k)
    if (kRowsPerItem[k] == rows_per_item) c = k;
  if (c < 0) return fail(ASG_ERR_INVALID, "batch_configure: rows_per_item=%d (1, 2 or 4)", rows_per_item);
  b->wpb = warps_per_cta;
  b->rpi_choice = c;
  return ASG_OK;
}

asg_status asg_batch_info(const asg_batch* b, int* warps_per_cta, int* rows_per_item, double* flops) {
  if (!b) return fail(ASG_ERR_INVALID, "batch_info: NULL batch");
  if (warps_per_cta) *warps_per_cta = b->wpb;
  if (rows_per_item) *rows_per_item = kRowsPerItem[b->rpi_choice];
  if (flops) *flops = b->flops;
  return ASG_OK;
}

}  // extern "C"
