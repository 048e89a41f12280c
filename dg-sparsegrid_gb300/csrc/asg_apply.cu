// Operator application y = A*f over the sparse-grid element pairs (apply_A.m:102-236).
//
// Row-stationary: a team of threads (one warp, or one CTA for large element blocks) owns an
// output element i, walks its work entries (column element j, term t), applies the term's
// Kronecker factors A_{t,m}[I_m(i), J_m(j)] to f_j as a chain of mode products (fastest
// dimension first, as kronmult{d}.m's method-1 recursion does), and accumulates in
// registers.  Each y block is written exactly once: no atomics, bitwise deterministic.
// FP32 accumulation across the column reduction is Kahan-compensated.
#include <cstdio>

#include <type_traits>

#include "asg_internal.h"
#include "asg_pipe.cuh"
#include "asg_rows.cuh"

namespace asg {
namespace {

// P contiguous values with the widest aligned vector access the element type allows.
template <typename T, int P>
struct Row {
  T v[P];
  __device__ __forceinline__ void load(const T* p) {
#pragma unroll
    for (int i = 0; i < P; ++i) v[i] = p[i];
  }
  __device__ __forceinline__ void store(T* p) const {
#pragma unroll
    for (int i = 0; i < P; ++i) p[i] = v[i];
  }
};
template <>
struct Row<float, 4> {
  float v[4];
  __device__ __forceinline__ void load(const float* p) {
    const float4 q = *reinterpret_cast<const float4*>(p);
    v[0] = q.x; v[1] = q.y; v[2] = q.z; v[3] = q.w;
  }
  __device__ __forceinline__ void store(float* p) const {
    *reinterpret_cast<float4*>(p) = make_float4(v[0], v[1], v[2], v[3]);
  }
};
template <>
struct Row<double, 4> {
  double v[4];
  __device__ __forceinline__ void load(const double* p) {
    const double2 a = reinterpret_cast<const double2*>(p)[0];
    const double2 b = reinterpret_cast<const double2*>(p)[1];
    v[0] = a.x; v[1] = a.y; v[2] = b.x; v[3] = b.y;
  }
  __device__ __forceinline__ void store(double* p) const {
    reinterpret_cast<double2*>(p)[0] = make_double2(v[0], v[1]);
    reinterpret_cast<double2*>(p)[1] = make_double2(v[2], v[3]);
  }
};

// Cooperative copy of n values (16-byte vectors when both ends allow it).
template <typename T>
__device__ __forceinline__ void team_copy(T* dst, const T* src, int n, int rank, int size) {
  constexpr int V = 16 / sizeof(T);
  if ((n % V) == 0 && ((reinterpret_cast<uintptr_t>(src) | reinterpret_cast<uintptr_t>(dst)) & 15) == 0) {
    const int4* s4 = reinterpret_cast<const int4*>(src);
    int4* d4 = reinterpret_cast<int4*>(dst);
    for (int k = rank; k < n / V; k += size) d4[k] = s4[k];
  } else {
    for (int k = rank; k < n; k += size) dst[k] = src[k];
  }
}

// One mode product of the chain on an element block held in shared memory:
// out[.., a, ..] = sum_b A[a][b] * in[.., b, ..] along dimension m (stride s).
// Fibers are numbered fi = hi * s + lo (lo < s); for a power-of-two degree s is a power of two
// and the split takes a shift and a mask instead of an integer division.  In FP32 with
// deg <= 4 a thread takes two fibers at once (fi and fi + size) on the paired FMA; every output
// sees the scalar loop's operations in its order (a product, then fused multiply-adds), so
// the result is bitwise the same.
template <typename T, int P>
__device__ __forceinline__ void mode_pass(const T* __restrict__ in, T* __restrict__ out, const T* A, int B, int s,
                                          int rank, int size) {
  const int nf = B / P;
  constexpr bool POW2 = (P & (P - 1)) == 0;
  const int sh = POW2 ? __ffs(s) - 1 : 0;
  auto fiber_base = [&](int fi) {
    if constexpr (POW2) {
      return (((fi >> sh) * P) << sh) + (fi & (s - 1));
    } else {
      const int hi = fi / s;
      return hi * s * P + (fi - hi * s);
    }
  };
  int fi = rank;
  if constexpr (sizeof(T) == 4 && P <= 4) {
    float2 A2[P * P];
#pragma unroll
    for (int r = 0; r < P * P; ++r) A2[r] = make_float2(A[r], A[r]);
    for (; fi + size < nf; fi += 2 * size) {
      const int b0 = fiber_base(fi), b1 = fiber_base(fi + size);
      float2 x2[P];
#pragma unroll
      for (int b = 0; b < P; ++b) x2[b] = make_float2(in[b0 + b * s], in[b1 + b * s]);
#pragma unroll
      for (int a = 0; a < P; ++a) {
        float2 sum = __fmul2_rn(A2[a * P], x2[0]);
#pragma unroll
        for (int b = 1; b < P; ++b) sum = __ffma2_rn(A2[a * P + b], x2[b], sum);
        out[b0 + a * s] = sum.x;
        out[b1 + a * s] = sum.y;
      }
    }
  }
  for (; fi < nf; fi += size) {
    const int base = fiber_base(fi);
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

// ---------------------------------------------------------------------------------------
// Chain kernel, one warp per output element (element blocks of at most 256 values).
// ---------------------------------------------------------------------------------------
template <typename T, int P, bool KAHAN>
__global__ void __launch_bounds__(128) k_chain_warp(ApplyArgs<T> a) {
  constexpr int MAXE = 8;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
  const int wpb = blockDim.x >> 5;
  const int B = a.B, D = a.D;
  const int Bpad = (B + 3) & ~3;
  T* buf0 = reinterpret_cast<T*>(smem_raw) + static_cast<size_t>(warp) * 2 * Bpad;
  T* buf1 = buf0 + Bpad;
  for (int row = blockIdx.x * wpb + warp; row < a.N; row += gridDim.x * wpb) {
    T acc[MAXE], cmp[MAXE];
#pragma unroll
    for (int k = 0; k < MAXE; ++k) acc[k] = cmp[k] = T(0);
    int ii[kMaxDims];
    for (int m = 0; m < D; ++m) ii[m] = a.idx1d[row * D + m];
    const long long q1 = a.row_ptr[row + 1];
    for (long long q = a.row_ptr[row]; q < q1; ++q) {
      const int e = a.ent[q];
      const int j = e >> 4;
      const int t = e & 15;
      const unsigned act = a.active[t];
      team_copy(buf0, a.f + static_cast<size_t>(j) * B, B, lane, 32);
      __syncwarp();
      T* in = buf0;
      T* out = buf1;
      for (int m = D - 1; m >= 0; --m) {
        if (!((act >> m) & 1u)) continue;
        const int tm = t * D + m;
        const T* Ag = a.ops + a.op_off[tm] +
                      (static_cast<long long>(ii[m]) * a.op_nb[tm] + a.idx1d[j * D + m]) * (P * P);
        T A[P * P];
#pragma unroll
        for (int r = 0; r < P * P; ++r) A[r] = Ag[r];
        mode_pass<T, P>(in, out, A, B, a.stride[m], lane, 32);
        __syncwarp();
        T* tmp = in;
        in = out;
        out = tmp;
      }
#pragma unroll
      for (int k = 0; k < MAXE; ++k) {
        const int idx = lane + 32 * k;
        if (idx < B) acc_add(acc[k], cmp[k], in[idx], KAHAN);
      }
      __syncwarp();
    }
    T* yr = a.y + static_cast<size_t>(row) * B;
#pragma unroll
    for (int k = 0; k < MAXE; ++k) {
      const int idx = lane + 32 * k;
      if (idx < B) yr[idx] = acc[k];
    }
  }
}

template <typename T, int P, int MAXO, bool KAHAN>
__global__ void __launch_bounds__(128) k_single_small(ApplyArgs<T> a) {
  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
  const int wpb = blockDim.x >> 5;
  const SmallLane<MAXO> sl = small_lane<T, P, MAXO>(a, lane);
  for (int row = blockIdx.x * wpb + warp; row < a.N; row += gridDim.x * wpb) small_row<T, P, MAXO, KAHAN>(a, row, sl);
}

// Fiber-per-lane variant for P <= 4 (see fiber_entry), one CTA of WR warps per output
// element: warp w takes the row's entries w Gf + g, (w + WR) Gf + g, ... (g its lane group),
// writes its partial block to shared memory, and the CTA adds the WR partials in warp order
// (deterministic) -- WR times the parallelism of a warp per row, for the small element
// counts these plans have (hundreds to a few thousand rows).
template <typename T, int P, int MAXF, bool KAHAN, int WR>
__global__ void __launch_bounds__(32 * WR) k_single_fiber_split(ApplyArgs<T> a) {
  __shared__ __align__(16) T part[WR][256];
  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
  const int B = a.B;
  const FiberLane<MAXF> fl = fiber_lane<T, P, MAXF>(a, lane);
  for (int row = blockIdx.x; row < a.N; row += gridDim.x) {
    fiber_chunk<T, P, MAXF, KAHAN>(a, a.f, a.row_ptr[row], a.row_ptr[row + 1], fl, part[warp], warp * fl.Gf,
                                   WR * fl.Gf);
    __syncthreads();
    T* yr = a.y + static_cast<size_t>(row) * B;
    for (int e = threadIdx.x; e < B; e += 32 * WR) {
      T v = part[0][e];
#pragma unroll
      for (int w = 1; w < WR; ++w) v += part[w][e];
      yr[e] = v;
    }
    __syncthreads();
  }
}


// ---------------------------------------------------------------------------------------
// Chain kernel, one CTA per output element (element blocks up to 4096 values).
// ---------------------------------------------------------------------------------------
template <typename T, int P, bool KAHAN, int NT>
__global__ void __launch_bounds__(NT) k_chain_cta(ApplyArgs<T> a) {
  constexpr int MAXE = kMaxBlock / NT;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int tid = threadIdx.x;
  const int B = a.B, D = a.D;
  const int Bpad = (B + 3) & ~3;
  T* buf0 = reinterpret_cast<T*>(smem_raw);
  T* buf1 = buf0 + Bpad;
  T* blk = buf1 + Bpad;  // D*P*P operator blocks of the current entry
  for (int row = blockIdx.x; row < a.N; row += gridDim.x) {
    T acc[MAXE], cmp[MAXE];
#pragma unroll
    for (int k = 0; k < MAXE; ++k) acc[k] = cmp[k] = T(0);
    const long long q1 = a.row_ptr[row + 1];
    for (long long q = a.row_ptr[row]; q < q1; ++q) {
      const int e = a.ent[q];
      const int j = e >> 4;
      const int t = e & 15;
      const unsigned act = a.active[t];
      team_copy(buf0, a.f + static_cast<size_t>(j) * B, B, tid, NT);
      for (int idx = tid; idx < D * P * P; idx += NT) {
        const int m = idx / (P * P);
        if ((act >> m) & 1u) {
          const int tm = t * D + m;
          blk[idx] = a.ops[a.op_off[tm] +
                           (static_cast<long long>(a.idx1d[row * D + m]) * a.op_nb[tm] + a.idx1d[j * D + m]) * (P * P) +
                           (idx - m * P * P)];
        }
      }
      __syncthreads();
      T* in = buf0;
      T* out = buf1;
      for (int m = D - 1; m >= 0; --m) {
        if (!((act >> m) & 1u)) continue;
        T A[P * P];
#pragma unroll
        for (int r = 0; r < P * P; ++r) A[r] = blk[m * P * P + r];
        mode_pass<T, P>(in, out, A, B, a.stride[m], tid, NT);
        __syncthreads();
        T* tmp = in;
        in = out;
        out = tmp;
      }
#pragma unroll
      for (int k = 0; k < MAXE; ++k) {
        const int idx = tid + NT * k;
        if (idx < B) acc_add(acc[k], cmp[k], in[idx], KAHAN);
      }
      __syncthreads();
    }
    T* yr = a.y + static_cast<size_t>(row) * B;
#pragma unroll
    for (int k = 0; k < MAXE; ++k) {
      const int idx = tid + NT * k;
      if (idx < B) yr[idx] = acc[k];
    }
  }
}

// ---------------------------------------------------------------------------------------
// Single-mode fiber kernel.  Used when every term has exactly one non-identity factor
// (I x .. x D_k x .. x I, the shape of every advection/diffusion term once the mass
// factors are the identity) and the block is large (deg^d >= 32*deg^2).
//
// The CTA has B/P^2 threads; thread t owns the P x P output tile over dimensions (d-2, d-1)
// starting at t*P^2 (its "natural" tile).  Entries of a row are sorted by term.  For a term
// acting on dimension m the thread reads, straight from global memory, the P fibers along m
// that hit a P x P tile over (m, d-1) and contracts them with the P x P block in registers:
// 4-wide vector loads, P^3 FMAs per tile.  Terms on dimensions d-2 and d-1 land directly on
// the natural tile; the others are summed per term and moved to the natural tile through
// one shared-memory transpose.
// ---------------------------------------------------------------------------------------
template <typename T, int P, bool KAHAN>
__global__ void __launch_bounds__(256) k_single_mode(ApplyArgs<T> a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* scratch = reinterpret_cast<T*>(smem_raw);  // B values
  const int tid = threadIdx.x;
  const int B = a.B, D = a.D;
  const int row = blockIdx.x;
  if (row >= a.N) return;
  T nat[P][P], natc[P][P], g[P][P], gc[P][P];
#pragma unroll
  for (int r = 0; r < P; ++r)
#pragma unroll
    for (int c = 0; c < P; ++c) nat[r][c] = natc[r][c] = g[r][c] = gc[r][c] = T(0);

  int cur_m = -1;
  int base_g = 0, s_g = 0;
  const long long q0 = a.row_ptr[row], q1 = a.row_ptr[row + 1];
  for (long long q = q0; q <= q1; ++q) {
    int m = -1, j = 0, t = 0;
    if (q < q1) {
      const int e = a.ent[q];
      j = e >> 4;
      t = e & 15;
      m = __ffs(a.active[t]) - 1;
    }
    if (m != cur_m) {
      if (cur_m >= 0 && cur_m < D - 2) {
        // flush the per-term sum through shared memory onto the natural tiles
#pragma unroll
        for (int r = 0; r < P; ++r) {
          Row<T, P> rr;
#pragma unroll
          for (int c = 0; c < P; ++c) rr.v[c] = g[r][c];
          rr.store(scratch + base_g + r * s_g);
        }
        __syncthreads();
#pragma unroll
        for (int r = 0; r < P; ++r) {
          Row<T, P> rr;
          rr.load(scratch + tid * P * P + r * P);
#pragma unroll
          for (int c = 0; c < P; ++c) acc_add(nat[r][c], natc[r][c], rr.v[c], KAHAN);
        }
        __syncthreads();
      }
      cur_m = m;
      if (m >= 0) {
        // new term group: reset its sum and place this thread's tile over (m, d-1)
#pragma unroll
        for (int r = 0; r < P; ++r)
#pragma unroll
          for (int c = 0; c < P; ++c) g[r][c] = gc[r][c] = T(0);
        if (m < D - 1) {
          int pw = 1;
          for (int k = 0; k < D - 2 - m; ++k) pw *= P;
          const int lo = tid % pw, hi = tid / pw;
          s_g = a.stride[m];
          base_g = hi * s_g * P + lo * P;
        } else {
          s_g = P;
          base_g = tid * P * P;
        }
      }
    }
    if (m < 0) break;
    // P x P block of operator (t, m) at (I_m(row), J_m(j))
    const int tm = t * D + m;
    const T* Ag = a.ops + a.op_off[tm] +
                  (static_cast<long long>(a.idx1d[row * D + m]) * a.op_nb[tm] + a.idx1d[j * D + m]) * (P * P);
    T A[P][P];
#pragma unroll
    for (int r = 0; r < P; ++r) {
      Row<T, P> rr;
      rr.load(Ag + r * P);
#pragma unroll
      for (int c = 0; c < P; ++c) A[r][c] = rr.v[c];
    }
    const T* fj = a.f + static_cast<size_t>(j) * B + base_g;
    T x[P][P];
#pragma unroll
    for (int r = 0; r < P; ++r) {
      Row<T, P> rr;
      rr.load(fj + r * s_g);
#pragma unroll
      for (int c = 0; c < P; ++c) x[r][c] = rr.v[c];
    }
    if (m == D - 1) {
      // contraction along the contiguous index: out[r][a] = sum_b A[a][b] x[r][b]
#pragma unroll
      for (int r = 0; r < P; ++r)
#pragma unroll
        for (int aa = 0; aa < P; ++aa) {
          T s = A[aa][0] * x[r][0];
#pragma unroll
          for (int b = 1; b < P; ++b) s = fma(A[aa][b], x[r][b], s);
          acc_add(nat[r][aa], natc[r][aa], s, KAHAN);
        }
    } else {
      // contraction across rows: out[a][c] = sum_b A[a][b] x[b][c]
#pragma unroll
      for (int aa = 0; aa < P; ++aa)
#pragma unroll
        for (int c = 0; c < P; ++c) {
          T s = A[aa][0] * x[0][c];
#pragma unroll
          for (int b = 1; b < P; ++b) s = fma(A[aa][b], x[b][c], s);
          if (m == D - 2)
            acc_add(nat[aa][c], natc[aa][c], s, KAHAN);
          else
            acc_add(g[aa][c], gc[aa][c], s, KAHAN);
        }
    }
  }
  const size_t y0 = static_cast<size_t>(row) * B + tid * P * P;
  T* yr = a.y + y0;
#pragma unroll
  for (int r = 0; r < P; ++r) {
    Row<T, P> rr;
#pragma unroll
    for (int c = 0; c < P; ++c) rr.v[c] = minus_sub(nat[r][c], a.ysub, y0 + r * P + c);
    rr.store(yr + r * P);
  }
}

// ---------------------------------------------------------------------------------------
// Single-mode fiber kernel, TMA-pipelined (deg 4).
//
// Same thread/tile mapping as k_single_mode, but the operand blocks stream into shared
// memory with bulk asynchronous copies (cp.async.bulk, one elected thread, completion on an
// mbarrier with a transaction count): the column element's whole f block (deg^d values)
// plus its P x P operator block per work entry, S entries in flight.  The threads never
// wait on a global load; they wait on the stage's mbarrier (bounded: after ~2^31 cycles
// the CTA records ASG_ERR_TIMEOUT in the plan's status word and stops).  Per term group the
// products are summed in FP32 registers; groups are merged into the output tile with Kahan
// compensation.  FP32 products use the paired FMA (fma.rn.f32x2).
// ---------------------------------------------------------------------------------------
// g[a][c] += sum_b A[a][b] * x[b][c]   (contraction across the tile rows)
template <typename T>
__device__ __forceinline__ void tile_rows(T (&g)[4][4], const T* A, const T* xs, int s) {
#pragma unroll
  for (int b = 0; b < 4; ++b) {
    Row<T, 4> x;
    x.load(xs + b * s);
#pragma unroll
    for (int aa = 0; aa < 4; ++aa)
#pragma unroll
      for (int c = 0; c < 4; ++c) g[aa][c] = fma(A[aa * 4 + b], x.v[c], g[aa][c]);
  }
}
// g[r][a] += sum_b A[a][b] * x[r][b] with tile rows s apart
template <typename T>
__device__ __forceinline__ void tile_cols_s(T (&g)[4][4], const T* A, const T* xs, int s) {
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    Row<T, 4> x;
    x.load(xs + r * s);
#pragma unroll
    for (int aa = 0; aa < 4; ++aa)
#pragma unroll
      for (int b = 0; b < 4; ++b) g[r][aa] = fma(A[aa * 4 + b], x.v[b], g[r][aa]);
  }
}

__device__ __forceinline__ void consumer_sync() { asm volatile("bar.sync 1, 256;" ::: "memory"); }

// Base offset and row stride of a thread's 4 x 4 tile spanning dimensions (u, d-1) of a
// deg-4 block (dimension k has stride 4^(d-1-k)): the thread's other digits run over
// dimensions {0..d-2} \ {u}, the highest dimension fastest.  Shifts and masks only.
__device__ __forceinline__ void tile_place(int tid, int u, int D, int& base, int& s) {
  const int sh = 2 * (D - 2 - u);  // the digits below dimension u, 2 bits each
  s = 1 << (2 * (D - 1 - u));
  base = ((tid >> sh) * s + (tid & ((1 << sh) - 1))) * 4;
}

// Warp-specialised pipeline: warps 0..7 consume (256 threads, one P x P output tile each),
// warp 8 produces.  Stage st holds the column element's f block and its operator block;
// full[st] completes when both bulk copies land (transaction count), empty[st] when all 8
// consumer warps have released it.  A consumer releases a stage one entry late, so at a term
// group boundary the stage just consumed doubles as the transpose buffer (no separate
// scratch).  The natural output tile of a thread spans dimensions (d-3, d-1): consecutive
// threads sit 16 bytes apart in shared memory; terms on dimensions d-3 and d-1 accumulate
// straight into it, the others through the transpose.  FP32 operator blocks arrive with each
// column's values duplicated ((A0b,A0b,A1b,A1b), (A2b,A2b,A3b,A3b)), so the paired FMA takes
// an operator value pair and two neighbouring inputs along d-1 straight from shared memory;
// on dimension d-1 (the contraction runs along the float4) an input value is paired with
// itself instead.  Groups merge into the output tile with Kahan compensation (paired adds).
// With OWN the row's own f block stays resident: the row's diagonal entries, one per term,
// read it and copy only their operator block.  Rows launch longest first (row_order).
template <typename T, int S, int MINB, bool CSMEM, bool OWN>
__global__ void __launch_bounds__(288, MINB) k_single_tma(ApplyArgs<T> a) {
  constexpr int P = 4;
  constexpr bool F32 = sizeof(T) == 4;
  constexpr bool CS = F32 && CSMEM;  // FP32 compensation tile in shared memory (else registers)
  // operator block values per stage: FP32 32 (rows: duplicated columns (A0b,A0b,A1b,A1b),
  // (A2b,A2b,A3b,A3b); dimension d-1: columns (A0b,A1b,A2b,A3b) + padding), FP64 16
  constexpr int AB = F32 ? 32 : 16;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ int s_abort;
  const int tid = threadIdx.x;
  const int warp = tid >> 5, lane = tid & 31;
  const int B = a.B, D = a.D;
  const int SST = B + AB;
  T* stages = reinterpret_cast<T*>(smem_raw);
  // FP32: the Kahan compensation of the output tiles lives in shared memory (B values)
  float* comp = reinterpret_cast<float*>(stages + S * SST);
  // OWN: the row's own f block, resident for the whole row: the row's diagonal entries (one
  // per term) read it here and copy only their operator block
  T* own = reinterpret_cast<T*>(comp + (CS ? B : 0));
  uint64_t* full = reinterpret_cast<uint64_t*>(own + (OWN ? B : 0));
  uint64_t* empty = full + S;
  uint64_t* own_full = empty + S;
  const int row = a.row_order ? a.row_order[blockIdx.x] : blockIdx.x;
  const long long q0 = a.row_ptr[row];
  const int n = static_cast<int>(a.row_ptr[row + 1] - q0);
  const EntryDesc* ed = a.ed + q0;
  const uint32_t fbytes = static_cast<uint32_t>(B * sizeof(T)), abytes = AB * sizeof(T);
  const T* opsrc = F32 ? reinterpret_cast<const T*>(a.ops_pair) : a.ops;

  if (tid == 0) {
    s_abort = 0;
    for (int k = 0; k < S; ++k) {
      mbar_init(&full[k], 1);
      mbar_init(&empty[k], 8);
    }
    mbar_init(own_full, 1);
    mbar_fence_init();
  }
  __syncthreads();
  volatile int* abort_flag = &s_abort;

  if (warp == 8) {
    // ---------------- producer warp ----------------
    int kdone = 0;
    bool stop = false;
    if (OWN && lane == 0 && n > 0) {
      fence_proxy_async();
      mbar_expect_tx(own_full, fbytes);
      bulk_g2s(own, a.f + static_cast<size_t>(row) * B, fbytes, own_full);
    }
    for (int k0 = 0; k0 < n && !stop; k0 += 32) {
      EntryDesc mine{};
      if (k0 + lane < n) mine = ed[k0 + lane];
      const int cnt = min(32, n - k0);
      for (int l = 0; l < cnt; ++l) {
        const int j = __shfl_sync(0xffffffffu, mine.j, l);
        const long long aoff = __shfl_sync(0xffffffffu, mine.aoff, l);
        const int k = k0 + l;
        const int st = k % S;
        bool ok = true;
        if (k >= S) ok = mbar_wait_bounded(&empty[st], static_cast<uint32_t>(((k / S) - 1) & 1));
        if (!__all_sync(0xffffffffu, ok)) {
          if (lane == 0) *abort_flag = 1;
          stop = true;
          break;
        }
        if (lane == 0) {
          T* dst = stages + st * SST;
          const bool self = OWN && j == row;
          fence_proxy_async();
          mbar_expect_tx(&full[st], (self ? 0u : fbytes) + abytes);
          if (!self) bulk_g2s(dst, a.f + static_cast<size_t>(j) * B, fbytes, &full[st]);
          bulk_g2s(dst + B, opsrc + aoff * (AB / 16), abytes, &full[st]);
        }
        kdone = k + 1;
        __syncwarp();
      }
    }
    if (lane == 0) {
      if (*abort_flag) atomicExch(a.err, static_cast<int>(ASG_ERR_TIMEOUT));
      // every issued copy lands before the CTA's shared memory is released (bounded)
      for (int k = max(0, kdone - S); k < kdone; ++k) {
        const long long t0 = clock64();
        while (!mbar_test(&full[k % S], static_cast<uint32_t>((k / S) & 1)) && clock64() - t0 < (1LL << 28)) {
        }
      }
      if (OWN && n > 0) {
        const long long t0 = clock64();
        while (!mbar_test(own_full, 0u) && clock64() - t0 < (1LL << 28)) {
        }
      }
    }
    return;
  }

  // ---------------- consumer warps ----------------
  int nat_base, nat_s;
  tile_place(tid, D - 3, D, nat_base, nat_s);
  int cur_m = -1, base_g = 0, s_g = 0, pend = -1;
  bool direct = false, gave_up = false, own_ready = false;
  int mlane = -1;
  unsigned selfmask = 0;
  // FP32: paired state, compensation in registers or shared memory; FP64: scalar state
  F32Tile g32;  // a group's sums (rows along its dimension, column pairs along d-1)
  F32Tile n32, c32;
  T g[P][P], nat[P][P];
#pragma unroll
  for (int r = 0; r < P; ++r) {
#pragma unroll
    for (int cp = 0; cp < 2; ++cp) g32.v[r][cp] = n32.v[r][cp] = c32.v[r][cp] = make_float2(0.f, 0.f);
#pragma unroll
    for (int c = 0; c < P; ++c) g[r][c] = nat[r][c] = T(0);
    if constexpr (CS) *reinterpret_cast<float4*>(comp + nat_base + r * nat_s) = make_float4(0.f, 0.f, 0.f, 0.f);
  }
  // Kahan-merge a tile row pair into the output tile (compensation where this variant keeps it)
  auto merge_row = [&](int r, float2 v0, float2 v1) {
    if constexpr (CS) {
      float4* cq = reinterpret_cast<float4*>(comp + nat_base + r * nat_s);
      const float4 c4 = *cq;
      float2 c0 = make_float2(c4.x, c4.y), c1 = make_float2(c4.z, c4.w);
      kahan2(n32.v[r][0], c0, v0);
      kahan2(n32.v[r][1], c1, v1);
      *cq = make_float4(c0.x, c0.y, c1.x, c1.y);
    } else {
      kahan2(n32.v[r][0], c32.v[r][0], v0);
      kahan2(n32.v[r][1], c32.v[r][1], v1);
    }
  };
  for (int k = 0; k <= n; ++k) {
    int m = -1;
    const int st = k % S;
    if (k < n) {
      if ((k & 31) == 0) {
        const bool in = k + lane < n;
        mlane = in ? ed[k + lane].m : -1;
        selfmask = __ballot_sync(0xffffffffu, OWN && in && ed[k + lane].j == row);
      }
      // the dimension comes from the immutable descriptors: consumer control flow (and every
      // named barrier below) is uniform even after a timeout; later waits are skipped
      m = __shfl_sync(0xffffffffu, mlane, k & 31);
      if (!gave_up) {
        bool ok = mbar_wait_bounded(&full[st], static_cast<uint32_t>((k / S) & 1));
        if (ok && !own_ready && ((selfmask >> (k & 31)) & 1u)) {
          ok = mbar_wait_bounded(own_full, 0u);
          own_ready = true;
        }
        // a warp that gave up on a stage never releases a stage again: the producer then
        // cannot re-arm a stage whose copy may still be in flight; its own bounded wait on
        // the empty barrier expires and it waits for its issued copies before exiting
        if (!__all_sync(0xffffffffu, ok)) {
          gave_up = true;
          *abort_flag = 1;
        }
      }
    }
    if (m != cur_m) {
      if (direct) {
        if constexpr (F32) {
#pragma unroll
          for (int r = 0; r < P; ++r) {
            const float4 v = f32_row(g32, r);
            merge_row(r, make_float2(v.x, v.y), make_float2(v.z, v.w));
          }
        } else {
#pragma unroll
          for (int r = 0; r < P; ++r)
#pragma unroll
            for (int c = 0; c < P; ++c) nat[r][c] += g[r][c];
        }
      } else if (cur_m >= 0) {
        // transpose the group's sums onto the natural tiles through the stage just consumed
        consumer_sync();
        T* scr = stages + pend * SST;
#pragma unroll
        for (int i = 0; i < P; ++i) {
          if constexpr (F32) {
            // rows of a group on dimension d-2 in a per-thread rotated order (bank-conflict free)
            const int r = (i + (cur_m == D - 2 ? (tid >> 1) & 3 : 0)) & 3;
            *reinterpret_cast<float4*>(scr + base_g + r * s_g) = f32_row_sel(g32, r);
          } else {
            const int r = i;
            Row<T, P> rr;
#pragma unroll
            for (int c = 0; c < P; ++c) rr.v[c] = g[r][c];
            rr.store(scr + base_g + r * s_g);
          }
        }
        consumer_sync();
#pragma unroll
        for (int r = 0; r < P; ++r) {
          if constexpr (F32) {
            const float4 v = *reinterpret_cast<const float4*>(scr + nat_base + r * nat_s);
            merge_row(r, make_float2(v.x, v.y), make_float2(v.z, v.w));
          } else {
            Row<T, P> rr;
            rr.load(scr + nat_base + r * nat_s);
#pragma unroll
            for (int c = 0; c < P; ++c) nat[r][c] += rr.v[c];
          }
        }
      }
      cur_m = m;
      if (m >= 0) {
#pragma unroll
        for (int r = 0; r < P; ++r) {
#pragma unroll
          for (int cp = 0; cp < 2; ++cp) g32.v[r][cp] = make_float2(0.f, 0.f);
#pragma unroll
          for (int c = 0; c < P; ++c) g[r][c] = T(0);
        }
        direct = (m == D - 1) || (m == D - 3);
        if (m == D - 1) {
          base_g = nat_base;
          s_g = nat_s;
        } else {
          tile_place(tid, m, D, base_g, s_g);
        }
      }
    }
    if (pend >= 0) {
      __syncwarp();
      if (lane == 0 && !gave_up) mbar_arrive(&empty[pend]);
      pend = -1;
    }
    if (m < 0) break;
    const T* sp = stages + st * SST;
    const T* xp = (((selfmask >> (k & 31)) & 1u) ? own : sp) + base_g;  // the column's f tile
    if constexpr (F32) {
      if (m == D - 1)
        f32_cols(g32, reinterpret_cast<const float*>(sp + B), reinterpret_cast<const float*>(xp), s_g);
      else
        f32_rows_rot(g32, reinterpret_cast<const float*>(sp + B), reinterpret_cast<const float*>(xp), s_g,
                     m == D - 2 ? (tid >> 1) & 3 : 0);
    } else {
      T A[P * P];
#pragma unroll
      for (int r = 0; r < P; ++r) {
        Row<T, P> rr;
        rr.load(sp + B + r * P);
#pragma unroll
        for (int c = 0; c < P; ++c) A[r * P + c] = rr.v[c];
      }
      if (m == D - 1)
        tile_cols_s<T>(g, A, xp, s_g);
      else
        tile_rows<T>(g, A, xp, s_g);
    }
    pend = st;
  }
  if (*abort_flag) return;  // y is undefined; the plan's status word reports the timeout
  const size_t y0 = static_cast<size_t>(row) * B + nat_base;
  T* yr = a.y + y0;
#pragma unroll
  for (int r = 0; r < P; ++r) {
    if constexpr (F32) {
      *reinterpret_cast<float4*>(reinterpret_cast<float*>(yr) + r * nat_s) =
          minus_sub4(make_float4(n32.v[r][0].x, n32.v[r][0].y, n32.v[r][1].x, n32.v[r][1].y),
                     reinterpret_cast<const float*>(a.ysub), y0 + r * nat_s);
    } else {
      Row<T, P> rr;
#pragma unroll
      for (int c = 0; c < P; ++c) rr.v[c] = minus_sub(nat[r][c], a.ysub, y0 + r * nat_s + c);
      rr.store(yr + r * nat_s);
    }
  }
}

// k_single_tma in FP32 with two output tiles per consumer thread: 4 consumer warps (128
// threads) and one producer warp.  Consumer thread t owns the tiles kind-3 threads t and t+128
// own, so every output value sees kind 3's operations in kind 3's order (the results are
// bitwise those of kind 3).  Per entry, the stage wait, the descriptor broadcast, the stage
// release and the operator block's shared loads are paid once for two tiles, and a term
// group's transpose synchronises 128 threads instead of 256.
__device__ __forceinline__ void consumer_sync_x2() { asm volatile("bar.sync 1, 128;" ::: "memory"); }

template <int S, int MINB>
__global__ void __launch_bounds__(160, MINB) k_single_tma_x2(ApplyArgs<float> a) {
  constexpr int P = 4, AB = 32, NCW = 4, NT = 2, HALF = 32 * NCW;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ int s_abort;
  const int tid = threadIdx.x;
  const int warp = tid >> 5, lane = tid & 31;
  const int B = a.B, D = a.D;
  const int SST = B + AB;
  float* stages = reinterpret_cast<float*>(smem_raw);
  float* own = stages + S * SST;  // the row's own f block (diagonal entries read it here)
  uint64_t* full = reinterpret_cast<uint64_t*>(own + B);
  uint64_t* empty = full + S;
  uint64_t* own_full = empty + S;
  const int row = a.row_order ? a.row_order[blockIdx.x] : blockIdx.x;
  const long long q0 = a.row_ptr[row];
  const int n = static_cast<int>(a.row_ptr[row + 1] - q0);
  const EntryDesc* ed = a.ed + q0;
  const uint32_t fbytes = static_cast<uint32_t>(B * sizeof(float)), abytes = AB * sizeof(float);

  if (tid == 0) {
    s_abort = 0;
    for (int k = 0; k < S; ++k) {
      mbar_init(&full[k], 1);
      mbar_init(&empty[k], NCW);
    }
    mbar_init(own_full, 1);
    mbar_fence_init();
  }
  __syncthreads();
  volatile int* abort_flag = &s_abort;

  if (warp == NCW) {
    // ---------------- producer warp (as in k_single_tma) ----------------
    int kdone = 0;
    bool stop = false;
    if (lane == 0 && n > 0) {
      fence_proxy_async();
      mbar_expect_tx(own_full, fbytes);
      bulk_g2s(own, a.f + static_cast<size_t>(row) * B, fbytes, own_full);
    }
    for (int k0 = 0; k0 < n && !stop; k0 += 32) {
      EntryDesc mine{};
      if (k0 + lane < n) mine = ed[k0 + lane];
      const int cnt = min(32, n - k0);
      for (int l = 0; l < cnt; ++l) {
        const int j = __shfl_sync(0xffffffffu, mine.j, l);
        const long long aoff = __shfl_sync(0xffffffffu, mine.aoff, l);
        const int k = k0 + l;
        const int st = k % S;
        bool ok = true;
        if (k >= S) ok = mbar_wait_bounded(&empty[st], static_cast<uint32_t>(((k / S) - 1) & 1));
        if (!__all_sync(0xffffffffu, ok)) {
          if (lane == 0) *abort_flag = 1;
          stop = true;
          break;
        }
        if (lane == 0) {
          float* dst = stages + st * SST;
          const bool self = j == row;
          fence_proxy_async();
          mbar_expect_tx(&full[st], (self ? 0u : fbytes) + abytes);
          if (!self) bulk_g2s(dst, a.f + static_cast<size_t>(j) * B, fbytes, &full[st]);
          bulk_g2s(dst + B, a.ops_pair + 2 * aoff, abytes, &full[st]);
        }
        kdone = k + 1;
        __syncwarp();
      }
    }
    if (lane == 0) {
      if (*abort_flag) atomicExch(a.err, static_cast<int>(ASG_ERR_TIMEOUT));
      // every issued copy lands before the CTA's shared memory is released (bounded)
      for (int k = max(0, kdone - S); k < kdone; ++k) {
        const long long t0 = clock64();
        while (!mbar_test(&full[k % S], static_cast<uint32_t>((k / S) & 1)) && clock64() - t0 < (1LL << 28)) {
        }
      }
      if (n > 0) {
        const long long t0 = clock64();
        while (!mbar_test(own_full, 0u) && clock64() - t0 < (1LL << 28)) {
        }
      }
    }
    return;
  }

  // ---------------- consumer warps: tiles tid and tid + 128 ----------------
  int nat_base[NT], base_g[NT], nat_s = 0, s_g = 0;
#pragma unroll
  for (int q = 0; q < NT; ++q) tile_place(tid + q * HALF, D - 3, D, nat_base[q], nat_s);
  // the d-2 rotation of kind-3 thread t+128 equals that of thread t
  const int rot = (tid >> 1) & 3;
  int cur_m = -1, pend = -1, mlane = -1;
  bool direct = false, gave_up = false, own_ready = false;
  unsigned selfmask = 0;
  F32Tile g32[NT];
  F32Tile n32[NT], c32[NT];
#pragma unroll
  for (int q = 0; q < NT; ++q)
#pragma unroll
    for (int r = 0; r < P; ++r)
#pragma unroll
      for (int cp = 0; cp < 2; ++cp) g32[q].v[r][cp] = n32[q].v[r][cp] = c32[q].v[r][cp] = make_float2(0.f, 0.f);

  for (int k = 0; k <= n; ++k) {
    int m = -1;
    const int st = k % S;
    if (k < n) {
      if ((k & 31) == 0) {
        const bool in = k + lane < n;
        mlane = in ? ed[k + lane].m : -1;
        selfmask = __ballot_sync(0xffffffffu, in && ed[k + lane].j == row);
      }
      m = __shfl_sync(0xffffffffu, mlane, k & 31);
      if (!gave_up) {
        bool ok = mbar_wait_bounded(&full[st], static_cast<uint32_t>((k / S) & 1));
        if (ok && !own_ready && ((selfmask >> (k & 31)) & 1u)) {
          ok = mbar_wait_bounded(own_full, 0u);
          own_ready = true;
        }
        if (!__all_sync(0xffffffffu, ok)) {
          gave_up = true;
          *abort_flag = 1;
        }
      }
    }
    if (m != cur_m) {
      if (direct) {
#pragma unroll
        for (int q = 0; q < NT; ++q)
#pragma unroll
          for (int r = 0; r < P; ++r) {
            const float4 v = f32_row(g32[q], r);
            kahan2(n32[q].v[r][0], c32[q].v[r][0], make_float2(v.x, v.y));
            kahan2(n32[q].v[r][1], c32[q].v[r][1], make_float2(v.z, v.w));
          }
      } else if (cur_m >= 0) {
        // transpose the group's sums onto the natural tiles through the stage just consumed
        consumer_sync_x2();
        float* scr = stages + pend * SST;
        const int rr = cur_m == D - 2 ? rot : 0;
#pragma unroll
        for (int q = 0; q < NT; ++q)
#pragma unroll
          for (int i = 0; i < P; ++i) {
            const int r = (i + rr) & 3;
            *reinterpret_cast<float4*>(scr + base_g[q] + r * s_g) = f32_row_sel(g32[q], r);
          }
        consumer_sync_x2();
#pragma unroll
        for (int q = 0; q < NT; ++q)
#pragma unroll
          for (int r = 0; r < P; ++r) {
            const float4 v = *reinterpret_cast<const float4*>(scr + nat_base[q] + r * nat_s);
            kahan2(n32[q].v[r][0], c32[q].v[r][0], make_float2(v.x, v.y));
            kahan2(n32[q].v[r][1], c32[q].v[r][1], make_float2(v.z, v.w));
          }
      }
      cur_m = m;
      if (m >= 0) {
#pragma unroll
        for (int q = 0; q < NT; ++q) zero_f32(g32[q]);
        direct = (m == D - 1) || (m == D - 3);
        if (m == D - 1) {
#pragma unroll
          for (int q = 0; q < NT; ++q) base_g[q] = nat_base[q];
          s_g = nat_s;
        } else {
#pragma unroll
          for (int q = 0; q < NT; ++q) tile_place(tid + q * HALF, m, D, base_g[q], s_g);
        }
      }
    }
    if (pend >= 0) {
      __syncwarp();
      if (lane == 0 && !gave_up) mbar_arrive(&empty[pend]);
      pend = -1;
    }
    if (m < 0) break;
    const float* sp = stages + st * SST;
    const float* xs = ((selfmask >> (k & 31)) & 1u) ? own : sp;  // the column's f block
    if (m == D - 1)
      f32_cols2(g32[0], g32[1], sp + B, xs + base_g[0], xs + base_g[1], s_g);
    else
      f32_rows_rot2(g32[0], g32[1], sp + B, xs + base_g[0], xs + base_g[1], s_g, m == D - 2 ? rot : 0);
    pend = st;
  }
  if (*abort_flag) return;  // y is undefined; the plan's status word reports the timeout
#pragma unroll
  for (int q = 0; q < NT; ++q) {
    const size_t y0 = static_cast<size_t>(row) * B + nat_base[q];
    float* yr = a.y + y0;
#pragma unroll
    for (int r = 0; r < P; ++r)
      *reinterpret_cast<float4*>(yr + r * nat_s) =
          minus_sub4(make_float4(n32[q].v[r][0].x, n32[q].v[r][0].y, n32[q].v[r][1].x, n32[q].v[r][1].y),
                     a.ysub, y0 + r * nat_s);
  }
}

// Persistent variant of k_single_tma: one CTA per resident slot walks a static list of rows
// (longest-processing-time assignment made at plan creation, cta_ptr/cta_rows).  The
// producer streams entries across row boundaries, so only a CTA's first copy pays the
// cold-start latency, and the lists balance work instead of leaving a short last wave.
// Per row the consumers run exactly the k_single_tma algorithm (same group order, same
// Kahan merges, one write of the row's y block), so results are bitwise those of kind 3.
template <typename T, int S, int MINB>
__global__ void __launch_bounds__(288, MINB) k_single_tma_rows(ApplyArgs<T> a) {
  constexpr int P = 4;
  constexpr bool F32 = sizeof(T) == 4;
  constexpr int AB = 16;  // operator block values per stage (FP32: column by column)
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ int s_abort;
  const int tid = threadIdx.x;
  const int warp = tid >> 5, lane = tid & 31;
  const int B = a.B, D = a.D;
  const int SST = B + AB;
  T* stages = reinterpret_cast<T*>(smem_raw);
  uint64_t* full = reinterpret_cast<uint64_t*>(stages + S * SST);
  uint64_t* empty = full + S;
  const int ri0 = a.cta_ptr[blockIdx.x], ri1 = a.cta_ptr[blockIdx.x + 1];
  const uint32_t fbytes = static_cast<uint32_t>(B * sizeof(T)), abytes = AB * sizeof(T);
  const T* opsrc = F32 ? reinterpret_cast<const T*>(a.ops_cols) : a.ops;

  if (tid == 0) {
    s_abort = 0;
    for (int k = 0; k < S; ++k) {
      mbar_init(&full[k], 1);
      mbar_init(&empty[k], 8);
    }
    mbar_fence_init();
  }
  __syncthreads();
  volatile int* abort_flag = &s_abort;

  if (warp == 8) {
    // ---------------- producer warp: one stage counter g across all rows ----------------
    int g = 0;
    bool stop = false;
    for (int ri = ri0; ri < ri1 && !stop; ++ri) {
      const int row = a.cta_rows[ri];
      const long long q0 = a.row_ptr[row];
      const int n = static_cast<int>(a.row_ptr[row + 1] - q0);
      const EntryDesc* ed = a.ed + q0;
      for (int k0 = 0; k0 < n && !stop; k0 += 32) {
        EntryDesc mine{};
        if (k0 + lane < n) mine = ed[k0 + lane];
        const int cnt = min(32, n - k0);
        for (int l = 0; l < cnt; ++l) {
          const int j = __shfl_sync(0xffffffffu, mine.j, l);
          const long long aoff = __shfl_sync(0xffffffffu, mine.aoff, l);
          const int st = g % S;
          bool ok = true;
          if (g >= S) ok = mbar_wait_bounded(&empty[st], static_cast<uint32_t>(((g / S) - 1) & 1));
          if (!__all_sync(0xffffffffu, ok)) {
            if (lane == 0) *abort_flag = 1;
            stop = true;
            break;
          }
          if (lane == 0) {
            T* dst = stages + st * SST;
            fence_proxy_async();
            mbar_expect_tx(&full[st], fbytes + abytes);
            bulk_g2s(dst, a.f + static_cast<size_t>(j) * B, fbytes, &full[st]);
            bulk_g2s(dst + B, opsrc + aoff * (AB / 16), abytes, &full[st]);
          }
          ++g;
          __syncwarp();
        }
      }
    }
    if (lane == 0) {
      if (*abort_flag) atomicExch(a.err, static_cast<int>(ASG_ERR_TIMEOUT));
      // every issued copy lands before the CTA's shared memory is released (bounded)
      for (int k = max(0, g - S); k < g; ++k) {
        const long long t0 = clock64();
        while (!mbar_test(&full[k % S], static_cast<uint32_t>((k / S) & 1)) && clock64() - t0 < (1LL << 28)) {
        }
      }
    }
    return;
  }

  // ---------------- consumer warps ----------------
  int nat_base, nat_s;
  tile_place(tid, D - 3, D, nat_base, nat_s);
  int g = 0;
  bool gave_up = false;
  for (int ri = ri0; ri < ri1; ++ri) {
    const int row = a.cta_rows[ri];
    const long long q0 = a.row_ptr[row];
    const int n = static_cast<int>(a.row_ptr[row + 1] - q0);
    const EntryDesc* ed = a.ed + q0;
    int cur_m = -1, base_g = 0, s_g = 0, pend = -1, mlane = -1;
    bool direct = false;
    PairTile g32;  // a group's sums (pairs of operator rows)
    F32Tile n32, c32;
    T gg[P][P], nat[P][P];
#pragma unroll
    for (int r = 0; r < P; ++r) {
#pragma unroll
      for (int cp = 0; cp < 2; ++cp) g32.v[r][cp] = n32.v[r][cp] = c32.v[r][cp] = make_float2(0.f, 0.f);
#pragma unroll
      for (int c = 0; c < P; ++c) gg[r][c] = nat[r][c] = T(0);
    }
    for (int k = 0; k <= n; ++k) {
      int m = -1;
      const int st = g % S;
      if (k < n) {
        if ((k & 31) == 0) mlane = (k + lane < n) ? ed[k + lane].m : -1;
        m = __shfl_sync(0xffffffffu, mlane, k & 31);
        if (!gave_up) {
          const bool ok = mbar_wait_bounded(&full[st], static_cast<uint32_t>((g / S) & 1));
          if (!__all_sync(0xffffffffu, ok)) {
            gave_up = true;
            *abort_flag = 1;
          }
        }
      }
      if (m != cur_m) {
        if (direct) {
          if constexpr (F32) {
#pragma unroll
            for (int r = 0; r < P; ++r) {
              const float4 v = pt_row(g32, r, cur_m == D - 1);
              kahan2(n32.v[r][0], c32.v[r][0], make_float2(v.x, v.y));
              kahan2(n32.v[r][1], c32.v[r][1], make_float2(v.z, v.w));
            }
          } else {
#pragma unroll
            for (int r = 0; r < P; ++r)
#pragma unroll
              for (int c = 0; c < P; ++c) nat[r][c] += gg[r][c];
          }
        } else if (cur_m >= 0) {
          // transpose the group's sums onto the natural tiles through the stage just consumed
          consumer_sync();
          T* scr = stages + pend * SST;
#pragma unroll
          for (int i = 0; i < P; ++i) {
            if constexpr (F32) {
              // rows of a group on dimension d-2 in a per-thread rotated order (bank-conflict free)
              const int r = (i + (cur_m == D - 2 ? (tid >> 1) & 3 : 0)) & 3;
              *reinterpret_cast<float4*>(scr + base_g + r * s_g) = pt_row_sel(g32, r);
            } else {
              const int r = i;
              Row<T, P> rr;
#pragma unroll
              for (int c = 0; c < P; ++c) rr.v[c] = gg[r][c];
              rr.store(scr + base_g + r * s_g);
            }
          }
          consumer_sync();
#pragma unroll
          for (int r = 0; r < P; ++r) {
            if constexpr (F32) {
              const float4 v = *reinterpret_cast<const float4*>(scr + nat_base + r * nat_s);
              kahan2(n32.v[r][0], c32.v[r][0], make_float2(v.x, v.y));
              kahan2(n32.v[r][1], c32.v[r][1], make_float2(v.z, v.w));
            } else {
              Row<T, P> rr;
              rr.load(scr + nat_base + r * nat_s);
#pragma unroll
              for (int c = 0; c < P; ++c) nat[r][c] += rr.v[c];
            }
          }
        }
        cur_m = m;
        if (m >= 0) {
#pragma unroll
          for (int r = 0; r < P; ++r) {
#pragma unroll
            for (int cp = 0; cp < 2; ++cp) g32.v[r][cp] = make_float2(0.f, 0.f);
#pragma unroll
            for (int c = 0; c < P; ++c) gg[r][c] = T(0);
          }
          direct = (m == D - 1) || (m == D - 3);
          if (m == D - 1) {
            base_g = nat_base;
            s_g = nat_s;
          } else {
            tile_place(tid, m, D, base_g, s_g);
          }
        }
      }
      if (pend >= 0) {
        __syncwarp();
        if (lane == 0 && !gave_up) mbar_arrive(&empty[pend]);
        pend = -1;
      }
      if (m < 0) break;
      const T* sp = stages + st * SST;
      if constexpr (F32) {
        if (m == D - 1)
          pt_cols(g32, reinterpret_cast<const float*>(sp + B), reinterpret_cast<const float*>(sp + base_g), s_g);
        else
          pt_rows_rot(g32, reinterpret_cast<const float*>(sp + B), reinterpret_cast<const float*>(sp + base_g), s_g,
                      m == D - 2 ? (tid >> 1) & 3 : 0);
      } else {
        T A[P * P];
#pragma unroll
        for (int r = 0; r < P; ++r) {
          Row<T, P> rr;
          rr.load(sp + B + r * P);
#pragma unroll
          for (int c = 0; c < P; ++c) A[r * P + c] = rr.v[c];
        }
        if (m == D - 1)
          tile_cols_s<T>(gg, A, sp + base_g, s_g);
        else
          tile_rows<T>(gg, A, sp + base_g, s_g);
      }
      pend = st;
      ++g;
    }
    if (*abort_flag) continue;  // y is undefined; the plan's status word reports the timeout
    const size_t y0 = static_cast<size_t>(row) * B + nat_base;
    T* yr = a.y + y0;
#pragma unroll
    for (int r = 0; r < P; ++r) {
      if constexpr (F32) {
        *reinterpret_cast<float4*>(reinterpret_cast<float*>(yr) + r * nat_s) =
            minus_sub4(make_float4(n32.v[r][0].x, n32.v[r][0].y, n32.v[r][1].x, n32.v[r][1].y),
                       reinterpret_cast<const float*>(a.ysub), y0 + r * nat_s);
      } else {
        Row<T, P> rr;
#pragma unroll
        for (int c = 0; c < P; ++c) rr.v[c] = minus_sub(nat[r][c], a.ysub, y0 + r * nat_s + c);
        rr.store(yr + r * nat_s);
      }
    }
  }
}

// ---------------------------------------------------------------------------------------
// Gradient with respect to the 1-D operators.  For a work entry (i, j, t) and an applied
// factor k of term t, d L / d A_{t,k}[I_k(i), J_k(j)] (a P x P block) is the contraction of
// r_i with Z = (kron of the term's other applied factors) f_j over every dimension but k:
// G[a][b] = sum over the fibers along k of r_i[.., a, ..] * Z[.., b, ..].  Z is recomputed
// from f_j (mode products in shared memory) instead of being stored by the forward pass.
// One CTA owns one target block and sums its contributors in a fixed order; the P x P
// partial sums are reduced across the CTA with shuffles and one shared-memory pass, so the
// result is bitwise deterministic without atomics.
// ---------------------------------------------------------------------------------------
template <typename T, int P>
__global__ void __launch_bounds__(256) k_grad(GradArgs<T> a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int B = a.B, D = a.D, tid = threadIdx.x;
  const int lane = tid & 31, warp = tid >> 5;
  const int Bpad = (B + 3) & ~3;
  T* buf0 = reinterpret_cast<T*>(smem_raw);
  T* buf1 = buf0 + Bpad;
  T* red = buf1 + Bpad;  // [8][P*P]
  for (int g = blockIdx.x; g < a.ntgt; g += gridDim.x) {
    const GradTarget tg = a.tgt[g];
    T* Gout = a.G[tg.tm];
    if (Gout == nullptr) continue;  // uniform across the CTA
    T acc[P][P];
#pragma unroll
    for (int x = 0; x < P; ++x)
#pragma unroll
      for (int y = 0; y < P; ++y) acc[x][y] = T(0);
    for (long long c = a.tgt_ptr[g]; c < a.tgt_ptr[g + 1]; ++c) {
      const GradContrib e = a.contrib[c];
      const unsigned others = a.active[e.t] & ~(1u << e.k);
      const T* ri = a.r + static_cast<size_t>(e.i) * B;
      const T* z = a.f + static_cast<size_t>(e.j) * B;
      if (others) {
        team_copy(buf0, z, B, tid, 256);
        __syncthreads();
        T* in = buf0;
        T* out = buf1;
        for (int m = D - 1; m >= 0; --m) {
          if (!((others >> m) & 1u)) continue;
          const int tm = e.t * D + m;
          const T* Ag = a.ops + a.op_off[tm] +
                        (static_cast<long long>(a.idx1d[e.i * D + m]) * a.op_nb[tm] + a.idx1d[e.j * D + m]) * (P * P);
          T A[P * P];
#pragma unroll
          for (int r = 0; r < P * P; ++r) A[r] = Ag[r];
          mode_pass<T, P>(in, out, A, B, a.stride[m], tid, 256);
          __syncthreads();
          T* tmp = in;
          in = out;
          out = tmp;
        }
        z = in;
      }
      const int s = a.stride[e.k];
      const int nf = B / P;
      for (int fi = tid; fi < nf; fi += 256) {
        const int hi = fi / s, lo = fi - hi * s;
        const int base = hi * s * P + lo;
        T rv[P], zv[P];
#pragma unroll
        for (int x = 0; x < P; ++x) {
          rv[x] = ri[base + x * s];
          zv[x] = z[base + x * s];
        }
#pragma unroll
        for (int x = 0; x < P; ++x)
#pragma unroll
          for (int y = 0; y < P; ++y) acc[x][y] = fma(rv[x], zv[y], acc[x][y]);
      }
      __syncthreads();  // the staging buffers are reused by the next contributor
    }
#pragma unroll
    for (int x = 0; x < P; ++x)
#pragma unroll
      for (int y = 0; y < P; ++y) {
        T v = acc[x][y];
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
        if (lane == 0) red[warp * P * P + x * P + y] = v;
      }
    __syncthreads();
    if (tid < P * P) {
      T sum = T(0);
      for (int w = 0; w < 8; ++w) sum += red[w * P * P + tid];
      const int x = tid / P, y = tid % P;
      Gout[static_cast<long long>(tg.beta * P + y) * a.ldg[tg.tm] + tg.alpha * P + x] = sum;
    }
    __syncthreads();
  }
}

// Chunked gradient for plans whose terms have one applied factor (deg 4): no mode chain to
// recompute, so a contributor is a pure contraction of two 4096-value blocks.  One CTA per
// item of up to 8 contributors of one target, one warp per contributor reading both blocks
// with 16-byte loads (fibers along k grouped 4 at a time along the fastest dimension).  The
// item's 4 x 4 sum (warps added in a fixed order) goes to a partial slot; the CTA that
// finishes a target's last item (atomic counter) adds the target's partials in item order and
// writes G, so the result does not depend on which CTA arrives last.
template <typename T>
__device__ __forceinline__ void load4(const T* p, T (&v)[4]) {
  if constexpr (sizeof(T) == 4) {
    const float4 q = *reinterpret_cast<const float4*>(p);
    v[0] = q.x; v[1] = q.y; v[2] = q.z; v[3] = q.w;
  } else {
    const double2 q0 = *reinterpret_cast<const double2*>(p);
    const double2 q1 = *reinterpret_cast<const double2*>(p + 2);
    v[0] = q0.x; v[1] = q0.y; v[2] = q1.x; v[3] = q1.y;
  }
}

template <typename T>
__global__ void __launch_bounds__(256) k_grad_items(GradArgs<T> a) {
  constexpr int P = 4;
  __shared__ T red[8][P * P];
  __shared__ int s_last;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int B = a.B;
  for (int it = blockIdx.x; it < a.nitems; it += gridDim.x) {
    const GradItem item = a.items[it];
    const GradTarget tg = a.tgt[item.tgt];
    T* Gout = a.G[tg.tm];
    if (Gout == nullptr) continue;  // uniform across the CTA
    T acc[P][P];
#pragma unroll
    for (int x = 0; x < P; ++x)
#pragma unroll
      for (int y = 0; y < P; ++y) acc[x][y] = T(0);
    const int c = item.c0 + warp;
    if (c < item.c1) {
      const GradContrib e = a.contrib[c];
      const T* ri = a.r + static_cast<size_t>(e.i) * B;
      const T* zj = a.f + static_cast<size_t>(e.j) * B;
      const int s = a.stride[e.k];
      if (s == 1) {
        // fibers are 4 contiguous values: G[x][y] += r[x] z[y]
#pragma unroll 8
        for (int fb = lane; fb < B / P; fb += 32) {
          T rv[4], zv[4];
          load4(ri + fb * P, rv);
          load4(zj + fb * P, zv);
#pragma unroll
          for (int x = 0; x < P; ++x)
#pragma unroll
            for (int y = 0; y < P; ++y) acc[x][y] = fma(rv[x], zv[y], acc[x][y]);
        }
      } else {
        // 4 fibers with consecutive fastest-dimension offsets per lane: one 16-byte load per
        // (fiber position x) holds the 4 fibers' values
#pragma unroll 8
        for (int grp = lane; grp < B / (P * 4); grp += 32) {
          const int o = grp * 4;            // first of the 4 fibers (o = hi * s + lo)
          const int hi = o / s, lo = o - hi * s;
          const int base = hi * s * P + lo;
          T rv[P][4], zv[P][4];
#pragma unroll
          for (int x = 0; x < P; ++x) {
            load4(ri + base + x * s, rv[x]);
            load4(zj + base + x * s, zv[x]);
          }
#pragma unroll
          for (int x = 0; x < P; ++x)
#pragma unroll
            for (int y = 0; y < P; ++y)
#pragma unroll
              for (int q = 0; q < 4; ++q) acc[x][y] = fma(rv[x][q], zv[y][q], acc[x][y]);
        }
      }
    }
#pragma unroll
    for (int x = 0; x < P; ++x)
#pragma unroll
      for (int y = 0; y < P; ++y) {
        T v = acc[x][y];
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
        if (lane == 0) red[warp][x * P + y] = v;
      }
    __syncthreads();
    if (tid < P * P) {
      T sum = T(0);
#pragma unroll
      for (int w = 0; w < 8; ++w) sum += red[w][tid];
      a.partial[static_cast<size_t>(it) * P * P + tid] = sum;
      __threadfence();
    }
    __syncthreads();
    if (tid == 0) s_last = atomicAdd(&a.counter[item.tgt], 1) == item.count - 1;
    __syncthreads();
    if (s_last) {
      __threadfence();
      if (tid < P * P) {
        T sum = T(0);
        for (int q = item.first; q < item.first + item.count; ++q)
          sum += __ldcg(a.partial + static_cast<size_t>(q) * P * P + tid);
        const int x = tid / P, y = tid % P;
        Gout[static_cast<long long>(tg.beta * P + y) * a.ldg[tg.tm] + tg.alpha * P + x] = sum;
      }
      if (tid == 0) a.counter[item.tgt] = 0;  // ready for the next launch (stream order)
    }
    __syncthreads();
  }
}

template <typename T, int P>
cudaError_t launch_grad_p(const GradArgs<T>& a, cudaStream_t s) {
  const int Bpad = (a.B + 3) & ~3;
  const size_t sm = (static_cast<size_t>(2) * Bpad + 8 * P * P) * sizeof(T);
  auto kern = k_grad<T, P>;
  static bool done = false;
  if (sm > 48 * 1024 && !done) {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         static_cast<int>((2 * kMaxBlock + 8 * P * P) * sizeof(T)));
    if (e != cudaSuccess) return e;
    done = true;
  }
  const int grid = a.ntgt < 152 * 8 ? a.ntgt : 152 * 8;
  kern<<<grid, 256, sm, s>>>(a);
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_grad_items(const GradArgs<T>& a, cudaStream_t s) {
  const int grid = a.nitems < 152 * 8 ? a.nitems : 152 * 8;
  k_grad_items<T><<<grid, 256, 0, s>>>(a);
  return cudaGetLastError();
}

// Opt a kernel into more than 48 KB of dynamic shared memory (once per instantiation; the
// limit set is the largest this kernel can request, so later plans need no new call).
template <typename K>
cudaError_t ensure_smem(K kernel, size_t bytes, size_t max_bytes, bool& done) {
  if (bytes <= 48 * 1024 || done) return cudaSuccess;
  cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(max_bytes));
  if (e == cudaSuccess) done = true;
  return e;
}

// Dynamic shared memory of k_single_tma_rows: S stages of (f block + operator block) and the
// full/empty barriers.
template <typename T>
size_t rows_smem(int S, int B) {
  return static_cast<size_t>(S) * (B + 16) * sizeof(T) + 2 * S * sizeof(uint64_t);
}

template <typename T, int P>
cudaError_t launch_p(const ApplyArgs<T>& a, int kind, cudaStream_t s) {
  constexpr bool K = sizeof(T) == 4;
  const int Bpad = (a.B + 3) & ~3;
  if (kind == KK_CHAIN_WARP) {
    const int wpb = 4;
    const size_t sm = static_cast<size_t>(wpb) * 2 * Bpad * sizeof(T);
    auto kern = k_chain_warp<T, P, K>;
    static bool done = false;
    cudaError_t e = ensure_smem(kern, sm, static_cast<size_t>(wpb) * 2 * 256 * sizeof(T), done);
    if (e != cudaSuccess) return e;
    const int grid = (a.N + wpb - 1) / wpb;
    kern<<<grid, wpb * 32, sm, s>>>(a);
    return cudaGetLastError();
  }
  if (kind == KK_CHAIN_CTA) {
    constexpr int NT = 256;
    const size_t sm = (static_cast<size_t>(2) * Bpad + a.D * P * P) * sizeof(T);
    auto kern = k_chain_cta<T, P, K, NT>;
    static bool done = false;
    cudaError_t e = ensure_smem(kern, sm, (static_cast<size_t>(2) * kMaxBlock + kMaxDims * P * P) * sizeof(T), done);
    if (e != cudaSuccess) return e;
    kern<<<a.N, NT, sm, s>>>(a);
    return cudaGetLastError();
  }
  if constexpr (P == 4) {
    if (kind == KK_SINGLE_TMA || kind == KK_SINGLE_TMA3) {
      // kind 3: FP32 4 stages (2 CTAs per SM), FP64 3 stages (1 CTA per SM), each with the
      // row's own f block resident; kind 4 (FP32): 3 stages and the compensation tile in
      // shared memory, no resident block (3 CTAs per SM)
      if (a.B != 256 * P * P) return cudaErrorInvalidValue;  // 8 consumer warps own one tile each
      if (sizeof(T) == 4 && !a.ops_pair) return cudaErrorInvalidValue;
      constexpr int AB = sizeof(T) == 4 ? 32 : 16;  // operator values per stage
      auto smem_for = [&](int S, bool csmem, bool own) {
        return static_cast<size_t>(S) * (a.B + AB) * sizeof(T) + (csmem ? a.B * sizeof(float) : 0) +
               (own ? a.B * sizeof(T) : 0) + (2 * S + 1) * sizeof(uint64_t);
      };
      if constexpr (sizeof(T) == 4) {
        if (kind == KK_SINGLE_TMA3) {
          const size_t sm = smem_for(3, true, false);
          auto kern = k_single_tma<T, 3, 3, true, false>;
          static bool done = false;
          cudaError_t e = ensure_smem(kern, sm, sm, done);
          if (e != cudaSuccess) return e;
          kern<<<a.N, 288, sm, s>>>(a);
          return cudaGetLastError();
        }
      }
      constexpr int S0 = sizeof(T) == 4 ? 4 : 3;
      const size_t sm = smem_for(S0, false, true);
      auto kern = k_single_tma<T, S0, sizeof(T) == 4 ? 2 : 1, false, true>;
      static bool done = false;
      cudaError_t e = ensure_smem(kern, sm, sm, done);
      if (e != cudaSuccess) return e;
      kern<<<a.N, 288, sm, s>>>(a);
      return cudaGetLastError();
    }
  }
  if constexpr (P == 4 && sizeof(T) == 4) {
    if (kind == KK_SINGLE_TMA_X2) {
      // FP32, two tiles per consumer thread: 4 stages, 2 CTAs per SM
      if (a.B != 256 * P * P || !a.ops_pair) return cudaErrorInvalidValue;
      constexpr int S0 = 4;
      const size_t sm = (static_cast<size_t>(S0) * (a.B + 32) + a.B) * sizeof(float) + (2 * S0 + 1) * sizeof(uint64_t);
      auto kern = k_single_tma_x2<S0, 2>;
      static bool done = false;
      cudaError_t e = ensure_smem(kern, sm, sm, done);
      if (e != cudaSuccess) return e;
      kern<<<a.N, 160, sm, s>>>(a);
      return cudaGetLastError();
    }
  }
  if (kind == KK_SINGLE_SMALL) {
    if (a.B > 256 || !a.ed) return cudaErrorInvalidValue;
    const int wpb = 4;
    const int grid = (a.N + wpb - 1) / wpb;
    if constexpr (P <= 4) {
      const int Lf = a.B / P;
      // warps per row: 4 in FP32, 2 in FP64 (FP64 issue-bound sooner) -- the fastest or tied
      // on every measured plan (continuity2/3, diffusion2); fixed by the precision alone, so a
      // row is summed in the same order in every plan that holds it
      constexpr int WR = sizeof(T) == 4 ? 4 : 2;
      const int g2 = a.N < 152 * 16 ? a.N : 152 * 16;  // one CTA per row, at most 16 per SM
      auto launch = [&](auto maxf) -> cudaError_t {
        constexpr int MF = decltype(maxf)::value;
        k_single_fiber_split<T, P, MF, K, WR><<<g2, 32 * WR, 0, s>>>(a);
        return cudaGetLastError();
      };
      if (Lf <= 32) return launch(std::integral_constant<int, 1>{});
      if (Lf <= 64) return launch(std::integral_constant<int, 2>{});
      return launch(std::integral_constant<int, 4>{});
    }
    if (a.B <= 32)
      k_single_small<T, P, 1, K><<<grid, wpb * 32, 0, s>>>(a);
    else if (a.B <= 64)
      k_single_small<T, P, 2, K><<<grid, wpb * 32, 0, s>>>(a);
    else if (a.B <= 128)
      k_single_small<T, P, 4, K><<<grid, wpb * 32, 0, s>>>(a);
    else
      k_single_small<T, P, 8, K><<<grid, wpb * 32, 0, s>>>(a);
    return cudaGetLastError();
  }
  if constexpr (P == 4) {
    if (kind == KK_SINGLE_TMA_ROWS) {
      if (a.B != 256 * P * P || !a.cta_ptr || !a.cta_rows || a.nctas <= 0) return cudaErrorInvalidValue;
      if (sizeof(T) == 4 && !a.ops_cols) return cudaErrorInvalidValue;
      constexpr int S0 = sizeof(T) == 4 ? 4 : 3;
      const size_t sm = rows_smem<T>(S0, a.B);
      auto kern = k_single_tma_rows<T, S0, sizeof(T) == 4 ? 2 : 1>;
      static bool done = false;
      cudaError_t e = ensure_smem(kern, sm, sm, done);
      if (e != cudaSuccess) return e;
      kern<<<a.nctas, 288, sm, s>>>(a);
      return cudaGetLastError();
    }
  }
  if constexpr (P == 3 || P == 4) {
    if (kind == KK_SINGLE_MODE) {
      const int nt = a.B / (P * P);
      const size_t sm = static_cast<size_t>(a.B) * sizeof(T);
      auto kern = k_single_mode<T, P, K>;
      static bool done = false;
      cudaError_t e = ensure_smem(kern, sm, static_cast<size_t>(kMaxBlock) * sizeof(T), done);
      if (e != cudaSuccess) return e;
      kern<<<a.N, nt, sm, s>>>(a);
      return cudaGetLastError();
    }
  }
  return cudaErrorInvalidValue;
}

}  // namespace

int single_tma_rows_occupancy(int es) {
  int nb = 0;
  cudaError_t e;
  if (es == 4) {
    auto kern = k_single_tma_rows<float, 4, 2>;
    const size_t sm = rows_smem<float>(4, 4096);
    e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(sm));
    if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, kern, 288, sm);
  } else {
    auto kern = k_single_tma_rows<double, 3, 1>;
    const size_t sm = rows_smem<double>(3, 4096);
    e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(sm));
    if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, kern, 288, sm);
  }
  return e == cudaSuccess ? nb : 0;
}

template <typename T>
cudaError_t launch_apply(const ApplyArgs<T>& a, int P, int kind, cudaStream_t s) {
  if (a.N == 0) return cudaSuccess;
  switch (P) {
    case 1: return launch_p<T, 1>(a, kind, s);
    case 2: return launch_p<T, 2>(a, kind, s);
    case 3: return launch_p<T, 3>(a, kind, s);
    case 4: return launch_p<T, 4>(a, kind, s);
    case 5: return launch_p<T, 5>(a, kind, s);
    case 6: return launch_p<T, 6>(a, kind, s);
    case 7: return launch_p<T, 7>(a, kind, s);
    case 8: return launch_p<T, 8>(a, kind, s);
    default: return cudaErrorInvalidValue;
  }
}

template <typename T>
cudaError_t launch_grad(const GradArgs<T>& a, int P, cudaStream_t s) {
  if (a.ntgt == 0) return cudaSuccess;
  if (a.items) return P == 4 ? launch_grad_items<T>(a, s) : cudaErrorInvalidValue;
  switch (P) {
    case 1: return launch_grad_p<T, 1>(a, s);
    case 2: return launch_grad_p<T, 2>(a, s);
    case 3: return launch_grad_p<T, 3>(a, s);
    case 4: return launch_grad_p<T, 4>(a, s);
    case 5: return launch_grad_p<T, 5>(a, s);
    case 6: return launch_grad_p<T, 6>(a, s);
    case 7: return launch_grad_p<T, 7>(a, s);
    case 8: return launch_grad_p<T, 8>(a, s);
    default: return cudaErrorInvalidValue;
  }
}

template cudaError_t launch_grad<double>(const GradArgs<double>&, int, cudaStream_t);
template cudaError_t launch_grad<float>(const GradArgs<float>&, int, cudaStream_t);
template cudaError_t launch_apply<double>(const ApplyArgs<double>&, int, int, cudaStream_t);
template cudaError_t launch_apply<float>(const ApplyArgs<float>&, int, int, cudaStream_t);

}  // namespace asg
