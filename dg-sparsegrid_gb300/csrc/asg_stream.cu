// Streaming FP32 apply for plans with one applied factor per term and 4,096-value element
// blocks (deg 4, 6 dimensions: the continuity6 configuration), y = A*f over the pair list
// (apply_A.m:102-236, each term's Kronecker product I x .. x D_k x .. x I applied to f_j).
//
// One persistent CTA per SM walks a fixed stream of work entries: the rows assigned to it at
// plan creation (longest-processing-time balance of the bytes each row gathers), each row's
// entries grouped by the dimension of their applied factor.  Warp 8 produces, warps 0..7
// consume:
//   * a stage holds two consecutive entries.  Per stage the producer's elected lane issues
//     bulk copies (cp.async.bulk, completion as transaction bytes on the stage's mbarrier) of
//     each entry's column block (16 KB) and 4 x 4 operator block (64 B, stored column by
//     column).  The row's own block f_i, which every term's diagonal entry (i, i) reads, is
//     copied once per row into one of two resident buffers (its bytes ride on the stage of
//     the row's first entry); diagonal entries then move only their operator block.
//   * a consumer thread owns a 4 x 4 output tile.  Entries of a group (same applied
//     dimension m) accumulate in registers in the tile layout of m: rows along m, columns the
//     4 contiguous values of the last dimension.  The paired FMA (fma.rn.f32x2) runs on pairs
//     of operator rows, which an operator column delivers as they lie (one 128-bit shared
//     load per operator column), and on the input value duplicated in registers.  Groups on
//     dimensions 3 and 5 land in the natural tile (rows along 3); the others pass through one
//     of two transpose buffers behind one consumer barrier.  Groups merge into the natural
//     tile with Kahan compensation; each y block is written once, no atomics, in a fixed
//     order: bitwise reproducible.
// Every wait is bounded (~2^31 cycles, or at once when another warp gave up): the CTA then
// records ASG_ERR_TIMEOUT in the plan's status word, the producer waits (bounded) for the
// copies it issued, and the CTA exits.  Consumers keep the barrier sequence uniform after a
// timeout (work is skipped, barriers are not).
#include "asg_internal.h"
#include "asg_pipe.cuh"

namespace asg {
namespace {

constexpr int kB = 4096;           // values per element block
constexpr int kAB = 16;            // values per operator block (column-major 4 x 4)
constexpr int kSlot = kB + kAB;    // floats per entry slot
constexpr int kStage = 2 * kSlot;  // floats per pipeline stage (two entries)
constexpr int kDescSmem = 320;     // stream entries (header included) staged in shared memory

// Tile of consumer thread tid for a group on dimension u (0..4): rows along u (stride 4^(5-u)),
// columns the 4 contiguous values of dimension 5; the thread's other digits run over the
// remaining dimensions, the highest fastest.  u = 3 is the natural tile.
__device__ __forceinline__ void stream_tile(int tid, int u, int& base, int& s) {
  const int sh = 2 * (4 - u);
  s = 1 << (2 * (5 - u));
  base = (tid >> sh) * s * 4 + (tid & ((1 << sh) - 1)) * 4;
}

// Named hardware barrier among the 256 consumer threads (the transpose buffers).
__device__ __forceinline__ void consumers_sync() { asm volatile("bar.sync 15, 256;" ::: "memory"); }

template <int S>
__global__ void __launch_bounds__(288, 1) k_stream(StreamArgs a) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  __shared__ __align__(16) int4 sdesc[kDescSmem];
  __shared__ __align__(8) uint64_t dbar;
  __shared__ int s_abort;
  float* stages = reinterpret_cast<float*>(smem_raw);  // S x 2 x (f block, operator block)
  float* R = stages + S * kStage;                      // 2 resident row blocks
  float* X = R + 2 * kB;                               // 2 transpose buffers
  uint64_t* full = reinterpret_cast<uint64_t*>(X + 2 * kB);
  uint64_t* empty = full + S;
  uint64_t* rempty = empty + S;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int4* ws = a.ws + static_cast<size_t>(blockIdx.x) * a.ws_stride;

  if (tid == 0) {
    s_abort = 0;
    for (int k = 0; k < S; ++k) {
      mbar_init(&full[k], 1);
      mbar_init(&empty[k], 8);
    }
    for (int k = 0; k < 2; ++k) mbar_init(&rempty[k], 8);
    mbar_init(&dbar, 1);
    mbar_fence_init();
    // the CTA's stream (header and entries, padded) in one bulk copy: one dependent load
    const int nd = a.ws_stride < kDescSmem ? a.ws_stride : kDescSmem;
    mbar_expect_tx(&dbar, static_cast<uint32_t>(nd * sizeof(int4)));
    bulk_g2s(sdesc, ws, static_cast<uint32_t>(nd * sizeof(int4)), &dbar);
  }
  __syncthreads();
  volatile int* abort_flag = &s_abort;
  // entries past the staged part come from global memory (streams longer than kDescSmem - 1)
  auto desc = [&](int k) -> int4 { return k + 1 < kDescSmem ? sdesc[k + 1] : ws[k + 1]; };
  if (!__all_sync(0xffffffffu, mbar_wait_or_abort(&dbar, 0, abort_flag))) {
    if (lane == 0) {  // uniform across the CTA: every warp waited on the same phase
      *abort_flag = 1;
      atomicExch(a.err, static_cast<int>(ASG_ERR_TIMEOUT));
    }
    return;
  }
  const int count = sdesc[0].x;

  if (warp == 8) {
    // ---------------- producer: stage p holds staged entries 2p and 2p + 1 ----------------
    int q = 0, rows = 0, issued = 0;  // entries staged, rows started, stages issued
    bool ok = true;
    uint32_t bytes = 0;
    for (int k = 0; k < count && ok; ++k) {
      const int4 e = desc(k);
      const int j = e.x, row = e.y, blk = e.z, fl = e.w;
      if (fl & SF_ZERO) continue;
      const int p = q >> 1, slot = q & 1, st = p % S;
      if (slot == 0) {
        if (p >= S) ok = mbar_wait_or_abort(&empty[st], static_cast<uint32_t>(((p / S) - 1) & 1), abort_flag);
        // the stage's byte count: this entry and the next staged one
        bytes = 0;
        for (int k2 = k, n2 = 0; k2 < count && n2 < 2; ++k2) {
          const int4 e2 = desc(k2);
          if (e2.w & SF_ZERO) continue;
          bytes += (kAB + ((e2.w & SF_SELF) ? 0 : kB) + ((e2.w & SF_ROW0) ? kB : 0)) * 4;
          ++n2;
        }
      }
      if (ok && (fl & SF_ROW0) && rows >= 2)
        ok = mbar_wait_or_abort(&rempty[rows & 1], static_cast<uint32_t>(((rows >> 1) - 1) & 1), abort_flag);
      if (!__all_sync(0xffffffffu, ok)) {
        ok = false;
        if (lane == 0) *abort_flag = 1;
        break;
      }
      if (lane == 0) {
        float* dst = stages + st * kStage + slot * kSlot;
        if (slot == 0) {
          fence_proxy_async();
          mbar_expect_tx(&full[st], bytes);
        }
        bulk_g2s(dst + kB, a.ops_cols + static_cast<size_t>(blk) * kAB, kAB * 4, &full[st]);
        if (!(fl & SF_SELF)) bulk_g2s(dst, a.f + static_cast<size_t>(j) * kB, kB * 4, &full[st]);
        if (fl & SF_ROW0) bulk_g2s(R + (rows & 1) * kB, a.f + static_cast<size_t>(row) * kB, kB * 4, &full[st]);
      }
      __syncwarp();
      if (slot == 0) issued = p + 1;
      if (fl & SF_ROW0) ++rows;
      ++q;
    }
    if (lane == 0) {
      if (*abort_flag) atomicExch(a.err, static_cast<int>(ASG_ERR_TIMEOUT));
      // every issued copy lands before the CTA's shared memory is released (bounded; a stage
      // left with its second entry unissued by an abort never completes and just times out)
      for (int k = max(0, issued - S); k < issued; ++k) {
        const long long t0 = clock64();
        while (!mbar_test(&full[k % S], static_cast<uint32_t>((k / S) & 1)) && clock64() - t0 < (1LL << 28)) {
        }
      }
    }
    return;
  }

  // ---------------- consumers ----------------
  int nat_base, nat_s;
  stream_tile(tid, 3, nat_base, nat_s);
  PairTile g;
  F32Tile n, c;  // natural tile (rows along 3, column pairs along 5) and its compensation
  zero_pt(g);
#pragma unroll
  for (int r = 0; r < 4; ++r) n.v[r][0] = n.v[r][1] = c.v[r][0] = c.v[r][1] = make_float2(0.f, 0.f);
  int m = 3, base_g = nat_base, s_g = nat_s;
  int xcnt = 0, rows = 0, q = 0;  // q: entries staged so far
  bool live = true;
  auto merge_row = [&](int r, float4 v) {
    kahan2(n.v[r][0], c.v[r][0], make_float2(v.x, v.y));
    kahan2(n.v[r][1], c.v[r][1], make_float2(v.z, v.w));
  };
  for (int k = 0; k < count; ++k) {
    const int4 e = desc(k);
    const int fl = e.w;
    if (fl & SF_ZERO) {
      const size_t y0 = static_cast<size_t>(e.y) * kB + nat_base;
      float* yr = a.y + y0;
#pragma unroll
      for (int r = 0; r < 4; ++r)
        *reinterpret_cast<float4*>(yr + r * nat_s) = minus_sub4(make_float4(0.f, 0.f, 0.f, 0.f), a.ysub, y0 + r * nat_s);
      continue;
    }
    if (fl & SF_GRP0) {
      m = fl & 15;
      zero_pt(g);
      if (m == 3 || m == 5) {
        base_g = nat_base;
        s_g = nat_s;
      } else {
        stream_tile(tid, m, base_g, s_g);
      }
    }
    const int p = q >> 1, slot = q & 1, st = p % S;
    ++q;
    if (slot == 0 && live) {
      live = __all_sync(0xffffffffu, mbar_wait_or_abort(&full[st], static_cast<uint32_t>((p / S) & 1), abort_flag));
      if (!live && lane == 0) {
        *abort_flag = 1;
        atomicExch(a.err, static_cast<int>(ASG_ERR_TIMEOUT));
      }
    }
    const float* sp = stages + st * kStage + slot * kSlot;
    const float* xs = ((fl & SF_SELF) ? R + (rows & 1) * kB : sp) + base_g;
    if (live) {
      if (m == 5)
        pt_cols(g, sp + kB, xs, s_g);
      else
        pt_rows(g, sp + kB, xs, s_g);
    }
    // release the stage after its second entry (or the stream's last staged entry)
    bool last = k + 1 == count;
    for (int k2 = k + 1; k2 < count; ++k2) {
      if (!(desc(k2).w & SF_ZERO)) break;
      last = k2 + 1 == count;
    }
    if ((slot == 1 || last) && live) {
      __syncwarp();
      if (lane == 0) mbar_arrive(&empty[st]);
    }
    if (fl & SF_GRP1) {
      const bool cols = m == 5;
      if (m == 3 || m == 5) {
#pragma unroll
        for (int r = 0; r < 4; ++r) merge_row(r, pt_row(g, r, cols));
      } else {
        // transpose buffer X[xcnt & 1]: its previous contents were read before the consumers'
        // previous transpose barrier, which every consumer has passed
        float* xw = X + (xcnt & 1) * kB;
#pragma unroll
        for (int r = 0; r < 4; ++r) *reinterpret_cast<float4*>(xw + base_g + r * s_g) = pt_row(g, r, false);
        consumers_sync();
#pragma unroll
        for (int r = 0; r < 4; ++r) merge_row(r, *reinterpret_cast<const float4*>(xw + nat_base + r * nat_s));
        ++xcnt;
      }
    }
    if (fl & SF_ROW1) {
      if (live) {
        const size_t y0 = static_cast<size_t>(e.y) * kB + nat_base;
        float* yr = a.y + y0;
#pragma unroll
        for (int r = 0; r < 4; ++r)
          *reinterpret_cast<float4*>(yr + r * nat_s) =
              minus_sub4(make_float4(n.v[r][0].x, n.v[r][0].y, n.v[r][1].x, n.v[r][1].y), a.ysub, y0 + r * nat_s);
        __syncwarp();
        if (lane == 0) mbar_arrive(&rempty[rows & 1]);
      }
#pragma unroll
      for (int r = 0; r < 4; ++r) n.v[r][0] = n.v[r][1] = c.v[r][0] = c.v[r][1] = make_float2(0.f, 0.f);
      ++rows;
    }
  }
}

template <int S>
size_t stream_smem_bytes() {
  return static_cast<size_t>(S) * kStage * sizeof(float) + 4 * kB * sizeof(float) + (2 * S + 2) * sizeof(uint64_t);
}

constexpr int kStreamStages = 4;

}  // namespace

size_t stream_smem() { return stream_smem_bytes<kStreamStages>(); }

int stream_occupancy() {
  auto kern = k_stream<kStreamStages>;
  const size_t sm = stream_smem_bytes<kStreamStages>();
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(sm));
  int nb = 0;
  if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, kern, 288, sm);
  return e == cudaSuccess ? nb : 0;
}

cudaError_t launch_stream(const StreamArgs& a, cudaStream_t s) {
  if (a.nctas <= 0) return cudaSuccess;
  if (!a.ws || !a.ops_cols || a.ws_stride < 33) return cudaErrorInvalidValue;
  auto kern = k_stream<kStreamStages>;
  const size_t sm = stream_smem_bytes<kStreamStages>();
  static bool done = false;
  if (!done) {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(sm));
    if (e != cudaSuccess) return e;
    done = true;
  }
  kern<<<a.nctas, 288, sm, s>>>(a);
  return cudaGetLastError();
}

}  // namespace asg
