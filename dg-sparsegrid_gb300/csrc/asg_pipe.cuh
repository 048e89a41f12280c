// Shared-memory pipeline primitives of the deg-4 apply kernels: mbarriers, bulk global->shared
// copies (cp.async.bulk with transaction-count completion), bounded waits, and the FP32
// P x P tile contractions on the paired FMA (fma.rn.f32x2).
#pragma once

#include <cstdint>

#include "asg_internal.h"

namespace asg {

// The value a kernel stores for y: v, or v - s[i] for a residual apply (s = ApplyArgs::ysub,
// i the value's index in y).
template <typename T>
__device__ __forceinline__ T minus_sub(T v, const T* s, size_t i) {
  return s ? v - s[i] : v;
}
__device__ __forceinline__ float4 minus_sub4(float4 v, const float* s, size_t i) {
  if (s) {
    const float4 q = *reinterpret_cast<const float4*>(s + i);
    v.x -= q.x;
    v.y -= q.y;
    v.z -= q.z;
    v.w -= q.w;
  }
  return v;
}

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_fence_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
// One bulk copy of `bytes` (a multiple of 16; both addresses 16-byte aligned) from global to
// this CTA's shared memory; completion counted as transaction bytes on `bar`.
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_u32(dst)),
               "l"(src), "r"(bytes), "r"(smem_u32(bar))
               : "memory");
}
__device__ __forceinline__ bool mbar_test(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{ .reg .pred p; mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2; selp.u32 %0, 1, 0, p; }"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// Bounded wait: true when the phase completed, false after ~2^31 cycles (~1 s).
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity) {
  if (mbar_test(bar, parity)) return true;
  const long long t0 = clock64();
  while (!mbar_test(bar, parity)) {
    if (clock64() - t0 > (1LL << 31)) return false;
  }
  return true;
}
// Bounded wait that also gives up as soon as another warp of the CTA raised `abort_flag`.
__device__ __forceinline__ bool mbar_wait_or_abort(uint64_t* bar, uint32_t parity, const volatile int* abort_flag) {
  if (mbar_test(bar, parity)) return true;
  const long long t0 = clock64();
  while (!mbar_test(bar, parity)) {
    if (*abort_flag || clock64() - t0 > (1LL << 31)) return false;
  }
  return true;
}
__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

// Paired FP32 FMA (fma.rn.f32x2): two FMAs per instruction issue.
__device__ __forceinline__ float2 ffma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }

// A thread's P x P (4 x 4) FP32 tile as column pairs, the operand shape of the paired FMA.
struct F32Tile {
  float2 v[4][2];  // [tile row][column pair]
};

// g[a][c] += sum_b A[a][b] x[b][c]; A column b arrives as (A0b,A0b,A1b,A1b),(A2b,A2b,A3b,A3b)
__device__ __forceinline__ void f32_rows(F32Tile& g, const float* Ad, const float* xs, int s) {
#pragma unroll
  for (int b = 0; b < 4; ++b) {
    const float4 x = *reinterpret_cast<const float4*>(xs + b * s);
    const float4 q0 = *reinterpret_cast<const float4*>(Ad + b * 8);
    const float4 q1 = *reinterpret_cast<const float4*>(Ad + b * 8 + 4);
    const float2 x01 = make_float2(x.x, x.y), x23 = make_float2(x.z, x.w);
    const float2 a0 = make_float2(q0.x, q0.y), a1 = make_float2(q0.z, q0.w);
    const float2 a2 = make_float2(q1.x, q1.y), a3 = make_float2(q1.z, q1.w);
    g.v[0][0] = ffma2(a0, x01, g.v[0][0]); g.v[0][1] = ffma2(a0, x23, g.v[0][1]);
    g.v[1][0] = ffma2(a1, x01, g.v[1][0]); g.v[1][1] = ffma2(a1, x23, g.v[1][1]);
    g.v[2][0] = ffma2(a2, x01, g.v[2][0]); g.v[2][1] = ffma2(a2, x23, g.v[2][1]);
    g.v[3][0] = ffma2(a3, x01, g.v[3][0]); g.v[3][1] = ffma2(a3, x23, g.v[3][1]);
  }
}
// g[r][a] += sum_b A[a][b] x[r][b]; A column b arrives as (A0b,A1b,A2b,A3b)
__device__ __forceinline__ void f32_cols(F32Tile& g, const float* Ap, const float* xs, int s) {
  float4 q[4];
#pragma unroll
  for (int b = 0; b < 4; ++b) q[b] = *reinterpret_cast<const float4*>(Ap + b * 8);
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    const float4 x = *reinterpret_cast<const float4*>(xs + r * s);
    const float xv[4] = {x.x, x.y, x.z, x.w};
#pragma unroll
    for (int b = 0; b < 4; ++b) {
      const float2 xb = make_float2(xv[b], xv[b]);
      g.v[r][0] = ffma2(make_float2(q[b].x, q[b].y), xb, g.v[r][0]);
      g.v[r][1] = ffma2(make_float2(q[b].z, q[b].w), xb, g.v[r][1]);
    }
  }
}
// Paired subtraction a - b (sub.rn.f32x2).
__device__ __forceinline__ float2 fsub2(float2 a, float2 b) {
  float2 d;
  asm("{\n .reg .b64 ra, rb, rd;\n mov.b64 ra, {%2, %3};\n mov.b64 rb, {%4, %5};\n"
      " sub.rn.f32x2 rd, ra, rb;\n mov.b64 {%0, %1}, rd;\n}"
      : "=f"(d.x), "=f"(d.y)
      : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
  return d;
}
// Kahan-compensated s += v on a column pair (c carries the compensation), on paired adds:
// y = v - c, t = s + y, c = (t - s) - y, s = t, each rounded to nearest as in scalar Kahan.
__device__ __forceinline__ void kahan2(float2& s, float2& c, float2 v) {
  const float2 y = fsub2(v, c);
  const float2 t = __fadd2_rn(s, y);
  c = fsub2(fsub2(t, s), y);
  s = t;
}

// f32_rows visiting the contraction index from `rot` (0..3) on: each output sums the same
// products in the order pt_rows_rot uses (threads whose tiles lie 64 bytes apart then read
// different shared-memory banks)
__device__ __forceinline__ void f32_rank1(F32Tile& g, float4 q0, float4 q1, float4 x) {
  const float2 x01 = make_float2(x.x, x.y), x23 = make_float2(x.z, x.w);
  const float2 a0 = make_float2(q0.x, q0.y), a1 = make_float2(q0.z, q0.w);
  const float2 a2 = make_float2(q1.x, q1.y), a3 = make_float2(q1.z, q1.w);
  g.v[0][0] = ffma2(a0, x01, g.v[0][0]); g.v[0][1] = ffma2(a0, x23, g.v[0][1]);
  g.v[1][0] = ffma2(a1, x01, g.v[1][0]); g.v[1][1] = ffma2(a1, x23, g.v[1][1]);
  g.v[2][0] = ffma2(a2, x01, g.v[2][0]); g.v[2][1] = ffma2(a2, x23, g.v[2][1]);
  g.v[3][0] = ffma2(a3, x01, g.v[3][0]); g.v[3][1] = ffma2(a3, x23, g.v[3][1]);
}
__device__ __forceinline__ void f32_rows_rot(F32Tile& g, const float* Ad, const float* xs, int s, int rot) {
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int b = (i + rot) & 3;
    const float4 x = *reinterpret_cast<const float4*>(xs + b * s);
    const float4 q0 = *reinterpret_cast<const float4*>(Ad + b * 8);
    const float4 q1 = *reinterpret_cast<const float4*>(Ad + b * 8 + 4);
    f32_rank1(g, q0, q1, x);
  }
}
// f32_rows_rot on two tiles with one read of each duplicated operator column
__device__ __forceinline__ void f32_rows_rot2(F32Tile& g0, F32Tile& g1, const float* Ad, const float* x0s,
                                              const float* x1s, int s, int rot) {
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int b = (i + rot) & 3;
    const float4 q0 = *reinterpret_cast<const float4*>(Ad + b * 8);
    const float4 q1 = *reinterpret_cast<const float4*>(Ad + b * 8 + 4);
    const float4 x0 = *reinterpret_cast<const float4*>(x0s + b * s);
    const float4 x1 = *reinterpret_cast<const float4*>(x1s + b * s);
    f32_rank1(g0, q0, q1, x0);
    f32_rank1(g1, q0, q1, x1);
  }
}
// f32_cols on two tiles with one read of the operator block
__device__ __forceinline__ void f32_cols2(F32Tile& g0, F32Tile& g1, const float* Ap, const float* x0s,
                                          const float* x1s, int s) {
  float4 q[4];
#pragma unroll
  for (int b = 0; b < 4; ++b) q[b] = *reinterpret_cast<const float4*>(Ap + b * 8);
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    const float4 x0 = *reinterpret_cast<const float4*>(x0s + r * s);
    const float4 x1 = *reinterpret_cast<const float4*>(x1s + r * s);
    const float xv0[4] = {x0.x, x0.y, x0.z, x0.w}, xv1[4] = {x1.x, x1.y, x1.z, x1.w};
#pragma unroll
    for (int b = 0; b < 4; ++b) {
      g0.v[r][0] = ffma2(make_float2(q[b].x, q[b].y), make_float2(xv0[b], xv0[b]), g0.v[r][0]);
      g0.v[r][1] = ffma2(make_float2(q[b].z, q[b].w), make_float2(xv0[b], xv0[b]), g0.v[r][1]);
      g1.v[r][0] = ffma2(make_float2(q[b].x, q[b].y), make_float2(xv1[b], xv1[b]), g1.v[r][0]);
      g1.v[r][1] = ffma2(make_float2(q[b].z, q[b].w), make_float2(xv1[b], xv1[b]), g1.v[r][1]);
    }
  }
}
// Row r of a tile as the four values along dimension d-1
__device__ __forceinline__ float4 f32_row(const F32Tile& g, int r) {
  return make_float4(g.v[r][0].x, g.v[r][0].y, g.v[r][1].x, g.v[r][1].y);
}
// f32_row for a row index known only at run time (selects, no local memory)
__device__ __forceinline__ float4 f32_row_sel(const F32Tile& g, int r) {
  const float4 r0 = f32_row(g, 0), r1 = f32_row(g, 1), r2 = f32_row(g, 2), r3 = f32_row(g, 3);
  return r == 0 ? r0 : r == 1 ? r1 : r == 2 ? r2 : r3;
}
__device__ __forceinline__ void zero_f32(F32Tile& t) {
#pragma unroll
  for (int r = 0; r < 4; ++r) t.v[r][0] = t.v[r][1] = make_float2(0.f, 0.f);
}

// A group's sums as pairs of operator rows: v[c][p] = (y[2p][c], y[2p+1][c]) with y[r][c]
// row r along the applied dimension m, column c along dimension 5.  For m = 5 the roles swap:
// v[r][p] = (y[r][2p], y[r][2p+1]), the row r along dimension 3.
struct PairTile {
  float2 v[4][2];
};
__device__ __forceinline__ void zero_pt(PairTile& t) {
#pragma unroll
  for (int r = 0; r < 4; ++r) t.v[r][0] = t.v[r][1] = make_float2(0.f, 0.f);
}
__device__ __forceinline__ float2 dup(float x) { return make_float2(x, x); }

// m != 5: y[a][c] += sum_b A[a][b] x[b][c]; x rows s apart, A column b = (A0b, A1b, A2b, A3b)
__device__ __forceinline__ void pt_rows(PairTile& g, const float* A, const float* xs, int s) {
#pragma unroll
  for (int b = 0; b < 4; ++b) {
    const float4 x = *reinterpret_cast<const float4*>(xs + b * s);
    const float4 q = *reinterpret_cast<const float4*>(A + 4 * b);
    const float2 a01 = make_float2(q.x, q.y), a23 = make_float2(q.z, q.w);
    g.v[0][0] = ffma2(a01, dup(x.x), g.v[0][0]); g.v[0][1] = ffma2(a23, dup(x.x), g.v[0][1]);
    g.v[1][0] = ffma2(a01, dup(x.y), g.v[1][0]); g.v[1][1] = ffma2(a23, dup(x.y), g.v[1][1]);
    g.v[2][0] = ffma2(a01, dup(x.z), g.v[2][0]); g.v[2][1] = ffma2(a23, dup(x.z), g.v[2][1]);
    g.v[3][0] = ffma2(a01, dup(x.w), g.v[3][0]); g.v[3][1] = ffma2(a23, dup(x.w), g.v[3][1]);
  }
}
// pt_rows visiting the contraction index from `rot` (0..3) on: the same products summed in a
// rotated order, so that threads whose tiles lie 64 bytes apart read different shared-memory
// banks (the layout of a group on dimension d-2, where a thread's 16 values are contiguous)
__device__ __forceinline__ void pt_rows_rot(PairTile& g, const float* A, const float* xs, int s, int rot) {
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int b = (i + rot) & 3;
    const float4 x = *reinterpret_cast<const float4*>(xs + b * s);
    const float4 q = *reinterpret_cast<const float4*>(A + 4 * b);
    const float2 a01 = make_float2(q.x, q.y), a23 = make_float2(q.z, q.w);
    g.v[0][0] = ffma2(a01, dup(x.x), g.v[0][0]); g.v[0][1] = ffma2(a23, dup(x.x), g.v[0][1]);
    g.v[1][0] = ffma2(a01, dup(x.y), g.v[1][0]); g.v[1][1] = ffma2(a23, dup(x.y), g.v[1][1]);
    g.v[2][0] = ffma2(a01, dup(x.z), g.v[2][0]); g.v[2][1] = ffma2(a23, dup(x.z), g.v[2][1]);
    g.v[3][0] = ffma2(a01, dup(x.w), g.v[3][0]); g.v[3][1] = ffma2(a23, dup(x.w), g.v[3][1]);
  }
}
// One contraction index of pt_rows on a tile: operator column b (pairs a01, a23) times x row b.
__device__ __forceinline__ void pt_rank1(PairTile& g, float2 a01, float2 a23, float4 x) {
  g.v[0][0] = ffma2(a01, dup(x.x), g.v[0][0]); g.v[0][1] = ffma2(a23, dup(x.x), g.v[0][1]);
  g.v[1][0] = ffma2(a01, dup(x.y), g.v[1][0]); g.v[1][1] = ffma2(a23, dup(x.y), g.v[1][1]);
  g.v[2][0] = ffma2(a01, dup(x.z), g.v[2][0]); g.v[2][1] = ffma2(a23, dup(x.z), g.v[2][1]);
  g.v[3][0] = ffma2(a01, dup(x.w), g.v[3][0]); g.v[3][1] = ffma2(a23, dup(x.w), g.v[3][1]);
}
// pt_rows_rot on two tiles (x0s, x1s) with one read of each operator column: each tile sees
// pt_rows_rot's operations in pt_rows_rot's order
__device__ __forceinline__ void pt_rows_rot2(PairTile& g0, PairTile& g1, const float* A, const float* x0s,
                                             const float* x1s, int s, int rot) {
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int b = (i + rot) & 3;
    const float4 q = *reinterpret_cast<const float4*>(A + 4 * b);
    const float4 x0 = *reinterpret_cast<const float4*>(x0s + b * s);
    const float4 x1 = *reinterpret_cast<const float4*>(x1s + b * s);
    const float2 a01 = make_float2(q.x, q.y), a23 = make_float2(q.z, q.w);
    pt_rank1(g0, a01, a23, x0);
    pt_rank1(g1, a01, a23, x1);
  }
}
// m == 5: y[r][a] += sum_b A[a][b] x[r][b]; x rows s apart (natural rows along dimension 3)
__device__ __forceinline__ void pt_cols(PairTile& g, const float* A, const float* xs, int s) {
  float4 q[4];
#pragma unroll
  for (int b = 0; b < 4; ++b) q[b] = *reinterpret_cast<const float4*>(A + 4 * b);
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    const float4 x = *reinterpret_cast<const float4*>(xs + r * s);
    const float xv[4] = {x.x, x.y, x.z, x.w};
#pragma unroll
    for (int b = 0; b < 4; ++b) {
      g.v[r][0] = ffma2(make_float2(q[b].x, q[b].y), dup(xv[b]), g.v[r][0]);
      g.v[r][1] = ffma2(make_float2(q[b].z, q[b].w), dup(xv[b]), g.v[r][1]);
    }
  }
}
// pt_cols on two tiles with one read of the operator block (each tile: pt_cols's order)
__device__ __forceinline__ void pt_cols2(PairTile& g0, PairTile& g1, const float* A, const float* x0s,
                                         const float* x1s, int s) {
  float4 q[4];
#pragma unroll
  for (int b = 0; b < 4; ++b) q[b] = *reinterpret_cast<const float4*>(A + 4 * b);
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    const float4 x0 = *reinterpret_cast<const float4*>(x0s + r * s);
    const float4 x1 = *reinterpret_cast<const float4*>(x1s + r * s);
    const float xv0[4] = {x0.x, x0.y, x0.z, x0.w}, xv1[4] = {x1.x, x1.y, x1.z, x1.w};
#pragma unroll
    for (int b = 0; b < 4; ++b) {
      g0.v[r][0] = ffma2(make_float2(q[b].x, q[b].y), dup(xv0[b]), g0.v[r][0]);
      g0.v[r][1] = ffma2(make_float2(q[b].z, q[b].w), dup(xv0[b]), g0.v[r][1]);
      g1.v[r][0] = ffma2(make_float2(q[b].x, q[b].y), dup(xv1[b]), g1.v[r][0]);
      g1.v[r][1] = ffma2(make_float2(q[b].z, q[b].w), dup(xv1[b]), g1.v[r][1]);
    }
  }
}
// Row r (along the group's dimension; along dimension 3 for m == 5) of a group's sums, as the
// four values of dimension 5.
__device__ __forceinline__ float4 pt_row(const PairTile& g, int r, bool cols) {
  if (cols) return make_float4(g.v[r][0].x, g.v[r][0].y, g.v[r][1].x, g.v[r][1].y);
  const int p = r >> 1;
  return (r & 1) ? make_float4(g.v[0][p].y, g.v[1][p].y, g.v[2][p].y, g.v[3][p].y)
                 : make_float4(g.v[0][p].x, g.v[1][p].x, g.v[2][p].x, g.v[3][p].x);
}

// pt_row(g, r, false) for a row index known only at run time (selects, no local memory).
__device__ __forceinline__ float4 pt_row_sel(const PairTile& g, int r) {
  const float4 r0 = pt_row(g, 0, false), r1 = pt_row(g, 1, false), r2 = pt_row(g, 2, false),
               r3 = pt_row(g, 3, false);
  return r == 0 ? r0 : r == 1 ? r1 : r == 2 ? r2 : r3;
}

}  // namespace asg
