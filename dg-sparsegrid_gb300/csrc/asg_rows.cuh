// Row routines shared by the operator-application kernels and the fused solver kernels.
#pragma once

#include "asg_internal.h"

namespace asg {
namespace {

template <typename T>
__device__ __forceinline__ void acc_add(T& s, T& c, T v, bool kahan) {
  if (kahan) {
    const T yv = v - c;
    const T t = s + yv;
    c = (t - s) - yv;
    s = t;
  } else {
    s += v;
  }
}

// ---------------------------------------------------------------------------------------
// Small-block single-mode rows: every term has one applied factor and deg^d <= 256 (the
// 2-D/3-D configurations).  One warp per output element; the warp's lanes form G groups of
// L lanes (L = min(32, next power of two >= deg^d)), group g taking the row's entries
// g, g+G, ...; lane r of a group owns outputs r, r+L, ...  An entry adds, for each owned
// output o (digit a along the entry's dimension m, stride s), sum_b A[a][b] f_j[o + (b-a) s]:
// P strided loads of f_j and one row of the P x P block, straight from global memory (no
// shared-memory round trip, no barrier per entry), two entries in flight per group.  Group
// sums (Kahan-compensated in FP32) are added across groups by a fixed shuffle tree, so the
// result is deterministic.
// ---------------------------------------------------------------------------------------
// Per-lane constants of the small-block row routines, computed once per kernel: group width
// L (lanes per group), G groups, the lane's group g and rank r, and for each owned output
// o = r + L q the base-P digits of o packed 4 bits per dimension (dimension m at bit 4 m), so
// an entry finds its digit along its dimension without an integer division.
template <int MAXO>
struct SmallLane {
  int L, G, g, r;
  unsigned dig[MAXO];
};

template <typename T, int P, int MAXO>
__device__ __forceinline__ SmallLane<MAXO> small_lane(const ApplyArgs<T>& a, int lane) {
  SmallLane<MAXO> sl;
  const int B = a.B;
  int L = 1;
  while (L < B && L < 32) L <<= 1;
  sl.L = L;
  sl.G = 32 / L;
  sl.g = lane / L;
  sl.r = lane - sl.g * L;
#pragma unroll
  for (int q = 0; q < MAXO; ++q) {
    const int o = sl.r + L * q;
    unsigned d = 0u;
    if (o < B)
      for (int m = 0; m < a.D; ++m) d |= static_cast<unsigned>((o / a.stride[m]) % P) << (4 * m);
    sl.dig[q] = d;
  }
  return sl;
}

// One row of a P x P operator block (P consecutive values, 16-byte aligned for P = 4 and
// 8-byte aligned for P = 2): vector loads where the width allows.
template <typename T, int P>
__device__ __forceinline__ void load_prow(const T* __restrict__ p, T (&v)[P]) {
  if constexpr (sizeof(T) == 4 && P == 4) {
    const float4 t = *reinterpret_cast<const float4*>(p);
    v[0] = t.x;
    v[1] = t.y;
    v[2] = t.z;
    v[3] = t.w;
  } else if constexpr (sizeof(T) == 8 && P == 4) {
    const double2 t0 = reinterpret_cast<const double2*>(p)[0], t1 = reinterpret_cast<const double2*>(p)[1];
    v[0] = t0.x;
    v[1] = t0.y;
    v[2] = t1.x;
    v[3] = t1.y;
  } else if constexpr (sizeof(T) == 4 && P == 2) {
    const float2 t = *reinterpret_cast<const float2*>(p);
    v[0] = t.x;
    v[1] = t.y;
  } else if constexpr (sizeof(T) == 8 && P == 2) {
    const double2 t = *reinterpret_cast<const double2*>(p);
    v[0] = t.x;
    v[1] = t.y;
  } else {
#pragma unroll
    for (int b = 0; b < P; ++b) v[b] = p[b];
  }
}

template <typename T, int P, int MAXO>
__device__ __forceinline__ void small_entry(const ApplyArgs<T>& a, const T* __restrict__ f, const EntryDesc& e,
                                            const SmallLane<MAXO>& sl, int B, T (&v)[MAXO]) {
  const int s = a.stride[e.m];
  const int sh = 4 * e.m;
  const T* fj = f + static_cast<size_t>(e.j) * B;
  const T* Ab = a.ops + e.aoff;
#pragma unroll
  for (int q = 0; q < MAXO; ++q) {
    const int o = sl.r + sl.L * q;
    v[q] = T(0);
    if (o < B) {
      const int ad = static_cast<int>((sl.dig[q] >> sh) & 15u);
      const int base = o - ad * s;
      T arow[P];
      load_prow<T, P>(Ab + ad * P, arow);
      T acc = T(0);
#pragma unroll
      for (int b = 0; b < P; ++b) acc = fma(arow[b], fj[base + b * s], acc);
      v[q] = acc;
    }
  }
}

// Entries [q0, q1) of one row (a whole row, or one chunk of a long row) by one warp, reading
// the input vector f; the B sums go to out[0..B).
template <typename T, int P, int MAXO, bool KAHAN>
__device__ __forceinline__ void small_chunk(const ApplyArgs<T>& a, const T* __restrict__ f, long long q0, long long q1,
                                            const SmallLane<MAXO>& sl, T* out) {
  const int B = a.B, G = sl.G;
  T acc[MAXO], cmp[MAXO];
#pragma unroll
  for (int q = 0; q < MAXO; ++q) acc[q] = cmp[q] = T(0);
  long long q = q0 + sl.g;
  for (; q + G < q1; q += 2 * G) {  // two entries of this group in flight
    const EntryDesc e0 = a.ed[q], e1 = a.ed[q + G];
    T v0[MAXO], v1[MAXO];
    small_entry<T, P, MAXO>(a, f, e0, sl, B, v0);
    small_entry<T, P, MAXO>(a, f, e1, sl, B, v1);
#pragma unroll
    for (int k = 0; k < MAXO; ++k) {
      acc_add(acc[k], cmp[k], v0[k], KAHAN);
      acc_add(acc[k], cmp[k], v1[k], KAHAN);
    }
  }
  if (q < q1) {
    const EntryDesc e0 = a.ed[q];
    T v0[MAXO];
    small_entry<T, P, MAXO>(a, f, e0, sl, B, v0);
#pragma unroll
    for (int k = 0; k < MAXO; ++k) acc_add(acc[k], cmp[k], v0[k], KAHAN);
  }
  // fixed-order tree across the G groups (lane r of group 0 ends with the total)
  for (int off = sl.L; off < 32; off <<= 1) {
#pragma unroll
    for (int k = 0; k < MAXO; ++k) acc[k] += __shfl_down_sync(0xffffffffu, acc[k], off);
  }
  if (sl.g == 0) {
#pragma unroll
    for (int k = 0; k < MAXO; ++k) {
      const int o = sl.r + sl.L * k;
      if (o < B) out[o] = acc[k];
    }
  }
}

template <typename T, int P, int MAXO, bool KAHAN>
__device__ __forceinline__ void small_row(const ApplyArgs<T>& a, int row, const SmallLane<MAXO>& sl) {
  small_chunk<T, P, MAXO, KAHAN>(a, a.f, a.row_ptr[row], a.row_ptr[row + 1], sl, a.y + static_cast<size_t>(row) * a.B);
}

}  // namespace
}  // namespace asg
