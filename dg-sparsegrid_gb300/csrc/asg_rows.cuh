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
// Small-block single-mode rows, per-output form (used for P > 4; the fiber form below serves
// P <= 4): every term has one applied factor and deg^d <= 256.  One warp per output
// element; the warp's lanes form G groups of
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

// ---------------------------------------------------------------------------------------
// Fiber-per-lane small-block rows (P <= 4): lane r of a group owns the fibers phi = r,
// r + 32, ... of the output block along its last dimension (P consecutive values each);
// Lf = deg^(d-1) fibers per block, Gf = 32 / Lf groups per warp (one when Lf > 32), group g
// taking the entries g, g + Gf, ...  An entry along dimension m adds to fiber phi
//   m = d-1:  y[phi P + t] += sum_b A[t][b] f_j[phi P + b]
//   m < d-1:  y[phi P + t] += sum_b A[a][b] f_j[phi P + t + (b - a) s]   (a: phi's digit m)
// -- both as acc[t] += sum_b X[t][b] Y[b][t] over a P x P register tile, X the rows
// (t or a) of the P x P block and Y the input fibers (the one fiber at phi P, or the fibers at
// phi P + (b - a) s), loaded as P-wide vectors, so entries of any dimension run the same
// instructions (no divergence).  Group sums (Kahan-compensated in FP32 where asked) are added
// across groups by a fixed shuffle tree: deterministic.
// ---------------------------------------------------------------------------------------
template <int MAXF>
struct FiberLane {
  int Lf, Gf, g, r;  // fibers per block, groups per warp, this lane's group and rank
  unsigned dig[MAXF];  // base-P digits of each owned fiber's first output, 4 bits per dim
};

template <typename T, int P, int MAXF>
__device__ __forceinline__ FiberLane<MAXF> fiber_lane(const ApplyArgs<T>& a, int lane) {
  FiberLane<MAXF> fl;
  const int Lf = a.B / P;
  fl.Lf = Lf;
  fl.Gf = Lf <= 32 ? 32 / Lf : 1;
  fl.g = Lf <= 32 ? lane / Lf : 0;
  fl.r = Lf <= 32 ? lane - fl.g * Lf : lane;
#pragma unroll
  for (int q = 0; q < MAXF; ++q) {
    const int phi = fl.r + 32 * q;
    unsigned d = 0u;
    if (phi < Lf)
      for (int m = 0; m < a.D; ++m) d |= static_cast<unsigned>((phi * P / a.stride[m]) % P) << (4 * m);
    fl.dig[q] = d;
  }
  return fl;
}

template <typename T, int P>
__device__ __forceinline__ void store_prow(T* __restrict__ p, const T (&v)[P]) {
  if constexpr (sizeof(T) == 4 && P == 4) {
    *reinterpret_cast<float4*>(p) = make_float4(v[0], v[1], v[2], v[3]);
  } else if constexpr (sizeof(T) == 8 && P == 4) {
    reinterpret_cast<double2*>(p)[0] = make_double2(v[0], v[1]);
    reinterpret_cast<double2*>(p)[1] = make_double2(v[2], v[3]);
  } else if constexpr (sizeof(T) == 4 && P == 2) {
    *reinterpret_cast<float2*>(p) = make_float2(v[0], v[1]);
  } else if constexpr (sizeof(T) == 8 && P == 2) {
    *reinterpret_cast<double2*>(p) = make_double2(v[0], v[1]);
  } else {
#pragma unroll
    for (int t = 0; t < P; ++t) p[t] = v[t];
  }
}

// Adds one entry to the lane's fibers (acc[q][t]); lanes of groups past Gf and fibers past
// Lf add nothing.
template <typename T, int P, int MAXF, bool KAHAN>
__device__ __forceinline__ void fiber_entry(const ApplyArgs<T>& a, const T* __restrict__ f, const EntryDesc& e,
                                            const FiberLane<MAXF>& fl, T (&acc)[MAXF][P], T (&cmp)[MAXF][P]) {
  const int B = a.B;
  const bool last = e.m == a.D - 1;
  const int s = a.stride[e.m];
  const int sh = 4 * e.m;
  const T* fj = f + static_cast<size_t>(e.j) * B;
  const T* Ab = a.ops + e.aoff;
#pragma unroll
  for (int q = 0; q < MAXF; ++q) {
    const int phi = fl.r + 32 * q;
    if (phi < fl.Lf) {
      const int ad = static_cast<int>((fl.dig[q] >> sh) & 15u);
      T X[P][P], Y[P][P];
#pragma unroll
      for (int t = 0; t < P; ++t) load_prow<T, P>(Ab + (last ? t : ad) * P, X[t]);
#pragma unroll
      for (int b = 0; b < P; ++b) load_prow<T, P>(fj + phi * P + (last ? 0 : (b - ad) * s), Y[b]);
#pragma unroll
      for (int t = 0; t < P; ++t) {
        T v = T(0);
#pragma unroll
        for (int b = 0; b < P; ++b) v = fma(X[t][b], last ? Y[0][b] : Y[b][t], v);
        acc_add(acc[q][t], cmp[q][t], v, KAHAN);
      }
    }
  }
}

// Entries q0 + gofs + g, q0 + gofs + g + gstride, ... (< q1) of one row by one warp (g: the
// lane's group; a whole row: gofs 0, gstride Gf), reading the input vector f; the warp's B
// sums go to out[0..B) (16-byte aligned for P = 4).
template <typename T, int P, int MAXF, bool KAHAN>
__device__ __forceinline__ void fiber_chunk(const ApplyArgs<T>& a, const T* __restrict__ f, long long q0, long long q1,
                                            const FiberLane<MAXF>& fl, T* out, int gofs = 0, int gstride = 0) {
  T acc[MAXF][P], cmp[MAXF][P];
#pragma unroll
  for (int q = 0; q < MAXF; ++q)
#pragma unroll
    for (int t = 0; t < P; ++t) acc[q][t] = cmp[q][t] = T(0);
  const int step = gstride > 0 ? gstride : fl.Gf;
  if (fl.g < fl.Gf)
    for (long long q = q0 + gofs + fl.g; q < q1; q += step) fiber_entry<T, P, MAXF, KAHAN>(a, f, a.ed[q], fl, acc, cmp);
  // fixed-order tree across the groups: group g takes group g + off's sums (g % 2off == 0)
  const int lane = fl.g * fl.Lf + fl.r;
  for (int off = 1; off < fl.Gf; off <<= 1) {
    const bool take = (fl.g % (2 * off)) == 0 && fl.g + off < fl.Gf;
    const int src = take ? lane + off * fl.Lf : lane;
#pragma unroll
    for (int q = 0; q < MAXF; ++q)
#pragma unroll
      for (int t = 0; t < P; ++t) {
        const T o = __shfl_sync(0xffffffffu, acc[q][t], src);
        if (take) acc[q][t] += o;
      }
  }
  if (fl.g == 0) {
#pragma unroll
    for (int q = 0; q < MAXF; ++q) {
      const int phi = fl.r + 32 * q;
      if (phi < fl.Lf) store_prow<T, P>(out + phi * P, acc[q]);
    }
  }
}


}  // namespace
}  // namespace asg
