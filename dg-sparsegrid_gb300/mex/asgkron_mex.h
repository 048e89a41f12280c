/*
 * Shared part of the MATLAB / GNU Octave MEX gateways of libasgkron (apply_A_mex.c,
 * apply_A_T_mex.c): argument checks in the reference's error style, and one cached plan per
 * gateway keyed on the CONTENTS of its inputs.
 *
 * Inputs common to both gateways (the arguments of apply_A.m:1 that define the operator):
 *   ops     T x d cell of real double matrices, pde.terms{t}.terms_1D{k}.mat for the selected
 *           terms (apply_A.m:19-30, 163-168)
 *   idx1d   N x d real double, A_data.element_local_index_D{k} stacked as columns (1-based,
 *           global_matrix.m:69-70)
 *   deg     the polynomial degree
 *   row_ptr, cols (optional pair): pde.connectivity as CSR -- row_ptr N+1 0-based offsets,
 *           cols 1-based element numbers (connect_nD.m:102-105); absent = all pairs
 *           (opts.use_connectivity = false, apply_A.m:104-108)
 *
 * Plan cache.  Building a plan (structure analysis, work lists, operator upload) costs far
 * more than one application, so the gateway keeps the plan of its last call.  MATLAB may
 * modify an array in place when no other variable shares it, so a data pointer does not
 * identify an operator: the cache key is a 64-bit digest of the operators' values, the
 * index table, the degree and the pair list, recomputed on every call (one pass over the
 * inputs, far cheaper than a rebuild).  A different digest rebuilds the plan.
 */
#ifndef ASGKRON_MEX_H
#define ASGKRON_MEX_H

#include <stdint.h>
#include <stdio.h>
#include <string.h>

#include "asgkron.h"
#include "mex.h"

#define ASGM_MAX_OPS 96 /* T*d <= 16*6 (asg_plan_desc limits) */

typedef struct {
  asg_plan* plan;
  uint64_t key;
  int T, d, N, deg;
} asgm_cache;

static void asgm_fail(const char* gateway, asg_status st) {
  char msg[768];
  asg_last_error(msg, sizeof msg);
  mexErrMsgIdAndTxt("asgkron:apply", "%s: %s (status %d)", gateway, msg, (int)st);
}

static void asgm_args(const char* gateway, const char* what) {
  mexErrMsgIdAndTxt("asgkron:args", "%s: %s", gateway, what);
}

static int asgm_is_real_double(const mxArray* a) { return a && mxIsDouble(a) && !mxIsComplex(a); }

/* 64-bit digest of a byte range, folded into h (word-wise multiply-xorshift mixing). */
static uint64_t asgm_mix(uint64_t h, const void* data, size_t bytes) {
  const unsigned char* p = (const unsigned char*)data;
  size_t i = 0;
  for (; i + 8 <= bytes; i += 8) {
    uint64_t w;
    memcpy(&w, p + i, 8);
    h ^= w;
    h *= 0x9E3779B97F4A7C15ull;
    h ^= h >> 29;
  }
  for (; i < bytes; ++i) {
    h ^= p[i];
    h *= 0x100000001B3ull;
  }
  h ^= (uint64_t)bytes;
  h *= 0xBF58476D1CE4E5B9ull;
  return h ^ (h >> 31);
}

/* Validates ops / idx1d / deg / (row_ptr, cols) and returns the digest of their contents. */
static uint64_t asgm_check_and_key(const char* gateway, const mxArray* ops, const mxArray* idx, const mxArray* degv,
                                   const mxArray* rp, const mxArray* cl, int* T, int* d, int* N, int* deg) {
  if (!ops || !mxIsCell(ops)) asgm_args(gateway, "ops must be a T x d cell of operator matrices");
  *T = (int)mxGetM(ops);
  *d = (int)mxGetN(ops);
  if (*T < 1 || *d < 1 || *T * *d > ASGM_MAX_OPS) asgm_args(gateway, "ops must be T x d with 1 <= T*d <= 96");
  if (!asgm_is_real_double(idx) || (int)mxGetN(idx) != *d)
    asgm_args(gateway, "idx1d must be a real double N x d matrix (d = columns of ops)");
  *N = (int)mxGetM(idx);
  if (!asgm_is_real_double(degv) || mxGetNumberOfElements(degv) != 1) asgm_args(gateway, "deg must be a scalar");
  *deg = (int)mxGetScalar(degv);
  if ((double)*deg != mxGetScalar(degv) || *deg < 1) asgm_args(gateway, "deg must be a positive integer");
  uint64_t h = 0x243F6A8885A308D3ull;
  int hdr[4] = {*T, *d, *N, *deg};
  h = asgm_mix(h, hdr, sizeof hdr);
  for (int t = 0; t < *T; ++t)
    for (int m = 0; m < *d; ++m) {
      const mxArray* a = mxGetCell(ops, (size_t)t + (size_t)m * (size_t)*T); /* cells are column-major */
      if (!asgm_is_real_double(a) || mxGetM(a) != mxGetN(a) || mxGetM(a) == 0)
        asgm_args(gateway, "every ops{t,k} must be a square real double matrix");
      h = asgm_mix(h, mxGetDoubles(a), mxGetNumberOfElements(a) * sizeof(double));
    }
  h = asgm_mix(h, mxGetDoubles(idx), mxGetNumberOfElements(idx) * sizeof(double));
  if (rp || cl) {
    if (!asgm_is_real_double(rp) || !asgm_is_real_double(cl) || mxGetNumberOfElements(rp) != (size_t)*N + 1)
      asgm_args(gateway, "row_ptr must hold N+1 offsets and cols the connected elements (real double)");
    h = asgm_mix(h, mxGetDoubles(rp), mxGetNumberOfElements(rp) * sizeof(double));
    h = asgm_mix(h, mxGetDoubles(cl), mxGetNumberOfElements(cl) * sizeof(double));
  }
  return h;
}

static asgm_cache* g_asgm_cache_for_exit = NULL;
static void asgm_release(void) {
  if (g_asgm_cache_for_exit && g_asgm_cache_for_exit->plan) {
    asg_plan_destroy(g_asgm_cache_for_exit->plan);
    g_asgm_cache_for_exit->plan = NULL;
  }
}

/* The cached plan for these inputs, rebuilt when their digest differs from the cached one. */
static asg_plan* asgm_plan(const char* gateway, asgm_cache* c, const mxArray* ops, const mxArray* idx,
                           const mxArray* degv, const mxArray* rp, const mxArray* cl) {
  int T, d, N, deg;
  const uint64_t key = asgm_check_and_key(gateway, ops, idx, degv, rp, cl, &T, &d, &N, &deg);
  if (c->plan && c->key == key && c->T == T && c->d == d && c->N == N && c->deg == deg) return c->plan;
  if (c->plan) {
    asg_plan_destroy(c->plan);
    c->plan = NULL;
  }
  const double* ptr[ASGM_MAX_OPS];
  int ld[ASGM_MAX_OPS];
  for (int t = 0; t < T; ++t)
    for (int m = 0; m < d; ++m) {
      const mxArray* a = mxGetCell(ops, (size_t)t + (size_t)m * (size_t)T);
      ptr[t * d + m] = mxGetDoubles(a);
      ld[t * d + m] = (int)mxGetM(a);
    }
  int* id = (int*)mxMalloc(sizeof(int) * (size_t)(N > 0 ? N : 1) * (size_t)d); /* row-major N x d */
  const double* iv = mxGetDoubles(idx);
  for (int e = 0; e < N; ++e)
    for (int m = 0; m < d; ++m) id[(size_t)e * d + m] = (int)iv[e + (size_t)m * N];
  asg_plan_desc desc;
  memset(&desc, 0, sizeof desc);
  desc.num_dims = d;
  desc.deg = deg;
  desc.num_terms = T;
  desc.num_elems = N;
  desc.index_base = 1;
  desc.idx1d = id;
  desc.ops = ptr;
  desc.op_ld = ld;
  desc.structure = ASG_STRUCT_DETECT;
  desc.drop_tol = 1e-13;
  long long* rpi = NULL;
  int* cli = NULL;
  if (rp) {
    const size_t P = mxGetNumberOfElements(cl);
    rpi = (long long*)mxMalloc(sizeof(long long) * ((size_t)N + 1));
    cli = (int*)mxMalloc(sizeof(int) * (P > 0 ? P : 1));
    for (int i = 0; i <= N; ++i) rpi[i] = (long long)mxGetDoubles(rp)[i];
    for (size_t q = 0; q < P; ++q) cli[q] = (int)mxGetDoubles(cl)[q];
    desc.row_ptr = rpi;
    desc.cols = cli;
  }
  asg_plan* plan = NULL;
  const asg_status st = asg_plan_create(&desc, &plan); /* copies everything it keeps */
  mxFree(id);
  if (rpi) mxFree(rpi);
  if (cli) mxFree(cli);
  if (st != ASG_OK) asgm_fail(gateway, st);
  c->plan = plan;
  c->key = key;
  c->T = T;
  c->d = d;
  c->N = N;
  c->deg = deg;
  if (!mexIsLocked()) { /* keep the cached plan across calls; destroy it when MATLAB clears the MEX */
    g_asgm_cache_for_exit = c;
    mexLock();
    mexAtExit(asgm_release);
  }
  return plan;
}

/* numel(v) must equal N * deg^d. */
static void asgm_check_vector(const char* gateway, const mxArray* v, const char* name, const asgm_cache* c) {
  size_t block = 1;
  for (int m = 0; m < c->d; ++m) block *= (size_t)c->deg;
  if (!asgm_is_real_double(v) || mxGetNumberOfElements(v) != (size_t)c->N * block) {
    char what[128];
    snprintf(what, sizeof what, "%s must be a real double vector of N*deg^d elements", name);
    asgm_args(gateway, what);
  }
}

#endif /* ASGKRON_MEX_H */
