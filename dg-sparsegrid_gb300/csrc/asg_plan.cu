// Plan creation, structure analysis, work-list construction and the apply entry points of
// the C ABI.  Host-side code (compiled by nvcc for the runtime API); the kernels live in
// asg_apply.cu.
#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <map>
#include <new>
#include <queue>
#include <vector>

#include "asg_internal.h"

namespace asg {

static thread_local char g_err[1024] = "";

asg_status fail(asg_status st, const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
  return st;
}

asg_status cuda_fail(cudaError_t e, const char* what) {
  return fail(ASG_ERR_CUDA, "%s: %s (%s)", what, cudaGetErrorName(e), cudaGetErrorString(e));
}

namespace {

// Replaces *dst (freed first: finalize runs again when a plan's table changes) by a device
// copy of src, or leaves it NULL for an empty src.
template <typename X>
asg_status upload(X** dst, const std::vector<X>& src) {
  cudaFree(*dst);
  *dst = nullptr;
  if (src.empty()) return ASG_OK;
  ASG_CUDA(cudaMalloc(reinterpret_cast<void**>(dst), src.size() * sizeof(X)));
  ASG_CUDA(cudaMemcpy(*dst, src.data(), src.size() * sizeof(X), cudaMemcpyHostToDevice));
  return ASG_OK;
}

void free_device(asg_plan* p);
void free_plan(asg_plan* p) {
  if (!p) return;
  free_device(p);
  delete p;
}
void free_device(asg_plan* p) {
  if (p->tr) {
    free_plan(p->tr);
    p->tr = nullptr;
  }
  cudaFree(p->d_g_ptr);
  cudaFree(p->d_g_contrib);
  cudaFree(p->d_g_tgt);
  cudaFree(p->d_ldg);
  cudaFree(p->d_gptrs);
  cudaFree(p->d_g_items);
  cudaFree(p->d_g_partial);
  cudaFree(p->d_g_counter);
  cudaFree(p->d_idx1d);
  cudaFree(p->d_op_nb);
  cudaFree(p->d_active);
  cudaFree(p->d_op_off);
  cudaFree(p->d_row_ptr);
  cudaFree(p->d_ent);
  cudaFree(p->d_tr_row_ptr);
  cudaFree(p->d_tr_ent);
  cudaFree(p->d_ops64);
  cudaFree(p->d_ops32);
  cudaFree(p->d_ed);
  cudaFree(p->d_row_order);
  for (int k = 0; k < 2; ++k) {
    cudaFree(p->d_cta_ptr[k]);
    cudaFree(p->d_cta_rows[k]);
  }
  cudaFree(p->d_ops_pair);
  cudaFree(p->d_ops_cols);
  cudaFree(p->d_ws);
  for (int k = 0; k < 2; ++k) {
    cudaFree(p->d_fz_int[k]);
    cudaFree(p->d_fz_items[k]);
  }
  cudaFree(p->d_err);
  cudaFree(p->d_bar);
  cudaFree(p->d_io);
  if (p->stream) cudaStreamDestroy(p->stream);
  if (p->hg_exec) cudaGraphExecDestroy(p->hg_exec);
  for (int k = 0; k < 4; ++k) {
    cudaFree(p->d_hc_rows[k]);
    cudaFree(p->d_hc_order[k]);
  }
  for (int k = 0; k < asg_plan::kHostChunks; ++k) {
    if (p->cstream[k]) cudaStreamDestroy(p->cstream[k]);
    if (p->ev_done[k]) cudaEventDestroy(p->ev_done[k]);
  }
  for (cudaEvent_t e : p->ev_in)
    if (e) cudaEventDestroy(e);

}

// Pack operator (t,m) into block-major order: block (a,b) holds the P x P sub-matrix
// rows a*P.., cols b*P.. row-major, so one (row, column) element pair reads P*P
// contiguous values.
void pack_op(const double* op, int ld, int nb, int P, double* dst) {
  for (int a = 0; a < nb; ++a)
    for (int b = 0; b < nb; ++b) {
      double* blk = dst + (static_cast<long long>(a) * nb + b) * P * P;
      for (int r = 0; r < P; ++r)
        for (int c = 0; c < P; ++c)
          blk[r * P + c] = op[static_cast<long long>(b * P + c) * ld + (a * P + r)];
    }
}

void pack_host(asg_plan* p, const double* const* ops, const int* op_ld) {
  p->h64.assign(static_cast<size_t>(p->packed_elems), 0.0);
  for (int t = 0; t < p->T; ++t)
    for (int m = 0; m < p->D; ++m) {
      const int tm = t * p->D + m;
      if (p->op_off[tm] < 0) continue;
      pack_op(ops[tm], op_ld[tm], p->op_nb[tm], p->P, p->h64.data() + p->op_off[tm]);
    }
}

// Uploads the packed blocks in the three device layouts (FP64, FP32, FP32 paired).
asg_status upload_ops(asg_plan* p) {
  const std::vector<double>& h64 = p->h64;
  std::vector<float> h32(h64.size());
  for (size_t i = 0; i < h64.size(); ++i) h32[i] = static_cast<float>(h64[i]);
  if (!p->ed.empty() && p->P == 4) {
    // FP32 blocks for the paired FMA (fma.rn.f32x2): per column b, 8 values.  Blocks used on
    // the last dimension hold (A0b,A1b,A2b,A3b) + padding, all others the duplicated pairs
    // (A0b,A0b,A1b,A1b,A2b,A2b,A3b,A3b).  Block k of a packed operator sits at 32*k.
    std::vector<float> pr(h64.size() * 2, 0.f);
    for (int t = 0; t < p->T; ++t)
      for (int m = 0; m < p->D; ++m) {
        const int tm = t * p->D + m;
        if (p->op_off[tm] < 0) continue;
        const long long nblk = static_cast<long long>(p->op_nb[tm]) * p->op_nb[tm];
        for (long long k = 0; k < nblk; ++k) {
          const double* A = h64.data() + p->op_off[tm] + k * 16;
          float* d = pr.data() + (p->op_off[tm] + k * 16) * 2;
          for (int b = 0; b < 4; ++b)
            for (int r = 0; r < 4; ++r) {
              if (m == p->D - 1) {
                d[b * 8 + r] = static_cast<float>(A[r * 4 + b]);
              } else {
                d[b * 8 + 2 * r] = static_cast<float>(A[r * 4 + b]);
                d[b * 8 + 2 * r + 1] = static_cast<float>(A[r * 4 + b]);
              }
            }
        }
      }
    if (!p->d_ops_pair) ASG_CUDA(cudaMalloc(reinterpret_cast<void**>(&p->d_ops_pair), pr.size() * sizeof(float)));
    ASG_CUDA(cudaMemcpy(p->d_ops_pair, pr.data(), pr.size() * sizeof(float), cudaMemcpyHostToDevice));
    // the same blocks column by column, (A0b, A1b, A2b, A3b) for b = 0..3: the streaming
    // kernel's operator pairs (A0b, A1b), (A2b, A3b) for the paired FMA
    std::vector<float> cols(h64.size());
    for (size_t k = 0; k + 16 <= h64.size(); k += 16)
      for (int b = 0; b < 4; ++b)
        for (int r = 0; r < 4; ++r) cols[k + b * 4 + r] = static_cast<float>(h64[k + r * 4 + b]);
    if (!p->d_ops_cols) ASG_CUDA(cudaMalloc(reinterpret_cast<void**>(&p->d_ops_cols), cols.size() * sizeof(float)));
    ASG_CUDA(cudaMemcpy(p->d_ops_cols, cols.data(), cols.size() * sizeof(float), cudaMemcpyHostToDevice));
  }
  if (!p->d_ops64 && !h64.empty()) {
    ASG_CUDA(cudaMalloc(reinterpret_cast<void**>(&p->d_ops64), h64.size() * sizeof(double)));
    ASG_CUDA(cudaMalloc(reinterpret_cast<void**>(&p->d_ops32), h32.size() * sizeof(float)));
  }
  if (!h64.empty()) {
    ASG_CUDA(cudaMemcpy(p->d_ops64, h64.data(), h64.size() * sizeof(double), cudaMemcpyHostToDevice));
    ASG_CUDA(cudaMemcpy(p->d_ops32, h32.data(), h32.size() * sizeof(float), cudaMemcpyHostToDevice));
  }
  return ASG_OK;
}

// Work streams of the streaming FP32 kernel (one CTA per resident slot).  Rows go to CTAs by
// longest-processing-time assignment of their cost: the 16 KB blocks a row gathers (its own
// block once, plus one per off-diagonal entry) weighted 4, plus 1 per entry (consumer work).
// A row's entries are ordered by applied dimension 0, 1, 2, 4 (through the transpose
// buffers), then 3 and 5 (straight into the natural tile), each group in work-list order.
// Expects p->ed filled.
asg_status build_streams(asg_plan* p, int nsm) {
  const int N = p->N_out;
  const int occ = stream_occupancy();
  if (occ <= 0) return fail(ASG_ERR_CUDA, "streaming apply kernel cannot be resident");
  const int G = std::max(1, std::min(N, occ * nsm));
  std::vector<long long> cost(N);
  for (int i = 0; i < N; ++i) {
    long long gathers = 1, n = p->row_ptr[i + 1] - p->row_ptr[i];
    for (long long q = p->row_ptr[i]; q < p->row_ptr[i + 1]; ++q) gathers += p->ed[q].j != i;
    cost[i] = 4 * gathers + n;
  }
  std::vector<int> by_cost(N);
  for (int i = 0; i < N; ++i) by_cost[i] = i;
  std::stable_sort(by_cost.begin(), by_cost.end(), [&](int x, int y) { return cost[x] > cost[y]; });
  std::vector<std::vector<int>> lists(G);
  std::vector<std::pair<long long, int>> heap;  // (load, cta) min-heap
  for (int c = 0; c < G; ++c) heap.push_back({0, c});
  auto cmp = [](const std::pair<long long, int>& x, const std::pair<long long, int>& y) { return x > y; };
  for (int i : by_cost) {
    std::pop_heap(heap.begin(), heap.end(), cmp);
    auto& top = heap.back();
    lists[top.second].push_back(i);
    top.first += cost[i];
    std::push_heap(heap.begin(), heap.end(), cmp);
  }
  static const int kRank[6] = {0, 1, 2, 4, 3, 5};  // group position of applied dimension m
  long long maxcount = 0;
  std::vector<std::vector<int>> streams(G);
  for (int c = 0; c < G; ++c) {
    std::vector<int>& s = streams[c];
    for (int i : lists[c]) {
      if (p->row_ptr[i + 1] == p->row_ptr[i]) {  // no entries: y block of zeros
        s.insert(s.end(), {i, i, 0, SF_ZERO});
        continue;
      }
      std::vector<long long> q(p->row_ptr[i + 1] - p->row_ptr[i]);
      for (size_t k = 0; k < q.size(); ++k) q[k] = p->row_ptr[i] + static_cast<long long>(k);
      std::stable_sort(q.begin(), q.end(), [&](long long x, long long y) { return kRank[p->ed[x].m] < kRank[p->ed[y].m]; });
      for (size_t k = 0; k < q.size(); ++k) {
        const asg::EntryDesc& e = p->ed[q[k]];
        if (e.aoff % 16 != 0 || e.aoff / 16 > (1LL << 30)) return fail(ASG_ERR_UNSUPPORTED, "operator block offset");
        int fl = e.m;
        if (e.j == i) fl |= SF_SELF;
        if (k == 0) fl |= SF_ROW0;
        if (k + 1 == q.size()) fl |= SF_ROW1;
        if (k == 0 || p->ed[q[k - 1]].m != e.m) fl |= SF_GRP0;
        if (k + 1 == q.size() || p->ed[q[k + 1]].m != e.m) fl |= SF_GRP1;
        s.insert(s.end(), {e.j, i, static_cast<int>(e.aoff / 16), fl});
      }
    }
    maxcount = std::max<long long>(maxcount, static_cast<long long>(s.size() / 4));
  }
  if (maxcount > (1LL << 28)) return fail(ASG_ERR_UNSUPPORTED, "work stream too long");
  const int stride = 1 + static_cast<int>((maxcount + 31) / 32) * 32;
  p->ws.assign(static_cast<size_t>(G) * stride * 4, 0);
  for (int c = 0; c < G; ++c) {
    int* dst = p->ws.data() + static_cast<size_t>(c) * stride * 4;
    dst[0] = static_cast<int>(streams[c].size() / 4);
    std::copy(streams[c].begin(), streams[c].end(), dst + 4);
  }
  p->ws_stride = stride;
  p->ws_ctas = G;
  return ASG_OK;
}

// The cached graph of the chunked host apply (it names the plan's buffers and kernel).
void drop_host_graph(asg_plan* p) {
  if (p->hg_exec) cudaGraphExecDestroy(p->hg_exec);
  p->hg_exec = nullptr;
  p->hg_f = p->hg_y = p->hg_kf = p->hg_ky = nullptr;
  p->hg_kind = -1;
  p->hg_es = 0;
  p->hg_repeat = 0;
}

// What a plan derives from its table on first use (the transpose, gradient targets, the fused
// solve's partition) and the tuner's choice: dropped when the table changes.
void drop_derived(asg_plan* p) {
  if (p->tr) {
    free_plan(p->tr);
    p->tr = nullptr;
  }
  for (void** d : {reinterpret_cast<void**>(&p->d_g_ptr), reinterpret_cast<void**>(&p->d_g_contrib),
                   reinterpret_cast<void**>(&p->d_g_tgt), reinterpret_cast<void**>(&p->d_ldg),
                   reinterpret_cast<void**>(&p->d_gptrs), reinterpret_cast<void**>(&p->d_g_items),
                   reinterpret_cast<void**>(&p->d_g_partial), reinterpret_cast<void**>(&p->d_g_counter)}) {
    cudaFree(*d);
    *d = nullptr;
  }
  p->g_ptr.clear();
  p->g_contrib.clear();
  p->g_tgt.clear();
  p->g_items.clear();
  for (int k = 0; k < 2; ++k) {
    cudaFree(p->d_fz_int[k]);
    cudaFree(p->d_fz_items[k]);
    p->d_fz_int[k] = nullptr;
    p->d_fz_items[k] = nullptr;
    p->fz_G[k] = p->fz_max_rows[k] = p->fz_max_slots[k] = 0;
    p->tuned_kind[k] = -1;
  }
  for (int k = 0; k < 4; ++k) {
    cudaFree(p->d_hc_rows[k]);
    cudaFree(p->d_hc_order[k]);
    p->d_hc_rows[k] = p->d_hc_order[k] = nullptr;
    p->hc_estart[k].clear();
    p->hc_start[k].clear();
  }
  drop_host_graph(p);
}

// Kernel choice, launch order, single-mode descriptors and every upload; shared by a plan
// and its transpose.  Expects idx1d, op_nb, active, op_off, row_ptr, ent and h64 filled.
// Output rows are elements [0, N_out); `ops` false keeps the device operator copies.
asg_status finalize(asg_plan* p, bool ops) {
  const int D = p->D, P = p->P, T = p->T, N = p->N, NO = p->N_out;
  const long long B = p->B;
  const bool detect = p->structure == ASG_STRUCT_DETECT;
  std::vector<int>& ent = p->ent;
  double pd1 = 1.0;
  for (int k = 0; k <= D; ++k) pd1 *= P;
  p->flops_exec = 0.0;
  for (int i = 0; i < N; ++i)
    for (long long q = p->row_ptr[i]; q < p->row_ptr[i + 1]; ++q)
      p->flops_exec += 2.0 * pd1 * __builtin_popcount(p->active[ent[q] & 15]);
  // single_terms: every term has exactly one applied factor (advection/diffusion terms once
  // the mass factors are the identity); single: additionally a large block for the fiber kernels
  bool single_terms = detect && N > 0;
  for (int t = 0; t < T; ++t)
    if (__builtin_popcount(p->active[t]) != 1) single_terms = false;
  const bool single = single_terms && (P == 3 || P == 4) && B >= 32LL * P * P;
  p->kernel_kind = single ? ((P == 4 && B == 4096) ? KK_SINGLE_TMA : KK_SINGLE_MODE)
                          : (B <= 256 ? (single_terms ? KK_SINGLE_SMALL : KK_CHAIN_WARP) : KK_CHAIN_CTA);
  p->row_order.clear();
  p->ed.clear();
  if (single) {
    // rows launch longest first so the last wave is made of short rows
    p->row_order.resize(NO);
    for (int i = 0; i < NO; ++i) p->row_order[i] = i;
    std::stable_sort(p->row_order.begin(), p->row_order.end(), [&](int x, int y) {
      return p->row_ptr[x + 1] - p->row_ptr[x] > p->row_ptr[y + 1] - p->row_ptr[y];
    });
  }
  if (single_terms) {
    // per-entry descriptors of the single-mode kernels: column, dimension, block offset
    p->ed.resize(ent.size());
    for (int i = 0; i < N; ++i)
      for (long long q = p->row_ptr[i]; q < p->row_ptr[i + 1]; ++q) {
        const int j = ent[q] >> 4, t = ent[q] & 15;
        const int m = __builtin_ctz(p->active[t]);
        const int tm = t * D + m;
        p->ed[q].j = j;
        p->ed[q].m = m;
        p->ed[q].aoff = p->op_off[tm] + (static_cast<long long>(p->idx1d[i * D + m]) * p->op_nb[tm] +
                                         p->idx1d[j * D + m]) * P * P;
      }
  }
  // persistent single-mode kernel: per precision, a longest-processing-time assignment of
  // rows (cost = entries + 1) to the resident CTAs, each CTA's rows longest first
  for (int k = 0; k < 2; ++k) {
    p->cta_ptr[k].clear();
    p->cta_rows[k].clear();
  }
  int nsm = 0;
  if (single && P == 4 && B == 4096 && NO > 0) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return cuda_fail(e, "device attributes");
  }
  if (single && P == 4 && B == 4096 && NO > 0) {
    for (int k = 0; k < 2; ++k) {
      const int occ = single_tma_rows_occupancy(k == 0 ? 8 : 4);
      if (occ <= 0) return fail(ASG_ERR_CUDA, "persistent single-mode kernel cannot be resident");
      const int G = std::max(1, std::min(NO, occ * nsm));
      std::vector<std::vector<int>> lists(G);
      std::vector<std::pair<long long, int>> heap;  // (load, cta) min-heap
      for (int c = 0; c < G; ++c) heap.push_back({0, c});
      auto cmp = [](const std::pair<long long, int>& x, const std::pair<long long, int>& y) { return x > y; };
      std::vector<int> by_cost(NO);
      for (int i = 0; i < NO; ++i) by_cost[i] = i;
      std::stable_sort(by_cost.begin(), by_cost.end(), [&](int x, int y) {
        return p->row_ptr[x + 1] - p->row_ptr[x] > p->row_ptr[y + 1] - p->row_ptr[y];
      });
      for (int i : by_cost) {
        std::pop_heap(heap.begin(), heap.end(), cmp);
        auto& top = heap.back();
        lists[top.second].push_back(i);
        top.first += p->row_ptr[i + 1] - p->row_ptr[i] + 1;
        std::push_heap(heap.begin(), heap.end(), cmp);
      }
      p->cta_ptr[k].push_back(0);
      for (int c = 0; c < G; ++c) {
        p->cta_rows[k].insert(p->cta_rows[k].end(), lists[c].begin(), lists[c].end());
        p->cta_ptr[k].push_back(static_cast<int>(p->cta_rows[k].size()));
      }
    }
  }
  p->ws.clear();
  p->ws_stride = p->ws_ctas = 0;
  if (single && P == 4 && B == 4096 && NO > 0) {
    asg_status sst = build_streams(p, nsm);
    if (sst) return sst;
  }
  asg_status st;
  if ((st = upload(&p->d_ws, p->ws))) return st;
  for (int k = 0; k < 2; ++k) {
    if ((st = upload(&p->d_cta_ptr[k], p->cta_ptr[k]))) return st;
    if ((st = upload(&p->d_cta_rows[k], p->cta_rows[k]))) return st;
  }
  if ((st = upload(&p->d_row_order, p->row_order))) return st;
  if (ops && (st = upload_ops(p))) return st;
  if ((st = upload(&p->d_idx1d, p->idx1d))) return st;
  if ((st = upload(&p->d_op_nb, p->op_nb))) return st;
  if ((st = upload(&p->d_active, p->active))) return st;
  if ((st = upload(&p->d_op_off, p->op_off))) return st;
  if ((st = upload(&p->d_row_ptr, p->row_ptr))) return st;
  if ((st = upload(&p->d_ent, p->ent))) return st;
  if ((st = upload(&p->d_ed, p->ed))) return st;
  if (!p->d_err) ASG_CUDA(cudaMalloc(reinterpret_cast<void**>(&p->d_err), sizeof(int)));
  if (!p->d_bar) ASG_CUDA(cudaMalloc(reinterpret_cast<void**>(&p->d_bar), 4 * sizeof(unsigned)));
  ASG_CUDA(cudaMemset(p->d_err, 0, sizeof(int)));
  return ASG_OK;
}

// The transposed plan: A^T has block (j, i) = kron_d (A_td^T)[J_d(j), I_d(i)], so it is
// the same operator application with every packed block (a, b) replaced by block (b, a)
// transposed and the work list transposed (row j collects the entries (i, t) that had column
// j).  Structure classes (zero / identity) are invariant under transposition.
asg_status build_transpose(asg_plan* p) {
  if (p->tr) return ASG_OK;
  asg_plan* t = new (std::nothrow) asg_plan;
  if (!t) return fail(ASG_ERR_NOMEM, "transpose: out of host memory");
  t->D = p->D;
  t->P = p->P;
  t->T = p->T;
  t->N = p->N;
  t->B = p->B;
  t->structure = p->structure;
  t->drop_tol = p->drop_tol;
  t->idx1d = p->idx1d;
  t->op_nb = p->op_nb;
  t->active = p->active;
  t->op_off = p->op_off;
  t->packed_elems = p->packed_elems;
  t->pairs = p->pairs;
  t->flops_dense = p->flops_dense;
  const int P = p->P, PP = P * P;
  t->h64.assign(p->h64.size(), 0.0);
  for (int tm = 0; tm < p->T * p->D; ++tm) {
    if (p->op_off[tm] < 0) continue;
    const int nb = p->op_nb[tm];
    const double* src = p->h64.data() + p->op_off[tm];
    double* dst = t->h64.data() + p->op_off[tm];
    for (int a = 0; a < nb; ++a)
      for (int b = 0; b < nb; ++b)
        for (int r = 0; r < P; ++r)
          for (int c = 0; c < P; ++c)
            dst[(static_cast<long long>(a) * nb + b) * PP + r * P + c] =
                src[(static_cast<long long>(b) * nb + a) * PP + c * P + r];
  }
  // CSR transpose of the work list (row order of the forward plan preserved per column)
  const int N = p->N;
  t->row_ptr.assign(N + 1, 0);
  for (int e : p->ent) t->row_ptr[(e >> 4) + 1]++;
  for (int i = 0; i < N; ++i) t->row_ptr[i + 1] += t->row_ptr[i];
  t->ent.assign(p->ent.size(), 0);
  std::vector<long long> fill(t->row_ptr.begin(), t->row_ptr.end() - 1);
  for (int i = 0; i < N; ++i)
    for (long long q = p->row_ptr[i]; q < p->row_ptr[i + 1]; ++q) {
      const int j = p->ent[q] >> 4, term = p->ent[q] & 15;
      t->ent[fill[j]++] = (i << 4) | term;
    }
  if (p->structure == ASG_STRUCT_DETECT)  // single-mode kernels walk a row's entries term by term
    for (int j = 0; j < N; ++j)
      std::stable_sort(t->ent.begin() + t->row_ptr[j], t->ent.begin() + t->row_ptr[j + 1],
                       [](int x, int y) { return (x & 15) < (y & 15); });
  t->N_out = t->N;
  asg_status st = finalize(t, true);
  if (st) {
    free_plan(t);
    return st;
  }
  p->tr = t;
  return ASG_OK;
}

asg_status check_ptr(const void* ptr, const char* name);

// Gradient targets: every (t, k, alpha, beta) block of an applied factor that some work
// entry touches, with its contributing entries in work-list order (deterministic sums).
// The derivative with respect to factor k is nonzero even where k's own block is zero, so the
// contributors are all listed pairs whose identity dimensions match and whose other applied
// factors have nonzero blocks (not only the forward work entries).
asg_status build_grad(asg_plan* p) {
  if (p->d_g_ptr) return ASG_OK;
  const int D = p->D, N = p->N;
  std::map<long long, std::vector<GradContrib>> tg;
  auto blk_zero = [&](int t, int m, int i, int j) {
    const auto& zb = p->zero_blk[t * D + m];
    return !zb.empty() && zb[static_cast<size_t>(p->idx1d[i * D + m]) * p->op_nb[t * D + m] + p->idx1d[j * D + m]];
  };
  auto add = [&](int i, int j, int t) {
    for (int m = 0; m < D; ++m)
      if (!((p->active[t] >> m) & 1u) && p->idx1d[i * D + m] != p->idx1d[j * D + m]) return;
    for (int k = 0; k < D; ++k) {
      if (!((p->active[t] >> k) & 1u)) continue;
      bool others_nonzero = true;
      for (int m = 0; m < D && others_nonzero; ++m)
        if (m != k && ((p->active[t] >> m) & 1u) && blk_zero(t, m, i, j)) others_nonzero = false;
      if (!others_nonzero) continue;
      const long long key = (static_cast<long long>(t * D + k) << 48) |
                            (static_cast<long long>(p->idx1d[i * D + k]) << 24) | p->idx1d[j * D + k];
      tg[key].push_back({i, j, t, k});
    }
  };
  for (int t = 0; t < p->T; ++t) {
    if (p->all_pairs) {
      std::map<std::vector<int>, std::vector<int>> groups;  // columns by identity-dimension indices
      for (int e = 0; e < N; ++e) {
        std::vector<int> key;
        for (int m = 0; m < D; ++m)
          if (!((p->active[t] >> m) & 1u)) key.push_back(p->idx1d[e * D + m]);
        groups[key].push_back(e);
      }
      for (int i = 0; i < N; ++i) {
        std::vector<int> key;
        for (int m = 0; m < D; ++m)
          if (!((p->active[t] >> m) & 1u)) key.push_back(p->idx1d[i * D + m]);
        for (int j : groups[key]) add(i, j, t);
      }
    } else {
      for (int i = 0; i < N; ++i)
        for (long long q = p->pr_ptr[i]; q < p->pr_ptr[i + 1]; ++q) add(i, p->pr_col[q], t);
    }
  }
  p->g_ptr.assign(1, 0);
  p->g_contrib.clear();
  p->g_tgt.clear();
  for (auto& kv : tg) {
    p->g_tgt.push_back({static_cast<int>(kv.first >> 48), static_cast<int>((kv.first >> 24) & 0xFFFFFF),
                        static_cast<int>(kv.first & 0xFFFFFF)});
    p->g_contrib.insert(p->g_contrib.end(), kv.second.begin(), kv.second.end());
    p->g_ptr.push_back(static_cast<long long>(p->g_contrib.size()));
  }
  // terms with one applied factor at deg 4: chunked kernel (items of up to 8 contributors)
  bool single = p->P == 4;
  for (int t = 0; t < p->T; ++t) single = single && __builtin_popcount(p->active[t]) == 1;
  p->g_items.clear();
  if (single) {
    for (size_t g = 0; g < p->g_tgt.size(); ++g) {
      const int first = static_cast<int>(p->g_items.size());
      const long long c0 = p->g_ptr[g], c1 = p->g_ptr[g + 1];
      const int count = static_cast<int>((c1 - c0 + 7) / 8);
      for (long long c = c0; c < c1; c += 8)
        p->g_items.push_back({static_cast<int>(g), static_cast<int>(c), static_cast<int>(std::min(c + 8, c1)), first,
                              count});
    }
  }
  asg_status st;
  if ((st = upload(&p->d_g_ptr, p->g_ptr))) return st;
  if ((st = upload(&p->d_g_contrib, p->g_contrib))) return st;
  if ((st = upload(&p->d_g_tgt, p->g_tgt))) return st;
  if (!p->g_items.empty()) {
    if ((st = upload(&p->d_g_items, p->g_items))) return st;
    ASG_CUDA(cudaMalloc(&p->d_g_partial, p->g_items.size() * 16 * sizeof(double)));
    ASG_CUDA(cudaMalloc(reinterpret_cast<void**>(&p->d_g_counter), p->g_tgt.size() * sizeof(int)));
    ASG_CUDA(cudaMemset(p->d_g_counter, 0, p->g_tgt.size() * sizeof(int)));
  }
  ASG_CUDA(cudaMalloc(reinterpret_cast<void**>(&p->d_ldg), sizeof(int) * p->T * D));
  ASG_CUDA(cudaMalloc(reinterpret_cast<void**>(&p->d_gptrs), sizeof(void*) * p->T * D));
  return ASG_OK;
}

template <typename T>
asg_status grad_ops(asg_plan* p, const T* f, const T* r, T* const* G, const int* ldg, void* stream) {
  if (!p || !G || !ldg) return fail(ASG_ERR_INVALID, "grad_ops: NULL argument");
  ASG_NOT_SLICE(p, "grad_ops");
  asg_status st = check_ptr(f, "f");
  if (st) return st;
  if ((st = check_ptr(r, "r"))) return st;
  for (int tm = 0; tm < p->T * p->D; ++tm)
    if (G[tm] && p->op_off[tm] >= 0 && ldg[tm] < p->op_nb[tm] * p->P)
      return fail(ASG_ERR_INVALID, "grad_ops: ldg[%d]=%d < %d", tm, ldg[tm], p->op_nb[tm] * p->P);
  if ((st = build_grad(p))) return st;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  std::vector<void*> gp(p->T * p->D);
  for (int tm = 0; tm < p->T * p->D; ++tm) gp[tm] = p->op_off[tm] >= 0 ? static_cast<void*>(G[tm]) : nullptr;
  ASG_CUDA(cudaMemcpyAsync(p->d_gptrs, gp.data(), sizeof(void*) * gp.size(), cudaMemcpyHostToDevice, s));
  ASG_CUDA(cudaMemcpyAsync(p->d_ldg, ldg, sizeof(int) * gp.size(), cudaMemcpyHostToDevice, s));
  GradArgs<T> a{};
  a.f = f;
  a.r = r;
  a.ops = sizeof(T) == 8 ? reinterpret_cast<const T*>(p->d_ops64) : reinterpret_cast<const T*>(p->d_ops32);
  a.op_off = p->d_op_off;
  a.op_nb = p->d_op_nb;
  a.idx1d = p->d_idx1d;
  a.active = p->d_active;
  a.tgt_ptr = p->d_g_ptr;
  a.contrib = p->d_g_contrib;
  a.tgt = p->d_g_tgt;
  a.G = reinterpret_cast<T* const*>(p->d_gptrs);
  a.ldg = p->d_ldg;
  a.ntgt = static_cast<int>(p->g_tgt.size());
  a.D = p->D;
  a.B = p->B;
  if (!p->g_items.empty()) {
    a.items = p->d_g_items;
    a.nitems = static_cast<int>(p->g_items.size());
    a.partial = static_cast<T*>(p->d_g_partial);
    a.counter = p->d_g_counter;
  }
  int sd = 1;
  for (int m = p->D - 1; m >= 0; --m) {
    a.stride[m] = sd;
    sd *= p->P;
  }
  cudaError_t e = launch_grad<T>(a, p->P, s);
  if (e != cudaSuccess) return cuda_fail(e, "grad kernel launch");
  // the pointer/ld tables are read by the kernel: keep the host arrays alive until the copy
  // is done (pageable copies are staged before cudaMemcpyAsync returns)
  return ASG_OK;
}

template <typename T>
ApplyArgs<T> make_args(const asg_plan* p, const T* f, T* y, const T* ops) {
  ApplyArgs<T> a{};
  a.f = f;
  a.y = y;
  a.ops = ops;
  a.op_off = p->d_op_off;
  a.op_nb = p->d_op_nb;
  a.idx1d = p->d_idx1d;
  a.row_ptr = p->d_row_ptr;
  a.ent = p->d_ent;
  a.active = p->d_active;
  a.N = p->N_out;  // rows the kernels write
  a.D = p->D;
  a.B = p->B;
  a.nterms = p->T;
  a.ed = p->d_ed;
  a.err = p->d_err;
  a.ops_pair = p->d_ops_pair;
  a.ops_cols = p->d_ops_cols;
  a.row_order = p->d_row_order;
  const int pk = sizeof(T) == 4 ? 1 : 0;
  a.cta_ptr = p->d_cta_ptr[pk];
  a.cta_rows = p->d_cta_rows[pk];
  a.nctas = p->cta_ptr[pk].empty() ? 0 : static_cast<int>(p->cta_ptr[pk].size()) - 1;
  int s = 1;
  for (int m = p->D - 1; m >= 0; --m) {
    a.stride[m] = s;
    s *= p->P;
  }
  return a;
}

asg_status check_ptr(const void* ptr, const char* name) {
  if (!ptr) return fail(ASG_ERR_INVALID, "%s is NULL", name);
  if (reinterpret_cast<uintptr_t>(ptr) & 15) return fail(ASG_ERR_INVALID, "%s must be 16-byte aligned", name);
  return ASG_OK;
}

// The kernel family a precision runs: the tuned choice when asg_plan_tune made one, else the
// plan's kind (whose FP64 side is kind 3 for the FP32-only kinds 7 and 8).
template <typename T>
int effective_kind(const asg_plan* p) {
  const int t = p->tuned_kind[sizeof(T) == 4 ? 1 : 0];
  const int k = t >= 0 ? t : p->kernel_kind;
  return ((k == KK_STREAM || k == KK_SINGLE_TMA_X2) && sizeof(T) == 8) ? KK_SINGLE_TMA : k;
}

// y -= s over n values: the residual step of the kernel families that store A f only.
template <typename T>
__global__ void k_sub_inplace(T* __restrict__ y, const T* __restrict__ s, long long n) {
  for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<long long>(gridDim.x) * blockDim.x)
    y[i] -= s[i];
}

// y = A f, or with ysub (laid out like y, not aliasing it) the residual y = A f - ysub: in the
// apply's own stores for the single-mode bulk-copy, fiber and streaming kinds (2, 3, 4, 5, 7,
// 8), by a second launch for the chain and small-block kinds (0, 1, 6), whose register
// budgets the extra operand would change.  Either way y = (A f) - ysub, rounded once.
template <typename T>
asg_status apply_dev(asg_plan* p, const T* f, T* y, void* stream, const T* ysub = nullptr) {
  if (!p) return fail(ASG_ERR_INVALID, "apply: NULL plan");
  asg_status st = check_ptr(f, "f");
  if (st) return st;
  st = check_ptr(y, "y");
  if (st) return st;
  if (f == y) return fail(ASG_ERR_INVALID, "apply: f and y must not alias");
  const int kind = effective_kind<T>(p);
  if (kind == KK_STREAM && sizeof(T) == 4) {
    StreamArgs sa{};
    sa.f = reinterpret_cast<const float*>(f);
    sa.y = reinterpret_cast<float*>(y);
    sa.ysub = reinterpret_cast<const float*>(ysub);
    sa.ops_cols = p->d_ops_cols;
    sa.ws = reinterpret_cast<const int4*>(p->d_ws);
    sa.ws_stride = p->ws_stride;
    sa.nctas = p->ws_ctas;
    sa.err = p->d_err;
    cudaError_t e = launch_stream(sa, static_cast<cudaStream_t>(stream));
    if (e != cudaSuccess) return cuda_fail(e, "apply kernel launch");
    return ASG_OK;
  }
  const T* ops = sizeof(T) == 8 ? reinterpret_cast<const T*>(p->d_ops64) : reinterpret_cast<const T*>(p->d_ops32);
  ApplyArgs<T> a = make_args<T>(p, f, y, ops);
  const bool second = ysub && (kind == KK_CHAIN_WARP || kind == KK_CHAIN_CTA || kind == KK_SINGLE_SMALL);
  a.ysub = second ? nullptr : ysub;
  cudaError_t e = launch_apply<T>(a, p->P, kind, static_cast<cudaStream_t>(stream));
  if (e != cudaSuccess) return cuda_fail(e, "apply kernel launch");
  if (second) {
    const long long n = static_cast<long long>(p->N_out) * p->B;
    const int grid = static_cast<int>(std::min<long long>((n + 255) / 256, 152 * 8));
    if (n > 0) k_sub_inplace<T><<<grid, 256, 0, static_cast<cudaStream_t>(stream)>>>(y, ysub, n);
    if ((e = cudaGetLastError()) != cudaSuccess) return cuda_fail(e, "residual kernel launch");
  }
  return ASG_OK;
}

template <typename T>
asg_status apply_residual(asg_plan* p, const T* f, const T* ystar, T* r, void* stream) {
  if (!p) return fail(ASG_ERR_INVALID, "apply_residual: NULL plan");
  asg_status st = check_ptr(ystar, "ystar");
  if (st) return st;
  if (ystar == f || ystar == r) return fail(ASG_ERR_INVALID, "apply_residual: ystar must alias neither f nor r");
  return apply_dev<T>(p, f, r, stream, ystar);
}

// Element chunks of the host-pointer apply (see asg_plan::hc_estart), per precision and
// arrival order.  Contiguous (g = 0): the table from its end (its coarsest elements, which
// rows of every level read) towards its start, one copy per chunk.  Gathered (g = 1, f
// page-locked): the row with the fewest elements still to come next, bringing them, so that
// rows become ready -- and their y starts over the link -- while f is still arriving.  A row
// is ready with the chunk that brings the last of its elements (itself and its columns).
// Chunk sizes, each the fastest of the splits measured on the continuity6 workload (a
// repeated 1.0 leaves the last chunk empty: no copy, no rows): contiguous FP32 N/2, N/4,
// 3N/20, N/10, FP64 (whose apply outlasts the copy, so it gains from starting earlier) 2N/5,
// 3N/10, N/5, N/10; gathered FP32 3N/10, N/4, N/5, 3N/20, N/10 (98 us with four chunks,
// 92 us with these five), FP64 3N/10, N/4, N/4, N/5 (311 us; 339 us with FP32's five).
asg_status host_chunks(asg_plan* p, int prec, bool gathered) {
  const int sch = 2 * gathered + prec;
  if (!p->hc_start[sch].empty()) return ASG_OK;
  const int N = p->N, K = asg_plan::kHostChunks;
  static const double kFracs[4][K] = {
      {0.4, 0.7, 0.9, 1.0, 1.0}, {0.5, 0.75, 0.9, 1.0, 1.0}, {0.3, 0.55, 0.8, 1.0, 1.0}, {0.3, 0.55, 0.75, 0.9, 1.0}};
  const double* kFrac = kFracs[sch];
  auto len = [&](int i) { return p->row_ptr[i + 1] - p->row_ptr[i]; };
  std::vector<int> order;
  order.reserve(N);
  if (!gathered) {
    for (int i = N - 1; i >= 0; --i) order.push_back(i);
  } else {
    // next, the row with the fewest elements still to come (ties: the lowest row), which
    // brings those elements, highest-numbered first
    std::vector<std::vector<int>> elems(N), users(N);
    for (int i = 0; i < N; ++i) {
      elems[i].push_back(i);
      for (long long q = p->row_ptr[i]; q < p->row_ptr[i + 1]; ++q) elems[i].push_back(p->ent[q] >> 4);
      std::sort(elems[i].begin(), elems[i].end(), [](int x, int y) { return x > y; });
      elems[i].erase(std::unique(elems[i].begin(), elems[i].end()), elems[i].end());
      for (int j : elems[i]) users[j].push_back(i);
    }
    std::vector<int> miss(N);
    std::vector<char> in(N, 0), done(N, 0);
    using Key = std::pair<int, int>;
    std::priority_queue<Key, std::vector<Key>, std::greater<Key>> heap;
    for (int i = 0; i < N; ++i) {
      miss[i] = static_cast<int>(elems[i].size());
      heap.push({miss[i], i});
    }
    while (!heap.empty()) {
      const Key top = heap.top();
      heap.pop();
      const int i = top.second;
      if (done[i] || top.first != miss[i]) continue;  // finished, or a stale key
      done[i] = 1;
      for (int j : elems[i])
        if (!in[j]) {
          in[j] = 1;
          order.push_back(j);
          for (int u : users[j])
            if (!done[u]) {
              --miss[u];
              heap.push({miss[u], u});
            }
        }
    }
  }
  std::vector<int> pos(N), estart(K + 1, 0);
  for (int k = 0; k < N; ++k) pos[order[k]] = k;
  for (int c = 0; c < K; ++c) estart[c + 1] = std::min(N, static_cast<int>(std::lround(N * kFrac[c])));
  estart[K] = N;
  std::vector<std::vector<int>> rows(K);
  for (int i = 0; i < N; ++i) {
    int last = pos[i];
    for (long long q = p->row_ptr[i]; q < p->row_ptr[i + 1]; ++q) last = std::max(last, pos[p->ent[q] >> 4]);
    int c = 0;
    while (last >= estart[c + 1]) ++c;
    rows[c].push_back(i);
  }
  std::vector<int> all, start(1, 0);
  for (int c = 0; c < K; ++c) {
    std::stable_sort(rows[c].begin(), rows[c].end(), [&](int x, int y) { return len(x) > len(y); });
    all.insert(all.end(), rows[c].begin(), rows[c].end());
    start.push_back(static_cast<int>(all.size()));
  }
  asg_status st = upload(&p->d_hc_rows[sch], all);
  if (!st && gathered) st = upload(&p->d_hc_order[sch], order);
  if (st) return st;
  for (int k = 0; k < asg_plan::kHostChunks; ++k) {
    if (!p->cstream[k]) ASG_CUDA(cudaStreamCreateWithFlags(&p->cstream[k], cudaStreamNonBlocking));
    if (!p->ev_done[k]) ASG_CUDA(cudaEventCreateWithFlags(&p->ev_done[k], cudaEventDisableTiming));
  }
  for (int c = 0; c < K; ++c)
    if (!p->ev_in[c]) ASG_CUDA(cudaEventCreateWithFlags(&p->ev_in[c], cudaEventDisableTiming));
  p->hc_estart[sch] = estart;
  p->hc_start[sch] = start;
  return ASG_OK;
}

// Copies the f blocks of elements order[0 .. gridDim.x) from page-locked host memory (its
// device alias) to the device, one CTA per block of vec 16-byte words: each thread issues
// its eight loads before its stores, so a CTA keeps 16 KB of reads in flight over the link.
constexpr int kGatherThreads = 128;
__global__ void __launch_bounds__(kGatherThreads) k_gather_blocks(const int* __restrict__ order, int vec,
                                                                   const uint4* src, uint4* __restrict__ dst) {
  const size_t base = static_cast<size_t>(order[blockIdx.x]) * vec;
  for (int v0 = 0; v0 < vec; v0 += 8 * kGatherThreads) {
    uint4 r[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      const int v = v0 + u * kGatherThreads + static_cast<int>(threadIdx.x);
      if (v < vec) r[u] = src[base + v];
    }
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      const int v = v0 + u * kGatherThreads + static_cast<int>(threadIdx.x);
      if (v < vec) dst[base + v] = r[u];
    }
  }
}

// The device alias of page-locked host memory the runtime knows (cudaHostAlloc /
// cudaHostRegister), or NULL.
const void* host_pinned(const void* h) {
  cudaPointerAttributes at{};
  if (cudaPointerGetAttributes(&at, h) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  return at.type == cudaMemoryTypeHost ? at.devicePointer : nullptr;
}

// The chunked host apply on the plan's streams: f by element chunks on p->stream (copies,
// or with kf -- f's device alias -- the gather kernel), each chunk's ready rows on the
// chunk's own compute stream once the chunk has landed (so no chunk's rows wait for an
// earlier chunk's last rows), then (y not mapped) one copy of y back; joined on p->stream.
// No synchronisation (capturable).
template <typename T>
asg_status host_pipeline(asg_plan* p, int kind, const T* hf, const T* kf, T* df, T* hy, T* ky, T* dy, size_t ny) {
  const int K = asg_plan::kHostChunks, N = p->N, pk = sizeof(T) == 4 ? 1 : 0, sch = 2 * (kf != nullptr) + pk;
  const std::vector<int>& estart = p->hc_estart[sch];
  const std::vector<int>& start = p->hc_start[sch];
  const int vec = static_cast<int>(static_cast<size_t>(p->B) * sizeof(T) / 16);
  for (int c = 0; c < K; ++c) {
    const int a = estart[c], b = estart[c + 1];
    if (b > a && kf) {
      k_gather_blocks<<<b - a, kGatherThreads, 0, p->stream>>>(p->d_hc_order[sch] + a, vec,
                                                               reinterpret_cast<const uint4*>(kf),
                                                               reinterpret_cast<uint4*>(df));
      cudaError_t e = cudaGetLastError();
      if (e != cudaSuccess) return cuda_fail(e, "f gather launch");
    } else if (b > a) {  // positions [a, b) of the reversed table: elements [N - b, N - a)
      const size_t e0 = static_cast<size_t>(N - b) * p->B, e1 = static_cast<size_t>(N - a) * p->B;
      ASG_CUDA(cudaMemcpyAsync(df + e0, hf + e0, (e1 - e0) * sizeof(T), cudaMemcpyHostToDevice, p->stream));
    }
    ASG_CUDA(cudaEventRecord(p->ev_in[c], p->stream));
  }
  const T* ops = sizeof(T) == 8 ? reinterpret_cast<const T*>(p->d_ops64) : reinterpret_cast<const T*>(p->d_ops32);
  for (int c = 0; c < K; ++c) {
    cudaStream_t cs = p->cstream[c];
    ASG_CUDA(cudaStreamWaitEvent(cs, p->ev_in[c], 0));
    const int r0 = start[c], r1 = start[c + 1];
    if (r1 > r0) {
      ApplyArgs<T> a = make_args<T>(p, df, ky, ops);
      a.N = r1 - r0;  // one CTA per listed row
      a.row_order = p->d_hc_rows[sch] + r0;
      cudaError_t e = launch_apply<T>(a, p->P, kind, cs);
      if (e != cudaSuccess) return cuda_fail(e, "apply kernel launch");
    }
  }
  for (int k = 0; k < K; ++k) {
    ASG_CUDA(cudaEventRecord(p->ev_done[k], p->cstream[k]));
    ASG_CUDA(cudaStreamWaitEvent(p->stream, p->ev_done[k], 0));
  }
  if (ky == dy) ASG_CUDA(cudaMemcpyAsync(hy, dy, ny * sizeof(T), cudaMemcpyDeviceToHost, p->stream));
  return ASG_OK;
}

template <typename T>
asg_status apply_host(asg_plan* p, const T* hf, T* hy) {
  if (!p) return fail(ASG_ERR_INVALID, "apply_host: NULL plan");
  if (!hf || !hy) return fail(ASG_ERR_INVALID, "apply_host: NULL host buffer");
  const size_t n = static_cast<size_t>(p->N) * p->B, ny = static_cast<size_t>(p->N_out) * p->B;
  const size_t need = (n + ny) * sizeof(T) + 256;
  if (!p->stream) ASG_CUDA(cudaStreamCreateWithFlags(&p->stream, cudaStreamNonBlocking));
  if (p->d_io_bytes < need) {
    cudaFree(p->d_io);
    p->d_io = nullptr;
    p->d_io_bytes = 0;
    ASG_CUDA(cudaMalloc(&p->d_io, need));
    p->d_io_bytes = need;
  }
  T* df = static_cast<T*>(p->d_io);
  T* dy = reinterpret_cast<T*>(reinterpret_cast<char*>(p->d_io) + ((n * sizeof(T) + 255) / 256) * 256);
  // A page-locked, device-mapped y (cudaHostAlloc / cudaHostRegister) is written by the kernel
  // itself: each row's block leaves over the host link as soon as the row is done, so the
  // device-to-host transfer overlaps the apply instead of following it.  The kernels store y
  // with plain stores, once per value, so the result is the same as through the copy.
  cudaPointerAttributes at{};
  T* ky = dy;
  if (cudaPointerGetAttributes(&at, hy) == cudaSuccess && at.type == cudaMemoryTypeHost && at.devicePointer &&
      (reinterpret_cast<uintptr_t>(at.devicePointer) & 15) == 0)
    ky = static_cast<T*>(at.devicePointer);
  else
    cudaGetLastError();  // clear a query error for host memory the runtime does not know
  // The one-CTA-per-row bulk-copy kernels (kinds 3, 4, 8; kind 5 runs kind 3's arithmetic)
  // take a row list, so the copy of f can overlap the apply: f comes in by element chunks
  // on the plan's stream, and each chunk's ready rows launch on the chunk's compute stream as
  // soon as their last block has landed, writing y (over the host link when y is mapped)
  // while later chunks are still arriving.  Same kernel per row, same result.
  int kind = effective_kind<T>(p);
  if (kind == KK_SINGLE_TMA_ROWS) kind = KK_SINGLE_TMA;
  if ((kind == KK_SINGLE_TMA || kind == KK_SINGLE_TMA3 || kind == KK_SINGLE_TMA_X2) && p->N_out == p->N &&
      p->N >= 4 * asg_plan::kHostChunks) {
    // A page-locked f with a 16-byte aligned alias arrives in the gathered order (read by a
    // kernel from the mapped buffer); any other f by copies of contiguous chunks (continuity6:
    // FP32 97 us gathered against 104 us contiguous, FP64 312 us against 346 us).
    const void* kf = host_pinned(hf);
    const T* gf = kf && (reinterpret_cast<uintptr_t>(kf) & 15) == 0 && (p->B * sizeof(T)) % 16 == 0
                      ? static_cast<const T*>(kf)
                      : nullptr;
    asg_status st = host_chunks(p, sizeof(T) == 4 ? 1 : 0, gf != nullptr);
    if (st) return st;
    // A caller that repeats its page-locked buffers (a time loop) gets the whole pipeline as one
    // graph launch instead of ~20 runtime calls: captured at the second call with the same f, y,
    // kernel and precision, replayed from the third.  The key holds the host pointers and their
    // device aliases: a buffer freed and registered again at the same address must not replay
    // a graph made for the old registration.
    const bool pinned = kf != nullptr && ky != dy;
    const bool same = pinned && p->hg_f == hf && p->hg_y == hy && p->hg_kf == kf && p->hg_ky == ky &&
                      p->hg_kind == kind && p->hg_es == sizeof(T);
    if (same && p->hg_exec) {
      ASG_CUDA(cudaGraphLaunch(p->hg_exec, p->stream));
      ASG_CUDA(cudaStreamSynchronize(p->stream));
      return ASG_OK;
    }
    if (same && ++p->hg_repeat >= 1) {
      cudaGraph_t g = nullptr;
      cudaGraphExec_t ge = nullptr;
      cudaError_t e = cudaStreamBeginCapture(p->stream, cudaStreamCaptureModeThreadLocal);
      if (e == cudaSuccess) {
        st = host_pipeline<T>(p, kind, hf, gf, df, hy, ky, dy, ny);
        e = cudaStreamEndCapture(p->stream, &g);  // ends the capture whatever the pipeline returned
        if (st) {
          if (g) cudaGraphDestroy(g);
          return st;
        }
      }
      if (e == cudaSuccess) e = cudaGraphInstantiate(&ge, g, 0);
      if (g) cudaGraphDestroy(g);
      if (e == cudaSuccess) {
        drop_host_graph(p);
        p->hg_exec = ge;
        p->hg_f = hf;
        p->hg_y = hy;
        p->hg_kf = kf;
        p->hg_ky = ky;
        p->hg_kind = kind;
        p->hg_es = sizeof(T);
        ASG_CUDA(cudaGraphLaunch(p->hg_exec, p->stream));
        ASG_CUDA(cudaStreamSynchronize(p->stream));
        return ASG_OK;
      }
      cudaGetLastError();  // capture unavailable: run the pipeline directly from now on
      p->hg_repeat = -1000000;
    }
    if (!same) {
      drop_host_graph(p);
      if (pinned) {
        p->hg_f = hf;
        p->hg_y = hy;
        p->hg_kf = kf;
        p->hg_ky = ky;
        p->hg_kind = kind;
        p->hg_es = sizeof(T);
      }
    }
    if ((st = host_pipeline<T>(p, kind, hf, gf, df, hy, ky, dy, ny))) return st;
    ASG_CUDA(cudaStreamSynchronize(p->stream));
    return ASG_OK;
  }
  ASG_CUDA(cudaMemcpyAsync(df, hf, n * sizeof(T), cudaMemcpyHostToDevice, p->stream));
  asg_status st = apply_dev<T>(p, df, ky, p->stream);
  if (st) return st;
  if (ky == dy) ASG_CUDA(cudaMemcpyAsync(hy, dy, ny * sizeof(T), cudaMemcpyDeviceToHost, p->stream));
  ASG_CUDA(cudaStreamSynchronize(p->stream));
  return ASG_OK;
}

}  // namespace

template <typename T>
bool small_plan_args(const asg_plan* p, ApplyArgs<T>* out) {
  if (!p || p->kernel_kind != KK_SINGLE_SMALL || p->ed.size() != p->ent.size() || p->N == 0) return false;
  const T* ops = sizeof(T) == 8 ? reinterpret_cast<const T*>(p->d_ops64) : reinterpret_cast<const T*>(p->d_ops32);
  *out = make_args<T>(p, nullptr, nullptr, ops);
  return true;
}
template bool small_plan_args<float>(const asg_plan*, ApplyArgs<float>*);
template bool small_plan_args<double>(const asg_plan*, ApplyArgs<double>*);

namespace {

// Checks of a plan description shared by plan creation and the element-table update (the isok
// checks of kron_multd.m:7-12,24-28 and the asserts of apply_A.m).
asg_status check_desc(const asg_plan_desc* desc) {
  const int D = desc->num_dims, P = desc->deg, T = desc->num_terms, N = desc->num_elems;
  if (D < 1 || D > kMaxDims)
    return fail(D < 1 ? ASG_ERR_INVALID : ASG_ERR_UNSUPPORTED, "kron_multd: invalid nkron=%d (1..%d supported)", D,
                kMaxDims);
  if (P < 1 || P > 8) return fail(P < 1 ? ASG_ERR_INVALID : ASG_ERR_UNSUPPORTED, "deg=%d outside 1..8", P);
  if (T < 1 || T > kMaxTerms)
    return fail(T < 1 ? ASG_ERR_INVALID : ASG_ERR_UNSUPPORTED, "num_terms=%d outside 1..%d", T, kMaxTerms);
  if (N < 0 || N >= (1 << 27)) return fail(ASG_ERR_UNSUPPORTED, "num_elems=%d outside 0..2^27-1", N);
  long long B = 1;
  for (int k = 0; k < D; ++k) B *= P;
  if (B > kMaxBlock) return fail(ASG_ERR_UNSUPPORTED, "deg^d=%lld exceeds %d", B, kMaxBlock);
  if (desc->index_base != 0 && desc->index_base != 1) return fail(ASG_ERR_INVALID, "index_base must be 0 or 1");
  if (desc->structure != ASG_STRUCT_NONE && desc->structure != ASG_STRUCT_DETECT)
    return fail(ASG_ERR_INVALID, "unknown structure mode %d", desc->structure);
  if (!(desc->drop_tol >= 0.0) || desc->drop_tol > 1e-3) return fail(ASG_ERR_INVALID, "drop_tol must be in [0, 1e-3]");
  if (N > 0 && (!desc->idx1d || !desc->ops || !desc->op_ld)) return fail(ASG_ERR_INVALID, "plan_create: NULL array");
  return ASG_OK;
}

// 0-based 1-D indices of a table; nb_dim[m] = 1 + the largest index in dimension m.
asg_status set_table(asg_plan* p, const int* idx1d, int base, std::vector<int>& nb_dim) {
  const int D = p->D, N = p->N;
  p->idx1d.resize(static_cast<size_t>(N) * D);
  nb_dim.assign(D, 0);
  for (long long i = 0; i < static_cast<long long>(N) * D; ++i) {
    const int v = idx1d[i] - base;
    if (v < 0) return fail(ASG_ERR_INVALID, "idx1d[%lld]=%d below index base %d", i, idx1d[i], base);
    p->idx1d[i] = v;
    nb_dim[i % D] = std::max(nb_dim[i % D], v + 1);
  }
  return ASG_OK;
}

// The listed pairs (validated, 0-based), or all N^2 pairs when row_ptr is NULL.
asg_status set_pairs(asg_plan* p, const long long* row_ptr, const int* cols, int base) {
  const int N = p->N;
  p->pr_ptr.clear();
  p->pr_col.clear();
  if (!row_ptr) {
    p->all_pairs = true;
    p->pairs = static_cast<long long>(N) * N;
    return ASG_OK;
  }
  if (row_ptr[0] != 0) return fail(ASG_ERR_INVALID, "row_ptr[0] must be 0");
  for (int i = 0; i < N; ++i)
    if (row_ptr[i + 1] < row_ptr[i]) return fail(ASG_ERR_INVALID, "row_ptr not monotone at %d", i);
  if (row_ptr[N] > 0 && !cols) return fail(ASG_ERR_INVALID, "cols is NULL");
  for (long long q = 0; q < row_ptr[N]; ++q) {
    const int j = cols[q] - base;
    if (j < 0 || j >= N) return fail(ASG_ERR_INVALID, "cols[%lld]=%d outside the element table", q, cols[q]);
  }
  p->all_pairs = false;
  p->pairs = row_ptr[N];
  p->pr_ptr.assign(row_ptr, row_ptr + N + 1);
  p->pr_col.resize(row_ptr[N]);
  for (long long q = 0; q < row_ptr[N]; ++q) p->pr_col[q] = cols[q] - base;
  return ASG_OK;
}

// Operator validation and structure analysis (identity factors, zero p x p blocks): fills
// op_nb (the packed extent: nb_dim blocks per side), active and zero_blk.
asg_status analyse_ops(asg_plan* p, const asg_plan_desc* desc, const std::vector<int>& nb_dim) {
  const int D = p->D, P = p->P, T = p->T, N = p->N;
  p->op_nb.assign(static_cast<size_t>(T) * D, 0);
  p->op_off.assign(static_cast<size_t>(T) * D, -1);
  p->active.assign(T, 0u);
  std::vector<std::vector<uint8_t>>& zero_blk = p->zero_blk;
  zero_blk.assign(static_cast<size_t>(T) * D, {});
  const bool detect = desc->structure == ASG_STRUCT_DETECT;
  for (int t = 0; t < T; ++t)
    for (int m = 0; m < D; ++m) {
      const int tm = t * D + m;
      const int nb = nb_dim[m];
      p->op_nb[tm] = nb;
      if (N == 0) continue;
      const double* op = desc->ops[tm];
      const int ld = desc->op_ld[tm];
      if (!op) return fail(ASG_ERR_INVALID, "operator (term %d, dim %d) is NULL", t, m);
      if (ld < nb * P)
        return fail(ASG_ERR_INVALID, "operator (term %d, dim %d): ld=%d < deg*max(idx1d)=%d", t, m, ld, nb * P);
      const int n = nb * P;
      double maxabs = 0.0;
      for (int c = 0; c < n; ++c)
        for (int r = 0; r < n; ++r) {
          const double v = op[static_cast<long long>(c) * ld + r];
          if (!std::isfinite(v))
            return fail(ASG_ERR_INVALID, "operator (term %d, dim %d) has a non-finite entry at (%d,%d)", t, m, r, c);
          maxabs = std::max(maxabs, std::fabs(v));
        }
      bool ident = false;
      if (detect) {
        const double thr = desc->drop_tol * maxabs;
        ident = true;
        for (int c = 0; c < n && ident; ++c)
          for (int r = 0; r < n; ++r)
            if (std::fabs(op[static_cast<long long>(c) * ld + r] - (r == c ? 1.0 : 0.0)) > thr) {
              ident = false;
              break;
            }
        if (!ident) {
          auto& zb = zero_blk[tm];
          zb.assign(static_cast<size_t>(nb) * nb, 1);
          for (int c = 0; c < n; ++c)
            for (int r = 0; r < n; ++r)
              if (std::fabs(op[static_cast<long long>(c) * ld + r]) > thr) zb[static_cast<size_t>(r / P) * nb + c / P] = 0;
        }
      }
      if (!ident) p->active[t] |= 1u << m;
    }
  long long off = 0;
  for (int t = 0; t < T; ++t)
    for (int m = 0; m < D; ++m) {
      const int tm = t * D + m;
      if (N == 0 || !((p->active[t] >> m) & 1u)) continue;
      p->op_off[tm] = off;
      off += static_cast<long long>(p->op_nb[tm]) * p->op_nb[tm] * P * P;
    }
  p->packed_elems = off;
  return ASG_OK;
}

// Work entries of rows [r0, r1) (the reference work model, or the structured one under
// ASG_STRUCT_DETECT): p->row_ptr over those rows (r1 - r0 + 1 values), p->ent with table
// column ids.  Summation order: a row's terms in order, each term's columns in list order.
void build_work(asg_plan* p, int r0, int r1) {
  const int D = p->D, T = p->T, N = p->N;
  const bool detect = p->structure == ASG_STRUCT_DETECT;
  p->row_ptr.assign(static_cast<size_t>(r1 - r0) + 1, 0);
  std::vector<int>& ent = p->ent;
  ent.clear();
  auto blk_zero = [&](int t, int m, int i, int j) {
    const auto& zb = p->zero_blk[t * D + m];
    return !zb.empty() && zb[static_cast<size_t>(p->idx1d[i * D + m]) * p->op_nb[t * D + m] + p->idx1d[j * D + m]];
  };
  auto keep = [&](int t, int i, int j) {
    for (int m = 0; m < D; ++m) {
      if ((p->active[t] >> m) & 1u) {
        if (blk_zero(t, m, i, j)) return false;
      } else if (p->idx1d[i * D + m] != p->idx1d[j * D + m]) {
        return false;
      }
    }
    return true;
  };
  if (!detect) {
    for (int t = 0; t < T; ++t) p->active[t] = (1u << D) - 1u;
    for (int i = r0; i < r1; ++i) {
      const long long q0 = p->all_pairs ? 0 : p->pr_ptr[i];
      const long long q1 = p->all_pairs ? N : p->pr_ptr[i + 1];
      for (long long q = q0; q < q1; ++q) {
        const int j = p->all_pairs ? static_cast<int>(q) : p->pr_col[q];
        for (int t = 0; t < T; ++t) ent.push_back((j << 4) | t);
      }
      p->row_ptr[i - r0 + 1] = static_cast<long long>(ent.size());
    }
    return;
  }
  // group candidate columns by the 1-D indices of the term's identity dimensions
  std::vector<std::map<std::vector<int>, std::vector<int>>> groups(T);
  if (p->all_pairs) {
    for (int t = 0; t < T; ++t)
      for (int e = 0; e < N; ++e) {
        std::vector<int> key;
        for (int m = 0; m < D; ++m)
          if (!((p->active[t] >> m) & 1u)) key.push_back(p->idx1d[e * D + m]);
        groups[t][key].push_back(e);
      }
  }
  for (int i = r0; i < r1; ++i) {
    for (int t = 0; t < T; ++t) {
      if (p->all_pairs) {
        std::vector<int> key;
        for (int m = 0; m < D; ++m)
          if (!((p->active[t] >> m) & 1u)) key.push_back(p->idx1d[i * D + m]);
        for (int j : groups[t][key])
          if (keep(t, i, j)) ent.push_back((j << 4) | t);
      } else {
        for (long long q = p->pr_ptr[i]; q < p->pr_ptr[i + 1]; ++q) {
          const int j = p->pr_col[q];
          if (keep(t, i, j)) ent.push_back((j << 4) | t);
        }
      }
    }
    p->row_ptr[i - r0 + 1] = static_cast<long long>(ent.size());
  }
}

// Renumbers a row slice's plan: elements become the rows r0..r1-1 (ids 0..R-1) followed by the
// halo, every other element the rows' entries read, in table order (ids R..R+H-1; rows without
// entries).  Expects build_work(p, r0, r1) done on the table's ids.
void compact_slice(asg_plan* p, int r0, int r1) {
  const int D = p->D, R = r1 - r0, Nt = p->N;
  std::vector<int> id(Nt, -1);
  for (int i = r0; i < r1; ++i) id[i] = i - r0;
  std::vector<uint8_t> used(Nt, 0);
  for (int e : p->ent) used[e >> 4] = 1;
  p->elem_global.clear();
  for (int i = r0; i < r1; ++i) p->elem_global.push_back(i);
  for (int j = 0; j < Nt; ++j)
    if (used[j] && id[j] < 0) {
      id[j] = static_cast<int>(p->elem_global.size());
      p->elem_global.push_back(j);
    }
  const int Ne = static_cast<int>(p->elem_global.size());
  std::vector<int> idx(static_cast<size_t>(Ne) * D);
  for (int e = 0; e < Ne; ++e)
    for (int m = 0; m < D; ++m) idx[static_cast<size_t>(e) * D + m] = p->idx1d[static_cast<size_t>(p->elem_global[e]) * D + m];
  p->idx1d.swap(idx);
  for (int& e : p->ent) e = (id[e >> 4] << 4) | (e & 15);
  p->row_ptr.resize(static_cast<size_t>(Ne) + 1, p->row_ptr[R]);  // halo elements: no entries
  long long listed = 0;
  for (int i = r0; i < r1; ++i) listed += p->all_pairs ? Nt : p->pr_ptr[i + 1] - p->pr_ptr[i];
  p->pairs = listed;
  p->all_pairs = false;  // listed pairs are not kept for a slice (no adjoint or gradients)
  p->pr_ptr.clear();
  p->pr_col.clear();
  p->N = Ne;
  p->N_out = R;
}

}  // namespace

// Plan over rows [r0, r1) of the table (r0 = 0, r1 = num_elems: the whole table); op_blocks
// (may be NULL) widens the packed operator extent per dimension.
asg_status create_plan(const asg_plan_desc* desc, int r0, int r1, const int* op_blocks, asg_plan** out) {
  if (!desc || !out) return fail(ASG_ERR_INVALID, "plan_create: NULL argument");
  *out = nullptr;
  asg_status st = check_desc(desc);
  if (st) return st;
  const int N = desc->num_elems;
  if (r0 < 0 || r1 < r0 || r1 > N) return fail(ASG_ERR_INVALID, "plan_create_ex: rows [%d, %d) outside 0..%d", r0, r1, N);
  const int base = desc->index_base;
  asg_plan* p = new (std::nothrow) asg_plan;
  if (!p) return fail(ASG_ERR_NOMEM, "plan_create: out of host memory");
  p->D = desc->num_dims;
  p->P = desc->deg;
  p->T = desc->num_terms;
  p->N = N;
  p->N_out = N;
  long long B = 1;
  for (int k = 0; k < p->D; ++k) B *= p->P;
  p->B = static_cast<int>(B);
  p->structure = desc->structure;
  p->drop_tol = desc->drop_tol;
  p->index_base = base;
  auto bail = [&](asg_status s) {
    free_device(p);
    delete p;
    return s;
  };
  std::vector<int> nb_dim;
  if ((st = set_table(p, desc->idx1d, base, nb_dim))) return bail(st);
  if (op_blocks)
    for (int m = 0; m < p->D; ++m) {
      if (op_blocks[m] < 0 || op_blocks[m] > (1 << 20))
        return bail(fail(ASG_ERR_INVALID, "plan_create_ex: op_blocks[%d]=%d", m, op_blocks[m]));
      nb_dim[m] = std::max(nb_dim[m], op_blocks[m]);
    }
  if ((st = analyse_ops(p, desc, nb_dim))) return bail(st);
  if ((st = set_pairs(p, desc->row_ptr, desc->cols, base))) return bail(st);
  build_work(p, r0, r1);
  const bool slice = r0 != 0 || r1 != N;
  if (slice) compact_slice(p, r0, r1);
  pack_host(p, desc->ops, desc->op_ld);
  double pd1 = 1.0;
  for (int k = 0; k <= p->D; ++k) pd1 *= p->P;
  p->flops_dense = static_cast<double>(p->pairs) * p->T * p->D * 2.0 * pd1;
  if ((st = finalize(p, true))) return bail(st);
  *out = p;
  return ASG_OK;
}

// A new element table and pair list on a plan's operators (the plan rebuild after adapt.m's
// coarsening and refinement, adapt.m:414-437, when the operators keep their values): the
// structure classes, packed operators and their device copies are kept; the work list, the
// launch data and everything derived from the table are rebuilt.
asg_status update_elements(asg_plan* p, int num_elems, const int* idx1d, const long long* row_ptr, const int* cols) {
  if (!p) return fail(ASG_ERR_INVALID, "plan_update_elements: NULL plan");
  if (p->N_out != p->N) return fail(ASG_ERR_UNSUPPORTED, "plan_update_elements: not for a row-slice plan");
  if (num_elems < 0 || num_elems >= (1 << 27)) return fail(ASG_ERR_UNSUPPORTED, "num_elems=%d outside 0..2^27-1", num_elems);
  if (num_elems > 0 && !idx1d) return fail(ASG_ERR_INVALID, "plan_update_elements: NULL idx1d");
  const int D = p->D;
  // validate against the packed extent before touching the plan
  for (long long i = 0; i < static_cast<long long>(num_elems) * D; ++i) {
    const int v = idx1d[i] - p->index_base;
    if (v < 0) return fail(ASG_ERR_INVALID, "idx1d[%lld]=%d below index base %d", i, idx1d[i], p->index_base);
    const int m = static_cast<int>(i % D);
    for (int t = 0; t < p->T; ++t)
      if (v >= p->op_nb[t * D + m])
        return fail(ASG_ERR_CAPACITY,
                    "plan_update_elements: 1-D index %d in dimension %d beyond the plan's operators (%d blocks); "
                    "create a new plan", v + p->index_base, m, p->op_nb[t * D + m]);
  }
  asg_plan tmp;  // validated pair list first, so a failure leaves the plan unchanged
  tmp.N = num_elems;
  asg_status st = set_pairs(&tmp, row_ptr, cols, p->index_base);
  if (st) return st;
  std::vector<int> nb_dim;
  p->N = p->N_out = num_elems;
  set_table(p, idx1d, p->index_base, nb_dim);
  p->all_pairs = tmp.all_pairs;
  p->pairs = tmp.pairs;
  p->pr_ptr.swap(tmp.pr_ptr);
  p->pr_col.swap(tmp.pr_col);
  build_work(p, 0, num_elems);
  double pd1 = 1.0;
  for (int k = 0; k <= D; ++k) pd1 *= p->P;
  p->flops_dense = static_cast<double>(p->pairs) * p->T * D * 2.0 * pd1;
  drop_derived(p);
  return finalize(p, false);
}

}  // namespace asg

using asg::fail;


namespace asg_tune {
// The kernel families asg_plan_set_kernel accepts for this plan.
std::vector<int> candidate_kinds(asg_plan* p) {
  std::vector<int> out;
  const int saved = p->kernel_kind;
  const int t0 = p->tuned_kind[0], t1 = p->tuned_kind[1];
  for (int k = 0; k <= 8; ++k) {
    if (asg_plan_set_kernel(p, k) == ASG_OK) out.push_back(k);
  }
  p->kernel_kind = saved;
  p->tuned_kind[0] = t0;
  p->tuned_kind[1] = t1;
  asg::fail(ASG_OK, "");  // the refusals above are not this call's error
  return out;
}

template <typename T>
asg_status tune_plan(asg_plan* p, cudaStream_t s, int* best_kind, float* best_ms, float* default_ms) {
  const size_t n = static_cast<size_t>(p->N) * p->B;
  T* buf = nullptr;
  ASG_CUDA(cudaMalloc(reinterpret_cast<void**>(&buf), 2 * n * sizeof(T) + 256));
  T* f = buf;
  T* y = reinterpret_cast<T*>(reinterpret_cast<char*>(buf) + ((n * sizeof(T) + 255) / 256) * 256);
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  asg_status st = ASG_OK;
  cudaError_t ce = cudaMemsetAsync(f, 0, n * sizeof(T), s);
  if (ce == cudaSuccess) ce = cudaEventCreate(&e0);
  if (ce == cudaSuccess) ce = cudaEventCreate(&e1);
  if (ce != cudaSuccess) st = asg::cuda_fail(ce, "plan_tune: setup");
  const int prec = sizeof(T) == 4 ? 1 : 0;
  const int def = asg::effective_kind<T>(p);
  std::vector<int> kinds = st ? std::vector<int>() : candidate_kinds(p);
  float best = 0.f, at_def = 0.f;
  int arg = def;
  for (int k : kinds) {
    p->tuned_kind[prec] = k;
    if (asg::effective_kind<T>(p) != k) continue;  // an FP32-only family in FP64
    constexpr int kReps = 10;
    for (int r = 0; r < 2 && !st; ++r) st = asg::apply_dev<T>(p, f, y, s);
    if (!st && (ce = cudaEventRecord(e0, s)) != cudaSuccess) st = asg::cuda_fail(ce, "plan_tune");
    for (int r = 0; r < kReps && !st; ++r) st = asg::apply_dev<T>(p, f, y, s);
    if (!st && (ce = cudaEventRecord(e1, s)) != cudaSuccess) st = asg::cuda_fail(ce, "plan_tune");
    if (!st && (ce = cudaEventSynchronize(e1)) != cudaSuccess) st = asg::cuda_fail(ce, "plan_tune");
    float ms = 0.f;
    if (!st && (ce = cudaEventElapsedTime(&ms, e0, e1)) != cudaSuccess) st = asg::cuda_fail(ce, "plan_tune");
    if (st) break;
    ms /= kReps;
    if (k == def) at_def = ms;
    if (best == 0.f || ms < best) {
      best = ms;
      arg = k;
    }
  }
  p->tuned_kind[prec] = st ? -1 : arg;
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  cudaFree(buf);
  if (st) return st;
  int dev_status = 0;
  if ((st = asg_plan_device_status(p, &dev_status))) return st;
  if (dev_status != ASG_OK) return fail(dev_status, "plan_tune: a kernel reported a device-side timeout");
  if (best_kind) *best_kind = arg;
  if (best_ms) *best_ms = best;
  if (default_ms) *default_ms = at_def;
  return ASG_OK;
}

}  // namespace asg_tune

extern "C" {

const char* asg_version(void) { return "asgkron 0.1 (sm_103a)"; }

asg_status asg_last_error(char* buf, size_t len) {
  if (!buf || len == 0) return ASG_ERR_INVALID;
  snprintf(buf, len, "%s", asg::g_err);
  return ASG_OK;
}

asg_status asg_plan_create(const asg_plan_desc* desc, asg_plan** out) {
  if (!desc || !out) return fail(ASG_ERR_INVALID, "plan_create: NULL argument");
  return asg::create_plan(desc, 0, desc->num_elems, nullptr, out);
}

asg_status asg_plan_create_ex(const asg_plan_desc* desc, const asg_plan_ext* ext, asg_plan** out) {
  if (!desc || !out) return fail(ASG_ERR_INVALID, "plan_create_ex: NULL argument");
  if (!ext) return asg::create_plan(desc, 0, desc->num_elems, nullptr, out);
  return asg::create_plan(desc, ext->row_begin, ext->row_end, ext->op_blocks, out);
}

asg_status asg_plan_halo(const asg_plan* p, int* elems, long long capacity, long long* count) {
  if (!p || !count) return fail(ASG_ERR_INVALID, "plan_halo: NULL argument");
  const long long h = p->elem_global.empty() ? 0 : static_cast<long long>(p->N - p->N_out);
  *count = h;
  if (capacity == 0) return ASG_OK;
  if (!elems) return fail(ASG_ERR_INVALID, "plan_halo: NULL elems");
  if (capacity < h) return fail(ASG_ERR_CAPACITY, "plan_halo: capacity %lld < %lld halo elements", capacity, h);
  for (long long k = 0; k < h; ++k) elems[k] = p->elem_global[p->N_out + k] + p->index_base;
  return ASG_OK;
}

asg_status asg_plan_row_entries(const asg_plan* p, long long* counts) {
  if (!p || !counts) return fail(ASG_ERR_INVALID, "plan_row_entries: NULL argument");
  for (int i = 0; i < p->N_out; ++i) counts[i] = p->row_ptr[i + 1] - p->row_ptr[i];
  return ASG_OK;
}

asg_status asg_plan_update_elements(asg_plan* p, int num_elems, const int* idx1d, const long long* row_ptr,
                                    const int* cols) {
  return asg::update_elements(p, num_elems, idx1d, row_ptr, cols);
}

asg_status asg_plan_destroy(asg_plan* plan) {
  if (!plan) return ASG_OK;
  asg::free_device(plan);
  delete plan;
  return ASG_OK;
}

asg_status asg_plan_stats_get(const asg_plan* p, asg_plan_stats* s) {
  if (!p || !s) return fail(ASG_ERR_INVALID, "plan_stats_get: NULL argument");
  s->num_pairs = p->pairs;
  s->num_entries = static_cast<long long>(p->ent.size());
  s->dof = static_cast<long long>(p->N_out) * p->B;  // output DOF (a row slice: its rows)
  s->flops_reference = p->flops_dense;
  s->flops_executed = p->flops_exec;
  s->op_bytes_f64 = p->packed_elems * 8;
  s->kernel_kind = p->kernel_kind;
  int amax = 0;
  for (unsigned a : p->active) amax = std::max(amax, __builtin_popcount(a));
  s->active_modes_max = amax;
  return ASG_OK;
}

asg_status asg_plan_active(const asg_plan* p, unsigned* masks) {
  if (!p || !masks) return fail(ASG_ERR_INVALID, "plan_active: NULL argument");
  for (int t = 0; t < p->T; ++t) masks[t] = p->active[t];
  return ASG_OK;
}

asg_status asg_plan_update_ops(asg_plan* p, const double* const* ops, const int* op_ld) {
  if (!p || !ops || !op_ld) return fail(ASG_ERR_INVALID, "plan_update_ops: NULL argument");
  for (int tm = 0; tm < p->T * p->D; ++tm) {
    if (p->op_off[tm] < 0) continue;
    if (!ops[tm]) return fail(ASG_ERR_INVALID, "plan_update_ops: operator %d is NULL", tm);
    if (op_ld[tm] < p->op_nb[tm] * p->P) return fail(ASG_ERR_INVALID, "plan_update_ops: ld too small for operator %d", tm);
  }
  asg::pack_host(p, ops, op_ld);
  if (p->tr) {  // the transpose is rebuilt from the new values on its next use
    asg::free_plan(p->tr);
    p->tr = nullptr;
  }
  return asg::upload_ops(p);
}

asg_status asg_plan_set_kernel(asg_plan* p, int kind) {
  if (!p) return fail(ASG_ERR_INVALID, "plan_set_kernel: NULL plan");
  if (kind == asg::KK_CHAIN_WARP && p->B > 256) return fail(ASG_ERR_UNSUPPORTED, "warp chain kernel needs deg^d <= 256");
  if (kind == asg::KK_STREAM && p->ws_ctas <= 0)
    return fail(ASG_ERR_UNSUPPORTED, "streaming kernel needs deg 4, d 6 and one non-identity factor per term");
  if (kind == asg::KK_SINGLE_MODE || kind == asg::KK_SINGLE_TMA || kind == asg::KK_SINGLE_TMA3 ||
      kind == asg::KK_SINGLE_TMA_ROWS || kind == asg::KK_SINGLE_TMA_X2) {
    bool ok = kind != asg::KK_SINGLE_MODE ? (p->P == 4 && p->B == 4096)
                                         : ((p->P == 3 || p->P == 4) && p->B >= 32 * p->P * p->P);
    for (unsigned a : p->active) ok = ok && __builtin_popcount(a) == 1;
    if (!ok || p->ed.size() != p->ent.size())
      return fail(ASG_ERR_UNSUPPORTED, "single-mode kernels need one non-identity factor per term (deg 3/4)");
  }
  if (kind == asg::KK_SINGLE_SMALL) {
    bool ok = p->B <= 256 && p->ed.size() == p->ent.size();
    for (unsigned a : p->active) ok = ok && __builtin_popcount(a) == 1;
    if (!ok) return fail(ASG_ERR_UNSUPPORTED, "small single-mode kernel needs one applied factor per term, deg^d <= 256");
  }
  if (kind < 0 || kind > 8) return fail(ASG_ERR_INVALID, "unknown kernel kind %d", kind);
  p->kernel_kind = kind;
  p->tuned_kind[0] = p->tuned_kind[1] = -1;
  return ASG_OK;
}

asg_status asg_plan_tune(asg_plan* p, int precision, void* stream, int* best_kind, float* best_ms, float* default_ms) {
  if (!p) return fail(ASG_ERR_INVALID, "plan_tune: NULL plan");
  if (precision != 0 && precision != 1) return fail(ASG_ERR_INVALID, "plan_tune: precision=%d", precision);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  return precision ? asg_tune::tune_plan<float>(p, s, best_kind, best_ms, default_ms)
                   : asg_tune::tune_plan<double>(p, s, best_kind, best_ms, default_ms);
}

asg_status asg_plan_kernel_for(const asg_plan* p, int precision, int* kind) {
  if (!p || !kind || (precision != 0 && precision != 1)) return fail(ASG_ERR_INVALID, "plan_kernel_for: bad argument");
  *kind = precision ? asg::effective_kind<float>(p) : asg::effective_kind<double>(p);
  return ASG_OK;
}

asg_status asg_plan_device_status(asg_plan* p, int* status) {
  if (!p || !status) return fail(ASG_ERR_INVALID, "plan_device_status: NULL argument");
  int v = 0;
  ASG_CUDA(cudaMemcpy(&v, p->d_err, sizeof(int), cudaMemcpyDeviceToHost));
  *status = v;
  if (v != 0) {
    ASG_CUDA(cudaMemset(p->d_err, 0, sizeof(int)));
    return fail(v, "a kernel of this plan reported status %d (bounded wait gave up)", v);
  }
  return ASG_OK;
}

asg_status asg_grad_ops_f64(asg_plan* p, const double* f, const double* r, double* const* G, const int* ldg,
                            void* stream) {
  return asg::grad_ops<double>(p, f, r, G, ldg, stream);
}
asg_status asg_grad_ops_f32(asg_plan* p, const float* f, const float* r, float* const* G, const int* ldg,
                            void* stream) {
  return asg::grad_ops<float>(p, f, r, G, ldg, stream);
}

asg_status asg_apply_T_host_f64(asg_plan* p, const double* h_ybar, double* h_fbar) {
  if (!p) return fail(ASG_ERR_INVALID, "apply_T_host: NULL plan");
  ASG_NOT_SLICE(p, "apply_T_host");
  asg_status st = asg::build_transpose(p);
  return st ? st : asg::apply_host<double>(p->tr, h_ybar, h_fbar);
}

asg_status asg_grad_ops_host_f64(asg_plan* p, const double* h_f, const double* h_r, double* const* h_G,
                                 const int* ldg) {
  if (!p || !h_f || !h_r || !h_G || !ldg) return fail(ASG_ERR_INVALID, "grad_ops_host: NULL argument");
  ASG_NOT_SLICE(p, "grad_ops_host");
  const int TD = p->T * p->D;
  const size_t n = static_cast<size_t>(p->N) * p->B;
  const size_t vec = ((n * sizeof(double) + 255) / 256) * 256;
  // staging: f, r and every requested gradient matrix (ldg x n1d, column-major), 256-byte aligned
  std::vector<size_t> off(TD, 0);
  size_t bytes = 2 * vec;
  for (int tm = 0; tm < TD; ++tm) {
    if (!h_G[tm] || p->op_off[tm] < 0) continue;
    const int n1 = p->op_nb[tm] * p->P;
    if (ldg[tm] < n1) return fail(ASG_ERR_INVALID, "grad_ops_host: ldg[%d]=%d < %d", tm, ldg[tm], n1);
    off[tm] = bytes;
    bytes += ((static_cast<size_t>(ldg[tm]) * n1 * sizeof(double) + 255) / 256) * 256;
  }
  if (!p->stream) ASG_CUDA(cudaStreamCreateWithFlags(&p->stream, cudaStreamNonBlocking));
  char* buf = nullptr;
  ASG_CUDA(cudaMalloc(reinterpret_cast<void**>(&buf), bytes));
  double* df = reinterpret_cast<double*>(buf);
  double* dr = reinterpret_cast<double*>(buf + vec);
  std::vector<double*> dG(TD, nullptr);
  cudaError_t e = cudaMemcpyAsync(df, h_f, n * sizeof(double), cudaMemcpyHostToDevice, p->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(dr, h_r, n * sizeof(double), cudaMemcpyHostToDevice, p->stream);
  for (int tm = 0; tm < TD && e == cudaSuccess; ++tm) {
    if (!off[tm]) continue;
    dG[tm] = reinterpret_cast<double*>(buf + off[tm]);
    const size_t gb = static_cast<size_t>(ldg[tm]) * p->op_nb[tm] * p->P * sizeof(double);
    e = cudaMemcpyAsync(dG[tm], h_G[tm], gb, cudaMemcpyHostToDevice, p->stream);  // untouched entries kept
  }
  asg_status st = e == cudaSuccess ? ASG_OK : asg::cuda_fail(e, "grad_ops_host: copy in");
  if (!st) st = asg::grad_ops<double>(p, df, dr, dG.data(), ldg, p->stream);
  for (int tm = 0; tm < TD && !st; ++tm) {
    if (!dG[tm]) continue;
    const size_t gb = static_cast<size_t>(ldg[tm]) * p->op_nb[tm] * p->P * sizeof(double);
    e = cudaMemcpyAsync(h_G[tm], dG[tm], gb, cudaMemcpyDeviceToHost, p->stream);
    if (e != cudaSuccess) st = asg::cuda_fail(e, "grad_ops_host: copy out");
  }
  e = cudaStreamSynchronize(p->stream);
  if (!st && e != cudaSuccess) st = asg::cuda_fail(e, "grad_ops_host: synchronize");
  cudaFree(buf);
  return st;
}

asg_status asg_apply_T_f64(asg_plan* p, const double* ybar, double* fbar, void* stream) {
  if (!p) return fail(ASG_ERR_INVALID, "apply_T: NULL plan");
  ASG_NOT_SLICE(p, "apply_T");
  asg_status st = asg::build_transpose(p);
  return st ? st : asg::apply_dev<double>(p->tr, ybar, fbar, stream);
}
asg_status asg_apply_T_f32(asg_plan* p, const float* ybar, float* fbar, void* stream) {
  if (!p) return fail(ASG_ERR_INVALID, "apply_T: NULL plan");
  ASG_NOT_SLICE(p, "apply_T");
  asg_status st = asg::build_transpose(p);
  return st ? st : asg::apply_dev<float>(p->tr, ybar, fbar, stream);
}

asg_status asg_apply_f64(asg_plan* p, const double* f, double* y, void* stream) { return asg::apply_dev<double>(p, f, y, stream); }
asg_status asg_apply_f32(asg_plan* p, const float* f, float* y, void* stream) { return asg::apply_dev<float>(p, f, y, stream); }
asg_status asg_apply_residual_f64(asg_plan* p, const double* f, const double* ystar, double* r, void* stream) {
  return asg::apply_residual<double>(p, f, ystar, r, stream);
}
asg_status asg_apply_residual_f32(asg_plan* p, const float* f, const float* ystar, float* r, void* stream) {
  return asg::apply_residual<float>(p, f, ystar, r, stream);
}
asg_status asg_apply_host_f64(asg_plan* p, const double* f, double* y) { return asg::apply_host<double>(p, f, y); }
asg_status asg_apply_host_f32(asg_plan* p, const float* f, float* y) { return asg::apply_host<float>(p, f, y); }

}  // extern "C"
