// Internal declarations shared by the asgkron translation units (not part of the C ABI).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <vector>

#include "asgkron.h"

namespace asg {

constexpr int kMaxDims = 6;    // kron_multd.m dispatches d<=6 to kronmult{d}; larger d is rejected
constexpr int kMaxTerms = 16;  // work entries pack the term id into 4 bits
constexpr int kMaxBlock = 4096;  // deg^d of one element block handled on chip

// Records a message for asg_last_error() and returns the status.
asg_status fail(asg_status st, const char* fmt, ...);
asg_status cuda_fail(cudaError_t e, const char* what);

#define ASG_CUDA(call)                                   \
  do {                                                   \
    cudaError_t _e = (call);                             \
    if (_e != cudaSuccess) return ::asg::cuda_fail(_e, #call); \
  } while (0)

// Precomputed work entry of the single-mode kernels: column element, the entry's
// non-identity dimension, and the element offset of its P x P operator block.
struct EntryDesc {
  int j;
  int m;
  long long aoff;
};

// One warp's share of a row in the fused GMRES cycle: entries [q0, q0 + len) of a row, summed
// into partial-sum slot `slot` (a row's slots are added in slot order).
struct FzItem {
  long long q0;
  int len;
  int slot;
};

// Arguments of the operator-application kernels.  One work entry is one
// (column element, term) product contributing to a row element; entries of a row are
// contiguous (CSR by row), packed as (col << 4) | term.
template <typename T>
struct ApplyArgs {
  const T* f;
  T* y;
  const T* ops;              // block-major packed 1-D operators
  const long long* op_off;   // [T*D] element offset of packed operator (t,d); -1 when not packed
  const int* op_nb;          // [T*D] 1-D blocks per side of packed operator (t,d)
  const int* idx1d;          // [N*D] 0-based 1-D index of each element per dimension
  const long long* row_ptr;  // [N+1]
  const int* ent;            // packed entries
  const unsigned* active;    // [T] bit m set <=> operator (t,m) is applied (else identity)
  int N, D, B, nterms;
  int stride[kMaxDims];      // deg^(D-1-m): element-block stride of dimension m
  const EntryDesc* ed;       // [entries] single-mode descriptors (NULL for chain plans)
  const float* ops_pair;     // FP32 blocks in paired-FMA order (32 values per block), single-mode plans
  const float* ops_cols;     // FP32 blocks column by column (A0b,A1b,A2b,A3b), 16 values, deg-4 single-mode plans
  const int* row_order;      // [N] launch order of rows (longest work first) or NULL
  int* err;                  // device status word (ASG_ERR_TIMEOUT after a bounded wait gave up)
  const int* cta_ptr;        // [nctas+1] persistent single-mode kernel: rows of CTA c are
  const int* cta_rows;       //   cta_rows[cta_ptr[c] .. cta_ptr[c+1]) (static LPT assignment)
  int nctas;
  const T* ysub;             // NULL, or a vector laid out like y: the kernels store A f - ysub
};

template <typename T>
cudaError_t launch_apply(const ApplyArgs<T>& a, int P, int kernel_kind, cudaStream_t s);

// Gradient with respect to the 1-D operators: one CTA per target block (t, k, alpha, beta)
// sums its contributing work entries (i, j, t, k) in a fixed order.
struct GradContrib {
  int i, j, t, k;
};
struct GradTarget {
  int tm;     // t*D + k
  int alpha;  // block row (1-D index of the row element in dimension k)
  int beta;   // block column
};
// Work item of the chunked gradient kernel (terms with one applied factor, deg 4): up to 8
// contributors [c0, c1) of target tgt, the items of one target being [first, first+count).
struct GradItem {
  int tgt, c0, c1, first, count;
};
template <typename T>
struct GradArgs {
  const T* f;                   // forward input
  const T* r;                   // cotangent (d L / d y)
  const T* ops;                 // packed blocks (same layout as the apply)
  const long long* op_off;
  const int* op_nb;
  const int* idx1d;
  const unsigned* active;
  const long long* tgt_ptr;     // [ntgt+1] contributors of each target
  const GradContrib* contrib;
  const GradTarget* tgt;
  T* const* G;                  // [T*D] dense column-major outputs (device), NULL = skip
  const int* ldg;               // [T*D]
  int ntgt, D, B;
  int stride[kMaxDims];
  const GradItem* items;        // chunked kernel: [nitems] (NULL: one CTA per target)
  int nitems;
  T* partial;                   // [nitems][P*P] item sums
  int* counter;                 // [ntgt] items finished (last arriver sums and resets to 0)
};
template <typename T>
cudaError_t launch_grad(const GradArgs<T>& a, int P, cudaStream_t s);

enum KernelKind { KK_CHAIN_WARP = 0, KK_CHAIN_CTA = 1, KK_SINGLE_MODE = 2, KK_SINGLE_TMA = 3, KK_SINGLE_TMA3 = 4,
                  KK_SINGLE_TMA_ROWS = 5, KK_SINGLE_SMALL = 6, KK_STREAM = 7, KK_SINGLE_TMA_X2 = 8 };

// Streaming FP32 apply (deg 4, 4,096-value blocks, one applied factor per term): every CTA
// walks its own work stream.  An entry is {column element j, row element, operator block
// index, flags | applied dimension (bits 0-3)}.
enum StreamFlags : int {
  SF_SELF = 1 << 4,  // j is the row element: read the row's resident block
  SF_ROW0 = 1 << 5,  // first entry of a row (its resident block is copied with this entry)
  SF_ROW1 = 1 << 6,  // last entry of a row (y block written after it)
  SF_GRP0 = 1 << 7,  // first entry of a group (entries of one applied dimension)
  SF_GRP1 = 1 << 8,  // last entry of a group
  SF_ZERO = 1 << 9   // a row without entries: its y block is written as zeros, nothing staged
};
struct StreamArgs {
  const float* f;
  float* y;
  const float* ops_cols;  // FP32 blocks stored column by column (A0b,A1b,A2b,A3b), 16 values per block
  const int4* ws;         // [nctas][ws_stride]: header {entry count}, then the entries; padded
  int ws_stride;          // int4 per CTA: 1 + entries rounded up to 32
  int nctas;
  int* err;
  const float* ysub;      // NULL, or a vector laid out like y: the kernel stores A f - ysub
};
// Dynamic shared memory and resident CTAs per SM of the streaming kernel (0 on error).
size_t stream_smem();
int stream_occupancy();
cudaError_t launch_stream(const StreamArgs& a, cudaStream_t s);

// Apply arguments (f and y unset) of a plan that runs the small-block single-mode kernel, for
// kernels that call its row routine themselves (the fused GMRES cycle); false for other plans.
template <typename T>
bool small_plan_args(const asg_plan* p, ApplyArgs<T>* out);

// Resident CTAs per SM of the persistent single-mode kernel for element size es (4 or 8);
// sets the kernel's dynamic shared-memory limit first.  0 on error.
int single_tma_rows_occupancy(int es);

}  // namespace asg

// The plan object behind the opaque C handle.
struct asg_plan {
  int D = 0, P = 0, T = 0, N = 0, B = 0;
  // Output rows: elements [0, N_out) are the rows the kernels write (y holds N_out blocks);
  // elements [N_out, N) are input-only (a row slice's halo, asg_plan_create_rows).  N_out == N
  // for a plan over the whole table.
  int N_out = 0;
  std::vector<int> elem_global;      // row-slice plans: the table id (0-based) of each element
  int index_base = 0;                // base of the caller's index arrays (0 or 1)
  int structure = 0;
  double drop_tol = 0.0;
  int kernel_kind = 0;
  int tuned_kind[2] = {-1, -1};      // asg_plan_tune's choice per precision (0 FP64, 1 FP32), -1: none
  // host-side metadata
  std::vector<int> idx1d;            // N*D, 0-based
  std::vector<int> op_nb;            // T*D
  std::vector<unsigned> active;      // T
  std::vector<long long> op_off;     // T*D
  std::vector<long long> row_ptr;    // N+1
  std::vector<int> ent;              // entries
  std::vector<long long> tr_row_ptr; // transposed work list (by column) for the adjoint
  std::vector<int> tr_ent;           // packed (row << 4) | term
  long long packed_elems = 0;
  long long pairs = 0;
  double flops_dense = 0, flops_exec = 0;
  // device-side copies
  int* d_idx1d = nullptr;
  int* d_op_nb = nullptr;
  unsigned* d_active = nullptr;
  long long* d_op_off = nullptr;
  long long* d_row_ptr = nullptr;
  int* d_ent = nullptr;
  long long* d_tr_row_ptr = nullptr;
  int* d_tr_ent = nullptr;
  std::vector<double> h64;           // packed FP64 blocks (host copy: transposes and gradients)
  bool all_pairs = true;             // listed pairs: all, or the CSR below (0-based)
  std::vector<long long> pr_ptr;
  std::vector<int> pr_col;
  std::vector<std::vector<uint8_t>> zero_blk;  // per (t,d): block (a,b) is zero (DETECT mode)
  asg_plan* tr = nullptr;            // transposed plan (A^T), built on first use
  // gradient targets (built on first use)
  std::vector<long long> g_ptr;
  std::vector<asg::GradContrib> g_contrib;
  std::vector<asg::GradTarget> g_tgt;
  long long* d_g_ptr = nullptr;
  asg::GradContrib* d_g_contrib = nullptr;
  asg::GradTarget* d_g_tgt = nullptr;
  int* d_ldg = nullptr;
  void** d_gptrs = nullptr;
  std::vector<asg::GradItem> g_items;  // chunked gradient (single-factor terms, deg 4)
  asg::GradItem* d_g_items = nullptr;
  void* d_g_partial = nullptr;         // nitems * 16 doubles
  int* d_g_counter = nullptr;
  std::vector<asg::EntryDesc> ed;   // single-mode descriptors (empty unless every term has one factor)
  asg::EntryDesc* d_ed = nullptr;
  std::vector<int> row_order;
  int* d_row_order = nullptr;
  // persistent single-mode kernel: per precision (0 FP64, 1 FP32) the rows of each CTA
  std::vector<int> cta_ptr[2], cta_rows[2];
  int* d_cta_ptr[2] = {nullptr, nullptr};
  int* d_cta_rows[2] = {nullptr, nullptr};
  float* d_ops_pair = nullptr;
  float* d_ops_cols = nullptr;       // FP32 blocks column by column (deg 4 single-mode plans)
  // streaming FP32 kernel: one padded work stream per CTA (4 ints per entry, header first)
  std::vector<int> ws;
  int ws_stride = 0, ws_ctas = 0;
  int* d_ws = nullptr;
  // fused backward-Euler solve (small-block plans, built on first use), per basis precision
  // (0 FP64, 1 FP32): contiguous row ranges per CTA and chunks of their rows' entries per warp
  int fz_G[2] = {0, 0}, fz_max_rows[2] = {0, 0}, fz_max_slots[2] = {0, 0};
  int* d_fz_int[2] = {nullptr, nullptr};  // blk_row[G+1], blk_slot[G+1], row_slot[N+1], warp_item[G*W+1]
  asg::FzItem* d_fz_items[2] = {nullptr, nullptr};
  int* d_err = nullptr;
  unsigned* d_bar = nullptr;  // grid barrier words of the fused RK3 step (zeroed per launch)
  double* d_ops64 = nullptr;
  float* d_ops32 = nullptr;
  // host-pointer apply path (staging owned by the plan)
  void* d_io = nullptr;
  size_t d_io_bytes = 0;
  cudaStream_t stream = nullptr;
  // host-pointer apply in element chunks (one-CTA-per-row kernels; built on first use, per
  // schedule s = 2 * g + k, k = 0 FP64, 1 FP32): f arrives in kHostChunks pieces of an element
  // order -- g = 0: the table reversed (coarsest elements first), one copy per chunk; g = 1
  // (page-locked f): the columns of the longest rows first, gathered by a kernel from the
  // mapped buffer, order d_hc_order[s]. Chunk c is positions [hc_estart[s][c],
  // hc_estart[s][c+1]) of the order, and its rows -- those whose blocks have all arrived with
  // it -- are hc_rows[s][hc_start[s][c] .. hc_start[s][c+1]), longest first
  static constexpr int kHostChunks = 5;
  std::vector<int> hc_estart[4], hc_start[4];
  int* d_hc_rows[4] = {};
  int* d_hc_order[4] = {};
  cudaStream_t cstream[kHostChunks] = {};  // one compute stream per chunk
  cudaEvent_t ev_in[kHostChunks] = {};
  cudaEvent_t ev_done[kHostChunks] = {};
  // the chunked host apply as one CUDA graph, replayed while the caller repeats its page-locked
  // f and y buffers (captured at the second call with the same buffers, kernel and precision)
  cudaGraphExec_t hg_exec = nullptr;
  const void* hg_f = nullptr;
  const void* hg_y = nullptr;
  const void* hg_kf = nullptr;       // the device aliases of f and y the graph was made with
  const void* hg_ky = nullptr;
  int hg_kind = -1, hg_es = 0, hg_repeat = 0;
};

// A row-slice plan (asg_plan_create_ex with a narrower row range): forward apply only.
inline bool asg_is_slice(const asg_plan* p) { return p && p->N_out != p->N; }
#define ASG_NOT_SLICE(p, what)                                                                   \
  do {                                                                                           \
    if (asg_is_slice(p)) return ::asg::fail(ASG_ERR_UNSUPPORTED, "%s: not for a row-slice plan", what); \
  } while (0)
