// The assembled operator as block-sparse rows: what apply_A.m builds with opts.build_A
// (apply_A.m:170-180 forms krond of the deg x deg factor blocks per pair and term and adds it
// at (I, J); apply_A.m:246-248 collects the sparse matrix).  Block (i, j) is the sum over the
// plan's terms of kron_k A_{t,k}[I_k(i), J_k(j)], identity factors as the exact identity and,
// under ASG_STRUCT_DETECT, products with a zero factor block left out -- the operator the
// kernels apply, as a matrix for direct solves and preconditioners.
#include <algorithm>
#include <vector>

#include "asg_internal.h"

namespace asg {
namespace {

struct BsrArgs {
  const double* ops;          // packed FP64 blocks (P x P row-major each)
  const long long* op_off;    // [T*D]
  const int* op_nb;           // [T*D]
  const int* idx1d;           // [N*D] 0-based
  const unsigned* active;     // [T]
  const int* blk_row;         // [nblocks] row element of each block
  const int* blk_col;         // [nblocks] column element
  const int* blk_tptr;        // [nblocks+1] its terms in blk_terms
  const int* blk_terms;
  double* out;                // [nblocks][B][B] row-major
  long long nblocks;
  int D, P, B;
};

// One CTA per block (grid-stride), a thread per output value (r, c): sum over the block's
// terms (in term order) of prod_k A_{t,k}[I_k(i) + r_k, J_k(j) + c_k], r_k and c_k the digits
// of r and c, dimension 1 slowest.
__global__ void k_assemble_bsr(BsrArgs a) {
  const int BB = a.B * a.B;
  for (long long q = blockIdx.x; q < a.nblocks; q += gridDim.x) {
    const int i = a.blk_row[q], j = a.blk_col[q];
    const int t0 = a.blk_tptr[q], t1 = a.blk_tptr[q + 1];
    for (int v = threadIdx.x; v < BB; v += blockDim.x) {
      const int r = v / a.B, c = v - r * a.B;
      double acc = 0.0;
      for (int tt = t0; tt < t1; ++tt) {
        const int t = a.blk_terms[tt];
        double prod = 1.0;
        int rr = r, cc = c, stride = a.B / a.P;
        for (int k = 0; k < a.D; ++k) {
          const int rk = rr / stride, ck = cc / stride;
          rr -= rk * stride;
          cc -= ck * stride;
          stride /= a.P;
          const int tm = t * a.D + k;
          if ((a.active[t] >> k) & 1u) {
            const long long blk = a.op_off[tm] +
                                  (static_cast<long long>(a.idx1d[i * a.D + k]) * a.op_nb[tm] + a.idx1d[j * a.D + k]) *
                                      a.P * a.P;
            prod *= a.ops[blk + rk * a.P + ck];
          } else if (rk != ck) {
            prod = 0.0;
          }
        }
        acc += prod;
      }
      a.out[q * BB + v] = acc;
    }
  }
}

}  // namespace
}  // namespace asg

using asg::fail;

extern "C" asg_status asg_assemble_bsr_f64(asg_plan* p, long long* row_ptr, int* cols, double* d_blocks,
                                           long long capacity, long long* num_blocks, void* stream) {
  if (!p || !num_blocks) return fail(ASG_ERR_INVALID, "assemble_bsr: NULL argument");
  ASG_NOT_SLICE(p, "assemble_bsr");
  if (p->B > 256) return fail(ASG_ERR_UNSUPPORTED, "assemble_bsr: deg^d = %d > 256 (blocks of %d values)", p->B, p->B * p->B);
  const int N = p->N, T = p->T;
  // unique columns per row (sorted) and each block's terms, from the work list
  std::vector<long long> rp(N + 1, 0);
  std::vector<int> bcol, brow, tptr(1, 0), terms;
  std::vector<std::vector<int>> per(0);
  for (int i = 0; i < N; ++i) {
    std::vector<std::pair<int, int>> ct;  // (column, term)
    for (long long q = p->row_ptr[i]; q < p->row_ptr[i + 1]; ++q) ct.push_back({p->ent[q] >> 4, p->ent[q] & 15});
    std::stable_sort(ct.begin(), ct.end());
    for (size_t k = 0; k < ct.size();) {
      size_t k2 = k;
      while (k2 < ct.size() && ct[k2].first == ct[k].first) terms.push_back(ct[k2++].second);
      brow.push_back(i);
      bcol.push_back(ct[k].first);
      tptr.push_back(static_cast<int>(terms.size()));
      k = k2;
    }
    rp[i + 1] = static_cast<long long>(bcol.size());
  }
  (void)T;
  const long long nb = static_cast<long long>(bcol.size());
  *num_blocks = nb;
  if (row_ptr) std::copy(rp.begin(), rp.end(), row_ptr);
  if (cols) std::copy(bcol.begin(), bcol.end(), cols);
  if (!d_blocks) return ASG_OK;  // structure query
  if (capacity < nb) return fail(ASG_ERR_CAPACITY, "assemble_bsr: %lld blocks, capacity %lld", nb, capacity);
  if (nb == 0) return ASG_OK;
  std::vector<int> ints;
  ints.insert(ints.end(), brow.begin(), brow.end());
  ints.insert(ints.end(), bcol.begin(), bcol.end());
  ints.insert(ints.end(), tptr.begin(), tptr.end());
  ints.insert(ints.end(), terms.begin(), terms.end());
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  int* d_ints = nullptr;
  ASG_CUDA(cudaMalloc(reinterpret_cast<void**>(&d_ints), ints.size() * sizeof(int)));
  cudaError_t e = cudaMemcpyAsync(d_ints, ints.data(), ints.size() * sizeof(int), cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) {
    asg::BsrArgs a{};
    a.ops = p->d_ops64;
    a.op_off = p->d_op_off;
    a.op_nb = p->d_op_nb;
    a.idx1d = p->d_idx1d;
    a.active = p->d_active;
    a.blk_row = d_ints;
    a.blk_col = d_ints + nb;
    a.blk_tptr = d_ints + 2 * nb;
    a.blk_terms = d_ints + 3 * nb + 1;
    a.out = d_blocks;
    a.nblocks = nb;
    a.D = p->D;
    a.P = p->P;
    a.B = p->B;
    const int grid = static_cast<int>(std::min<long long>(nb, 152LL * 8));
    asg::k_assemble_bsr<<<grid, 256, 0, s>>>(a);
    e = cudaGetLastError();
  }
  // the index tables are read by the kernel: free them once it is done
  cudaError_t e2 = cudaStreamSynchronize(s);
  cudaFree(d_ints);
  if (e != cudaSuccess) return asg::cuda_fail(e, "assemble_bsr");
  if (e2 != cudaSuccess) return asg::cuda_fail(e2, "assemble_bsr: synchronize");
  return ASG_OK;
}
