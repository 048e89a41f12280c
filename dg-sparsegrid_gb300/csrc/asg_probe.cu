// Measurement kernels for the roofline the apply is judged against (no reference
// counterpart): the rate at which one GB300 streams a plan's own gather pattern from L2 into
// shared memory with the bulk copies the apply kernels use, and the FP32 paired-FMA and FP64
// FMA issue rates.  They compute nothing the library returns; the caller times them.
#include "asg_internal.h"
#include "asg_pipe.cuh"

namespace asg {
namespace {

// One CTA per row (launch order as the apply), one elected thread streaming the row's column
// blocks (B values each) through S shared-memory stages, waiting on its own copies: the apply's
// gather with no arithmetic.  Waits bounded; a checksum of one value per block is written so
// the copies are used.
template <int S>
__global__ void __launch_bounds__(32) k_gather_stream(const float* f, const long long* row_ptr, const int* ent,
                                                       const int* row_order, int B, float* out, int* err) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  float* st = reinterpret_cast<float*>(smem_raw);
  uint64_t* full = reinterpret_cast<uint64_t*>(st + static_cast<size_t>(S) * B);
  const int row = row_order ? row_order[blockIdx.x] : blockIdx.x;
  const long long q0 = row_ptr[row];
  const int n = static_cast<int>(row_ptr[row + 1] - q0);
  if (threadIdx.x != 0) return;
  for (int k = 0; k < S; ++k) mbar_init(&full[k], 1);
  mbar_fence_init();
  float acc = 0.f;
  int issued = 0;
  bool ok = true;
  const uint32_t bytes = static_cast<uint32_t>(B) * sizeof(float);
  for (int k = 0; k < n && ok; ++k) {
    const int s = k % S;
    if (k >= S) {
      ok = mbar_wait_bounded(&full[s], static_cast<uint32_t>(((k / S) - 1) & 1));
      if (ok) acc += st[static_cast<size_t>(s) * B];
    }
    if (!ok) break;
    const int j = ent[q0 + k] >> 4;
    mbar_expect_tx(&full[s], bytes);
    bulk_g2s(st + static_cast<size_t>(s) * B, f + static_cast<size_t>(j) * B, bytes, &full[s]);
    issued = k + 1;
  }
  for (int k = max(0, issued - S); k < issued; ++k) {
    if (mbar_wait_bounded(&full[k % S], static_cast<uint32_t>((k / S) & 1)))
      acc += st[static_cast<size_t>(k % S) * B];
    else
      ok = false;
  }
  if (!ok) atomicExch(err, static_cast<int>(ASG_ERR_TIMEOUT));
  out[row] = acc;
}

// Independent FMA chains per thread (8 accumulators), `iters` rounds: FP32 paired FMA or FP64 FMA.
__global__ void k_fma_f32x2(int iters, float seed, float* out) {
  float2 a[8];
  const float2 m = make_float2(0.999f, 0.998f), c = make_float2(seed, seed * 0.5f);
#pragma unroll
  for (int k = 0; k < 8; ++k) a[k] = make_float2(seed + k, seed - k);
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int k = 0; k < 8; ++k) a[k] = ffma2(a[k], m, c);
  }
  float s = 0.f;
#pragma unroll
  for (int k = 0; k < 8; ++k) s += a[k].x + a[k].y;
  if (s == 1234.5f) out[0] = s;
}
__global__ void k_fma_f64(int iters, double seed, double* out) {
  double a[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) a[k] = seed + k;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int k = 0; k < 8; ++k) a[k] = fma(a[k], 0.999, seed);
  }
  double s = 0.0;
#pragma unroll
  for (int k = 0; k < 8; ++k) s += a[k];
  if (s == 1234.5) out[0] = s;
}

}  // namespace
}  // namespace asg

using asg::fail;

extern "C" {

asg_status asg_probe_gather_f32(asg_plan* p, const float* d_f, float* d_out, int stages, void* stream) {
  if (!p || !d_f || !d_out) return fail(ASG_ERR_INVALID, "probe_gather: NULL argument");
  ASG_NOT_SLICE(p, "probe_gather");
  if (reinterpret_cast<uintptr_t>(d_f) & 15) return fail(ASG_ERR_INVALID, "probe_gather: f must be 16-byte aligned");
  if ((p->B * sizeof(float)) % 16 != 0) return fail(ASG_ERR_UNSUPPORTED, "probe_gather: block of %d floats", p->B);
  if (stages != 2 && stages != 4 && stages != 8) return fail(ASG_ERR_INVALID, "probe_gather: stages=%d", stages);
  if (p->N == 0) return ASG_OK;
  const size_t smem = static_cast<size_t>(stages) * p->B * sizeof(float) + stages * sizeof(uint64_t);
  if (smem > 200 * 1024) return fail(ASG_ERR_UNSUPPORTED, "probe_gather: %zu bytes of stages", smem);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  auto run = [&](auto kern) -> cudaError_t {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
    if (e != cudaSuccess) return e;
    kern<<<p->N, 32, smem, s>>>(d_f, p->d_row_ptr, p->d_ent, p->d_row_order, p->B, d_out, p->d_err);
    return cudaGetLastError();
  };
  cudaError_t e = stages == 2 ? run(asg::k_gather_stream<2>) : stages == 4 ? run(asg::k_gather_stream<4>)
                                                                             : run(asg::k_gather_stream<8>);
  if (e != cudaSuccess) return asg::cuda_fail(e, "probe_gather launch");
  return ASG_OK;
}

asg_status asg_probe_fma(int precision, int blocks, int iters, void* d_out, double* flops, void* stream) {
  if (precision != 0 && precision != 1) return fail(ASG_ERR_INVALID, "probe_fma: precision=%d", precision);
  if (blocks < 1 || iters < 1 || !d_out) return fail(ASG_ERR_INVALID, "probe_fma: bad argument");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const double threads = static_cast<double>(blocks) * 256;
  if (precision == 1) {
    asg::k_fma_f32x2<<<blocks, 256, 0, s>>>(iters, 1.0f, static_cast<float*>(d_out));
    if (flops) *flops = threads * iters * 8 * 4.0;  // 8 chains x 2 lanes x (multiply + add)
  } else {
    asg::k_fma_f64<<<blocks, 256, 0, s>>>(iters, 1.0, static_cast<double*>(d_out));
    if (flops) *flops = threads * iters * 8 * 2.0;
  }
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? ASG_OK : asg::cuda_fail(e, "probe_fma launch");
}

}  // extern "C"
