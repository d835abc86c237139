// FP64 pipe probe: the denominator of the recurrence's FP64 roofline.
//
// The Hermite recurrence and its VJP are complex128 multiply-add chains, so
// their ceiling on this GPU is the FP64 FMA rate, which no vendor number in the
// repository states.  This kernel measures it: every thread runs 8 independent
// DFMA chains (enough to cover the pipe latency), one CTA set per SM.
#include <cstdint>

#include "common.cuh"

namespace {
__global__ void __launch_bounds__(256) dfma_probe_kernel(double* __restrict__ out, int iters, double a, double b) {
  double x[8];
#pragma unroll
  for (int j = 0; j < 8; ++j) x[j] = 1e-3 * (threadIdx.x + j);
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int j = 0; j < 8; ++j) x[j] = fma(x[j], a, b);
  }
  double s = 0.0;
#pragma unroll
  for (int j = 0; j < 8; ++j) s += x[j];
  out[(int64_t)blockIdx.x * blockDim.x + threadIdx.x] = s;
}
}  // namespace

extern "C" {
// Launch blocks x 256 threads, each doing 8 * iters DFMA; `out` holds blocks * 256 doubles.
// FLOPs of one launch: 2 * 8 * iters * blocks * 256.
MM_API int mm_probe_dfma(double* out, int blocks, int iters, mm_stream_t stream) {
  if (!out || blocks < 1 || iters < 1) return MM_ERR_INVALID_ARG;
  dfma_probe_kernel<<<blocks, 256, 0, (cudaStream_t)stream>>>(out, iters, 0.9999999, 1e-9);
  return cudaGetLastError() == cudaSuccess ? MM_OK : MM_ERR_CUDA;
}
}
