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
__device__ __forceinline__ uint64_t splitmix64(uint64_t x) {
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}

// div_by_recip(a, s, RN(1/s)) against the correctly rounded a / s, s = RN(sqrt(n)) for n in
// [1, 100000] (the divisors of the recurrences), a with a random sign and mantissa and a
// binary exponent in [-1000, 1000], one in a thousand a zero.  Counts bitwise differences.
__global__ void __launch_bounds__(256) division_check_kernel(int64_t n, uint64_t seed,
                                                             unsigned long long* __restrict__ bad) {
  unsigned long long local = 0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const uint64_t x = splitmix64(seed + (uint64_t)i);
    const uint64_t z = splitmix64(x);
    const uint64_t ex = 23u + z % 2001u;
    double a = __longlong_as_double((long long)((x & 0x800FFFFFFFFFFFFFull) | (ex << 52)));
    if ((z >> 40) % 1000u == 0u) a = ((z >> 39) & 1u) ? -0.0 : 0.0;
    const int nn = 1 + (int)((z >> 12) % 100000u);
    const double b = sqrt((double)nn);
    const double y = __drcp_rn(b);
    if (__double_as_longlong(mm::div_by_recip(a, b, y)) != __double_as_longlong(__ddiv_rn(a, b))) ++local;
  }
  if (local) atomicAdd(bad, local);
}
}  // namespace

extern "C" {
// See include/mm_gb300.h.
MM_API int mm_probe_division(int64_t n, uint64_t seed, unsigned long long* bad, mm_stream_t stream) {
  if (!bad || n < 0) return MM_ERR_INVALID_ARG;
  if (n == 0) return MM_OK;
  division_check_kernel<<<1024, 256, 0, (cudaStream_t)stream>>>(n, seed, bad);
  mm::note_launches(1);
  return cudaGetLastError() == cudaSuccess ? MM_OK : MM_ERR_CUDA;
}

// Launch blocks x 256 threads, each doing 8 * iters DFMA; `out` holds blocks * 256 doubles.
// FLOPs of one launch: 2 * 8 * iters * blocks * 256.
MM_API int mm_probe_dfma(double* out, int blocks, int iters, mm_stream_t stream) {
  if (!out || blocks < 1 || iters < 1) return MM_ERR_INVALID_ARG;
  dfma_probe_kernel<<<blocks, 256, 0, (cudaStream_t)stream>>>(out, iters, 0.9999999, 1e-9);
  return cudaGetLastError() == cudaSuccess ? MM_OK : MM_ERR_CUDA;
}
}
