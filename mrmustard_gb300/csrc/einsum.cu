// Building blocks of the general Fock-space einsum: strided permutation, inner-axis sums
// and batched complex128 GEMM / GEMV.
//
// Reference: ArrayAnsatz.contract (mrmustard/physics/ansatz/array_ansatz.py:159-226) slices
// every contracted label to the smaller of its two dimensions and calls
// math.einsum(string, a, b) (mrmustard/math/backend_manager.py:526-548), which opt_einsum
// evaluates as permutations plus a BLAS matrix product (tensordot); mm_einsum
// (mrmustard/physics/mm_einsum.py:51-170) chains such pairwise contractions.  The host layer
// (mrmustard_gb300/einsum.py) plans every pairwise contraction as
//   A -> [batch, free_a, contracted] (one permutation of a strided view, which also takes the
//        reference's slices and the diagonals of repeated labels),
//   B -> [batch, contracted, free_b],
//   C[batch] = A[batch] @ B[batch]     (batched FP64 complex GEMM; GEMV when N or M is 1),
//   C -> output order                  (one permutation),
// with labels summed inside one operand reduced by mm_tensor_sum_inner first.
//
// Kernels:
//   permute_rows_kernel   gather with one warp per output row (all axes but the last) when
//                         no tile applies; permute_elems_kernel one thread per element when the
//                         output's innermost axis is short;
//   permute_tile_kernel   32 x 32 shared-memory tiles between the input's contiguous axis and
//                         the output's innermost axis (both accesses coalesced);
//   sum_inner_kernel      one warp per row, fixed-order shuffle reduction;
//   zgemm_batched_kernel  32 x 32 (2 x 2 outputs per thread) or 16 x 16 (1 x 1) tiles over 16-deep
//                         K slabs, batch in grid.z;
//   zgemv_rows_kernel     y = A x (N = 1): one warp per row of A;
//   zgemv_cols_kernel     y = x B (M = 1): one thread per column of B.
#include <algorithm>
#include <cstdint>
#include <cstring>

#include "common.cuh"

using mm::cfma;
using mm::cmk;

namespace {

constexpr int kMaxRank = 16;

struct PermArgs {
  int rank;
  int64_t shape[kMaxRank];    // output shape (C order)
  int64_t istride[kMaxRank];  // input element stride of each output axis
  int64_t ostride[kMaxRank];  // output C-order strides
  int64_t ioff;               // input element offset
  int64_t n;                  // elements
};

// One warp per output row (all axes but the last): lanes stride the innermost output axis.
__global__ void __launch_bounds__(256) permute_rows_kernel(PermArgs a, const double2* __restrict__ in,
                                                           double2* __restrict__ out) {
  const int r = a.rank;
  const int64_t inner = a.shape[r - 1];
  const int64_t rows = a.n / inner;
  const int lane = threadIdx.x & 31;
  const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  const int64_t s_in = a.istride[r - 1];
  for (int64_t row = warp; row < rows; row += nwarps) {
    int64_t rem = row, off = a.ioff;
    for (int k = r - 2; k >= 0; --k) {
      const int64_t i = rem % a.shape[k];
      rem /= a.shape[k];
      off += i * a.istride[k];
    }
    double2* o = out + row * inner;
    for (int64_t j = lane; j < inner; j += 32) o[j] = __ldg(in + off + j * s_in);
  }
}

// One thread per output element (short innermost output axes).
__global__ void __launch_bounds__(256) permute_elems_kernel(PermArgs a, const double2* __restrict__ in,
                                                            double2* __restrict__ out) {
  for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < a.n; idx += (int64_t)gridDim.x * blockDim.x) {
    int64_t rem = idx, off = a.ioff;
    for (int k = a.rank - 1; k >= 0; --k) {
      const int64_t i = rem % a.shape[k];
      rem /= a.shape[k];
      off += i * a.istride[k];
    }
    out[idx] = __ldg(in + off);
  }
}

// 32 x 32 tiles between output axis t (contiguous in the input) and the output's last axis.
__global__ void __launch_bounds__(256) permute_tile_kernel(PermArgs a, int t, const double2* __restrict__ in,
                                                           double2* __restrict__ out) {
  __shared__ double2 tile[32][33];
  const int r = a.rank;
  const int64_t ext_t = a.shape[t], ext_l = a.shape[r - 1];
  const int64_t tiles_t = (ext_t + 31) / 32, tiles_l = (ext_l + 31) / 32;
  const int64_t outer = a.n / (ext_t * ext_l);
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;  // 32 x 8
  for (int64_t job = blockIdx.x; job < outer * tiles_t * tiles_l; job += gridDim.x) {
    const int64_t tl = job % tiles_l, tt = (job / tiles_l) % tiles_t, o = job / (tiles_l * tiles_t);
    int64_t rem = o, ioff = a.ioff, ooff = 0;
    for (int k = r - 2; k >= 0; --k) {
      if (k == t) continue;
      const int64_t i = rem % a.shape[k];
      rem /= a.shape[k];
      ioff += i * a.istride[k];
      ooff += i * a.ostride[k];
    }
    const int64_t t0 = tt * 32, l0 = tl * 32;
    // read: lanes along t (stride 1 in the input)
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const int64_t it = t0 + tx, il = l0 + ty + 8 * k;
      if (it < ext_t && il < ext_l) tile[ty + 8 * k][tx] = __ldg(in + ioff + it * a.istride[t] + il * a.istride[r - 1]);
    }
    __syncthreads();
    // write: lanes along the output's last axis
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const int64_t it = t0 + ty + 8 * k, il = l0 + tx;
      if (it < ext_t && il < ext_l) out[ooff + it * a.ostride[t] + il] = tile[tx][ty + 8 * k];
    }
    __syncthreads();
  }
}

// out[row] = sum_j in[row * inner + j], one warp per row, fixed-order reduction.
__global__ void __launch_bounds__(256) sum_inner_kernel(int64_t rows, int64_t inner, const double2* __restrict__ in,
                                                        double2* __restrict__ out) {
  const int lane = threadIdx.x & 31;
  const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t row = warp; row < rows; row += nwarps) {
    double2 acc = cmk(0.0, 0.0);
    const double2* p = in + row * inner;
    for (int64_t j = lane; j < inner; j += 32) {
      const double2 v = __ldg(p + j);
      acc.x += v.x;
      acc.y += v.y;
    }
#pragma unroll
    for (int s = 16; s > 0; s >>= 1) {
      acc.x += __shfl_xor_sync(0xffffffffu, acc.x, s);
      acc.y += __shfl_xor_sync(0xffffffffu, acc.y, s);
    }
    if (lane == 0) out[row] = acc;
  }
}

// ---------------------------------------------------------------- batched GEMM
// BM x BN tiles over 16-deep K slabs, 256 threads, each TM x TN outputs (32 x 32 with 2 x 2,
// or 16 x 16 with 1 x 1 when the 32 x 32 grid would leave SMs idle: FP64 throughput per SM
// is the bound, so the number of CTAs in flight is what matters).
constexpr int BG_BK = 16;

template <int BM, int BN>
__global__ void __launch_bounds__(256) zgemm_batched_kernel(const double2* __restrict__ A, int64_t sA,
                                                            const double2* __restrict__ B, int64_t sB,
                                                            double2* __restrict__ C, int64_t sC, int64_t batch,
                                                            int M, int N, int K) {
  constexpr int TM = BM / 16, TN = BN / 16;
  __shared__ double2 As[BG_BK][BM];
  __shared__ double2 Bs[BG_BK][BN];
  const int tid = threadIdx.x;
  const int tx = tid & 15, ty = tid >> 4;
  const int m0 = blockIdx.y * BM, n0 = blockIdx.x * BN;
  for (int64_t z = blockIdx.z; z < batch; z += gridDim.z) {
    const double2* Az = A + z * sA;
    const double2* Bz = B + z * sB;
    double2 acc[TM][TN];
#pragma unroll
    for (int i = 0; i < TM; ++i)
#pragma unroll
      for (int j = 0; j < TN; ++j) acc[i][j] = cmk(0.0, 0.0);
    for (int k0 = 0; k0 < K; k0 += BG_BK) {
      for (int idx = tid; idx < BG_BK * BM; idx += 256) {
        const int row = idx / BG_BK, kk = idx % BG_BK;
        const int gm = m0 + row, gk = k0 + kk;
        As[kk][row] = (gm < M && gk < K) ? __ldg(Az + (int64_t)gm * K + gk) : cmk(0.0, 0.0);
      }
      for (int idx = tid; idx < BG_BK * BN; idx += 256) {
        const int kx = idx / BN, col = idx % BN;
        const int gk2 = k0 + kx, gn = n0 + col;
        Bs[kx][col] = (gk2 < K && gn < N) ? __ldg(Bz + (int64_t)gk2 * N + gn) : cmk(0.0, 0.0);
      }
      __syncthreads();
#pragma unroll
      for (int kk = 0; kk < BG_BK; ++kk) {
        double2 a[TM], b[TN];
#pragma unroll
        for (int i = 0; i < TM; ++i) a[i] = As[kk][ty * TM + i];
#pragma unroll
        for (int j = 0; j < TN; ++j) b[j] = Bs[kk][tx * TN + j];
#pragma unroll
        for (int i = 0; i < TM; ++i)
#pragma unroll
          for (int j = 0; j < TN; ++j) acc[i][j] = cfma(a[i], b[j], acc[i][j]);
      }
      __syncthreads();
    }
    double2* Cz = C + z * sC;
#pragma unroll
    for (int i = 0; i < TM; ++i)
#pragma unroll
      for (int j = 0; j < TN; ++j) {
        const int gm = m0 + ty * TM + i, gn = n0 + tx * TN + j;
        if (gm < M && gn < N) Cz[(int64_t)gm * N + gn] = acc[i][j];
      }
  }
}

// y[z][m] = sum_k A[z][m][k] x[z][k]: one warp per (z, m), lanes stride k.
__global__ void __launch_bounds__(256) zgemv_rows_kernel(const double2* __restrict__ A, int64_t sA,
                                                         const double2* __restrict__ x, int64_t sx,
                                                         double2* __restrict__ y, int64_t sy, int64_t batch, int64_t M,
                                                         int64_t K) {
  const int lane = threadIdx.x & 31;
  const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t w = warp; w < batch * M; w += nwarps) {
    const int64_t z = w / M, m = w - z * M;
    const double2* a = A + z * sA + m * K;
    const double2* xv = x + z * sx;
    double2 acc = cmk(0.0, 0.0);
    for (int64_t k = lane; k < K; k += 32) acc = cfma(__ldg(a + k), __ldg(xv + k), acc);
#pragma unroll
    for (int s = 16; s > 0; s >>= 1) {
      acc.x += __shfl_xor_sync(0xffffffffu, acc.x, s);
      acc.y += __shfl_xor_sync(0xffffffffu, acc.y, s);
    }
    if (lane == 0) y[z * sy + m] = acc;
  }
}

// y[z][n] = sum_k x[z][k] B[z][k][n]: one thread per (z, n), coalesced along n.
__global__ void __launch_bounds__(256) zgemv_cols_kernel(const double2* __restrict__ x, int64_t sx,
                                                         const double2* __restrict__ B, int64_t sB,
                                                         double2* __restrict__ y, int64_t sy, int64_t batch, int64_t N,
                                                         int64_t K) {
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < batch * N; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t z = t / N, nn = t - z * N;
    const double2* b = B + z * sB + nn;
    const double2* xv = x + z * sx;
    double2 acc = cmk(0.0, 0.0);
    for (int64_t k = 0; k < K; ++k) acc = cfma(__ldg(xv + k), __ldg(b + k * N), acc);
    y[z * sy + nn] = acc;
  }
}

int status() { return cudaGetLastError() == cudaSuccess ? MM_OK : MM_ERR_CUDA; }

int sms_of_device() {
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 0;
  return sms;
}

unsigned blocks_for(int64_t work, int per_block, int sms) {
  return (unsigned)std::max<int64_t>(1, std::min<int64_t>((work + per_block - 1) / per_block, (int64_t)sms * 32));
}

}  // namespace

MM_API int mm_tensor_permute(int rank, const int64_t* out_shape, const int64_t* in_strides, int64_t in_offset,
                             const mm_c128* in, mm_c128* out, mm_stream_t stream) {
  if (rank < 0 || (rank > 0 && (!out_shape || !in_strides))) return MM_ERR_INVALID_ARG;
  if (rank > kMaxRank) return MM_ERR_UNSUPPORTED;
  const int sms = sms_of_device();
  if (sms == 0) return MM_ERR_NO_DEVICE;
  cudaStream_t st = (cudaStream_t)stream;
  PermArgs a;
  memset(&a, 0, sizeof(a));
  a.ioff = in_offset;
  a.n = 1;
  // a rank-0 view is one element
  a.rank = rank > 0 ? rank : 1;
  if (rank == 0) {
    a.shape[0] = 1;
    a.istride[0] = 0;
  }
  for (int k = 0; k < rank; ++k) {
    if (out_shape[k] < 0) return MM_ERR_INVALID_ARG;
    a.shape[k] = out_shape[k];
    a.istride[k] = in_strides[k];
  }
  for (int k = a.rank - 1; k >= 0; --k) {
    a.ostride[k] = a.n;
    a.n *= a.shape[k];
  }
  if (a.n == 0) return MM_OK;
  if (!in || !out) return MM_ERR_INVALID_ARG;
  const int r = a.rank;
  // tile when the output's last axis is strided in the input and another axis is contiguous there
  int t = -1;
  if (a.istride[r - 1] != 1 && a.shape[r - 1] >= 8)
    for (int k = 0; k < r - 1; ++k)
      if (a.istride[k] == 1 && a.shape[k] >= 8) t = k;
  if (t >= 0) {
    const int64_t jobs = a.n / (a.shape[t] * a.shape[r - 1]) * ((a.shape[t] + 31) / 32) * ((a.shape[r - 1] + 31) / 32);
    permute_tile_kernel<<<blocks_for(jobs, 1, sms), 256, 0, st>>>(a, t, (const double2*)in, (double2*)out);
  } else if (a.shape[r - 1] < 16) {
    permute_elems_kernel<<<blocks_for(a.n, 256, sms), 256, 0, st>>>(a, (const double2*)in, (double2*)out);
  } else {
    const int64_t rows = a.n / a.shape[r - 1];
    permute_rows_kernel<<<blocks_for(rows, 8, sms), 256, 0, st>>>(a, (const double2*)in, (double2*)out);
  }
  mm::note_launches(1);
  return status();
}

MM_API int mm_tensor_sum_inner(int64_t rows, int64_t inner, const mm_c128* in, mm_c128* out, mm_stream_t stream) {
  if (rows < 0 || inner < 0) return MM_ERR_INVALID_ARG;
  const int sms = sms_of_device();
  if (sms == 0) return MM_ERR_NO_DEVICE;
  cudaStream_t st = (cudaStream_t)stream;
  if (rows == 0) return MM_OK;
  if (!out || (inner > 0 && !in)) return MM_ERR_INVALID_ARG;
  if (inner == 0) return cudaMemsetAsync(out, 0, (size_t)rows * sizeof(double2), st) == cudaSuccess ? MM_OK : MM_ERR_CUDA;
  sum_inner_kernel<<<blocks_for(rows, 8, sms), 256, 0, st>>>(rows, inner, (const double2*)in, (double2*)out);
  mm::note_launches(1);
  return status();
}

MM_API int mm_zgemm_batched(int64_t batch, int64_t M, int64_t N, int64_t K, const mm_c128* A, int64_t strideA,
                            const mm_c128* B, int64_t strideB, mm_c128* C, int64_t strideC, mm_stream_t stream) {
  if (batch < 0 || M < 0 || N < 0 || K < 0) return MM_ERR_INVALID_ARG;
  const int sms = sms_of_device();
  if (sms == 0) return MM_ERR_NO_DEVICE;
  cudaStream_t st = (cudaStream_t)stream;
  if (batch == 0 || M == 0 || N == 0) return MM_OK;
  if (!C || (K > 0 && (!A || !B))) return MM_ERR_INVALID_ARG;  // empty operands may have no storage
  if (K == 0) {  // empty sum: zeros
    for (int64_t z = 0; z < batch; ++z)
      if (cudaMemsetAsync(C + z * strideC, 0, (size_t)(M * N) * sizeof(double2), st) != cudaSuccess) return MM_ERR_CUDA;
    return MM_OK;
  }
  if (M > INT32_MAX / 2 || N > INT32_MAX / 2 || K > INT32_MAX / 2) return MM_ERR_TOO_LARGE;
  if (N == 1) {
    zgemv_rows_kernel<<<blocks_for(batch * M, 8, sms), 256, 0, st>>>((const double2*)A, strideA, (const double2*)B,
                                                                     strideB, (double2*)C, strideC, batch, M, K);
  } else if (M == 1) {
    zgemv_cols_kernel<<<blocks_for(batch * N, 256, sms), 256, 0, st>>>((const double2*)A, strideA, (const double2*)B,
                                                                       strideB, (double2*)C, strideC, batch, N, K);
  } else {
    const int64_t tiles32 = ((M + 31) / 32) * ((N + 31) / 32) * batch;
    const bool small = tiles32 < 2 * (int64_t)sms;
    const int bm = small ? 16 : 32, bn = bm;
    const int64_t gy = (M + bm - 1) / bm;
    if (gy > 65535) return MM_ERR_TOO_LARGE;
    dim3 grid((unsigned)((N + bn - 1) / bn), (unsigned)gy, (unsigned)std::min<int64_t>(batch, 65535));
    if (small)
      zgemm_batched_kernel<16, 16><<<grid, 256, 0, st>>>((const double2*)A, strideA, (const double2*)B, strideB,
                                                         (double2*)C, strideC, batch, (int)M, (int)N, (int)K);
    else
      zgemm_batched_kernel<32, 32><<<grid, 256, 0, st>>>((const double2*)A, strideA, (const double2*)B, strideB,
                                                         (double2*)C, strideC, batch, (int)M, (int)N, (int)K);
  }
  mm::note_launches(1);
  return status();
}
