// Fock-space contraction Y = U X (complex128, row-major), the dense step that
// follows the recurrence when a gate tensor is applied to a batch of kets
// (reference: ArrayAnsatz.contract, mrmustard/physics/ansatz/array_ansatz.py:159-226,
// via math.einsum -> opt_einsum -> tensordot -> zgemm, backend_manager.py:526-548).
//
// Two paths:
//  * MM_GEMM_FP64: complex DFMA GEMM (4 FP64 FMA per complex multiply-add).
//  * MM_GEMM_OZAKI_BF16: Ozaki-style split.  Each real and imaginary part of U
//    (per row) and of X (per column) is scaled by a power of two 2^E so that
//    |x| < 2^E, truncated to a 54-bit integer a = floor(|x| 2^(54-E)) and cut
//    into S signed 6-bit slices s_p (a = sum_p s_p 2^(54-6p)), each an integer
//    in [-63, 63] and therefore exact in BF16.  Slice products accumulate on the
//    tensor cores in FP32, exactly (|s_p s_q| <= 3969 < 2^12, so 4096 terms stay
//    below 2^24), and are flushed into 64-bit integer sums every 4096 terms.
//    All pairs (p, q) with the same p + q = d share a scale, so they add up in
//    the same integer sum; each group d = 2 .. S+1 is then scaled once by
//    2^(E_row + F_col - 6d) and added in FP64.  Pairs with p + q > S + 1 are
//    dropped (the Ozaki truncation); the slicing itself truncates below
//    2^(E-54).  The only FP64 work is one conversion and one FMA per element
//    and group, which matters on a part whose FP64 rate is 1/1000 of BF16.
#include <cstdint>
#include <cstdlib>
#include <mutex>

#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>

#include "common.cuh"

namespace {

using mm::cmk;

// ---------------------------------------------------------------- FP64 path
constexpr int FG_BM = 32, FG_BN = 32, FG_BK = 16;

__global__ void __launch_bounds__(256) zgemm_fp64_kernel(const double2* __restrict__ U, const double2* __restrict__ X,
                                                         double2* __restrict__ Y, int M, int N, int K) {
  __shared__ double2 Us[FG_BK][FG_BM];
  __shared__ double2 Xs[FG_BK][FG_BN];
  const int tid = threadIdx.x;
  const int tx = tid & 15, ty = tid >> 4;
  const int m0 = blockIdx.y * FG_BM, n0 = blockIdx.x * FG_BN;
  double2 acc[2][2];
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int j = 0; j < 2; ++j) acc[i][j] = cmk(0.0, 0.0);
  for (int k0 = 0; k0 < K; k0 += FG_BK) {
#pragma unroll
    for (int r = 0; r < 2; ++r) {
      const int idx = tid + r * 256;
      const int row = idx / FG_BK, kk = idx % FG_BK;
      const int gm = m0 + row, gk = k0 + kk;
      Us[kk][row] = (gm < M && gk < K) ? __ldg(U + (int64_t)gm * K + gk) : cmk(0.0, 0.0);
      const int kx = idx / FG_BN, col = idx % FG_BN;
      const int gk2 = k0 + kx, gn = n0 + col;
      Xs[kx][col] = (gk2 < K && gn < N) ? __ldg(X + (int64_t)gk2 * N + gn) : cmk(0.0, 0.0);
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < FG_BK; ++kk) {
      const double2 u0 = Us[kk][ty * 2], u1 = Us[kk][ty * 2 + 1];
      const double2 x0 = Xs[kk][tx * 2], x1 = Xs[kk][tx * 2 + 1];
      acc[0][0] = mm::cfma(u0, x0, acc[0][0]);
      acc[0][1] = mm::cfma(u0, x1, acc[0][1]);
      acc[1][0] = mm::cfma(u1, x0, acc[1][0]);
      acc[1][1] = mm::cfma(u1, x1, acc[1][1]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int j = 0; j < 2; ++j) {
      const int gm = m0 + ty * 2 + i, gn = n0 + tx * 2 + j;
      if (gm < M && gn < N) Y[(int64_t)gm * N + gn] = acc[i][j];
    }
}

// ---------------------------------------------------------------- FP64 tensor-core path
// The same product on the FP64 MMA instruction (mma.sync m8n8k4 .f64, the
// tensor-core FP64 path; tcgen05 has no FP64 kind).  Complex operands are split
// into real and imaginary planes in shared memory; per 8 x 8 output tile
// Y_re += U_re X_re + (-U_im) X_im and Y_im += U_re X_im + U_im X_re, four
// MMAs (256 FMAs each) per tile and k-step of 4.  CTA: 64 x 32 outputs, 4 warps
// of 32 x 16 (4 x 2 tiles); the next K tile is fetched into registers while the
// current one is multiplied.
constexpr int DM_BM = 64, DM_BN = 32, DM_BK = 8, DM_PAD = 4;

__device__ __forceinline__ void dmma_884(double& c0, double& c1, double a, double b) {
  asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1}, {%2}, {%3}, {%0,%1};"
               : "+d"(c0), "+d"(c1)
               : "d"(a), "d"(b));
}

__device__ __forceinline__ double neg(double x) {
  return __longlong_as_double(__double_as_longlong(x) ^ (long long)0x8000000000000000ull);
}

__global__ void __launch_bounds__(128) zgemm_dmma_kernel(const double2* __restrict__ U, const double2* __restrict__ X,
                                                         double2* __restrict__ Y, int M, int N, int K) {
  __shared__ double Ar[DM_BK][DM_BM + DM_PAD], Ai[DM_BK][DM_BM + DM_PAD];  // [k][m]
  __shared__ double Br[DM_BK][DM_BN + DM_PAD], Bi[DM_BK][DM_BN + DM_PAD];  // [k][n]
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int g = lane >> 2, t = lane & 3;
  const int wm = (warp >> 1) * 32, wn = (warp & 1) * 16;
  const int m0 = blockIdx.y * DM_BM, n0 = blockIdx.x * DM_BN;
  double cr[4][2][2], ci[4][2][2];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 2; ++j) cr[i][j][0] = cr[i][j][1] = ci[i][j][0] = ci[i][j][1] = 0.0;
  // global -> register staging: U tile 64 x 8 (4 per thread), X tile 8 x 32 (2 per thread)
  double2 ru[4], rx[2];
  auto fetch = [&](int k0) {
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      const int idx = tid + r * 128, row = idx >> 3, kk = idx & 7;
      const int gm = m0 + row, gk = k0 + kk;
      ru[r] = (gm < M && gk < K) ? __ldg(U + (int64_t)gm * K + gk) : cmk(0.0, 0.0);
    }
#pragma unroll
    for (int r = 0; r < 2; ++r) {
      const int idx = tid + r * 128, kk = idx >> 5, col = idx & 31;
      const int gk = k0 + kk, gn = n0 + col;
      rx[r] = (gk < K && gn < N) ? __ldg(X + (int64_t)gk * N + gn) : cmk(0.0, 0.0);
    }
  };
  auto stash = [&]() {
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      const int idx = tid + r * 128, row = idx >> 3, kk = idx & 7;
      Ar[kk][row] = ru[r].x;
      Ai[kk][row] = ru[r].y;
    }
#pragma unroll
    for (int r = 0; r < 2; ++r) {
      const int idx = tid + r * 128, kk = idx >> 5, col = idx & 31;
      Br[kk][col] = rx[r].x;
      Bi[kk][col] = rx[r].y;
    }
  };
  fetch(0);
  for (int k0 = 0; k0 < K; k0 += DM_BK) {
    stash();
    __syncthreads();
    if (k0 + DM_BK < K) fetch(k0 + DM_BK);
#pragma unroll
    for (int ks = 0; ks < DM_BK; ks += 4) {
      double ar[4], ai[4], bre[2], bim[2];
#pragma unroll
      for (int mt = 0; mt < 4; ++mt) {
        ar[mt] = Ar[ks + t][wm + mt * 8 + g];
        ai[mt] = Ai[ks + t][wm + mt * 8 + g];
      }
#pragma unroll
      for (int nt = 0; nt < 2; ++nt) {
        bre[nt] = Br[ks + t][wn + nt * 8 + g];
        bim[nt] = Bi[ks + t][wn + nt * 8 + g];
      }
#pragma unroll
      for (int mt = 0; mt < 4; ++mt) {
        const double an = neg(ai[mt]);
#pragma unroll
        for (int nt = 0; nt < 2; ++nt) {
          dmma_884(cr[mt][nt][0], cr[mt][nt][1], ar[mt], bre[nt]);
          dmma_884(cr[mt][nt][0], cr[mt][nt][1], an, bim[nt]);
          dmma_884(ci[mt][nt][0], ci[mt][nt][1], ar[mt], bim[nt]);
          dmma_884(ci[mt][nt][0], ci[mt][nt][1], ai[mt], bre[nt]);
        }
      }
    }
    __syncthreads();
  }
  // accumulator (mt, nt, i): row wm + mt*8 + g, column wn + nt*8 + 2t + i
#pragma unroll
  for (int mt = 0; mt < 4; ++mt)
#pragma unroll
    for (int nt = 0; nt < 2; ++nt)
#pragma unroll
      for (int i = 0; i < 2; ++i) {
        const int gm = m0 + wm + mt * 8 + g, gn = n0 + wn + nt * 8 + 2 * t + i;
        if (gm < M && gn < N) Y[(int64_t)gm * N + gn] = cmk(cr[mt][nt][i], ci[mt][nt][i]);
      }
}

// ---------------------------------------------------------------- Ozaki split
constexpr int OZ_BETA = 6;       // bits per slice
constexpr int OZ_MAX_SLICES = 9;  // 54 bits
constexpr int OZ_KALIGN = 64;     // Kp: K padded to a multiple of this (zeros)

// x = (-1)^neg * mant * 2^ex with mant < 2^53; returns the exponent bound E(x)
// with |x| < 2^E(x) (or INT32_MIN for x == 0).
__device__ __forceinline__ int exp_bound(double x) {
  const uint64_t bits = (uint64_t)__double_as_longlong(x);
  const int e = (int)((bits >> 52) & 0x7ff);
  const uint64_t frac = bits & ((1ull << 52) - 1);
  if (e == 0 && frac == 0) return INT32_MIN;
  const int ex = e ? e - 1075 : -1074;
  return ex + 53;
}

// Row exponents of U (M x K): E[r] = max over the row's re and im of exp_bound.
// Also sets every column exponent F[c] to INT32_MIN for col_exp_kernel's atomicMax.
__global__ void __launch_bounds__(256) row_exp_kernel(const double2* __restrict__ U, int M, int K, int* __restrict__ E,
                                                      int N, int* __restrict__ F) {
  const int gtid = blockIdx.x * blockDim.x + threadIdx.x;
  for (int c = gtid; c < N; c += gridDim.x * blockDim.x) F[c] = INT32_MIN;
  const int warp = gtid >> 5, lane = threadIdx.x & 31;
  if (warp >= M) return;
  int m = INT32_MIN;
  for (int k = lane; k < K; k += 32) {
    const double2 v = __ldg(U + (int64_t)warp * K + k);
    m = max(m, max(exp_bound(v.x), exp_bound(v.y)));
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
  if (lane == 0) E[warp] = m;
}

// Column exponents of X (K x N): F[c] = max over the column.  CTA (x, y) covers
// 32 columns and rows [y * COL_EXP_ROWS, +COL_EXP_ROWS): 8 row strides x 32
// columns, coalesced along the row, merged into F with atomicMax.
constexpr int COL_EXP_ROWS = 128;
__global__ void __launch_bounds__(256) col_exp_kernel(const double2* __restrict__ X, int K, int N, int* __restrict__ F) {
  __shared__ int part[8][32];
  const int cl = threadIdx.x & 31, rl = threadIdx.x >> 5;
  const int c = blockIdx.x * 32 + cl;
  const int k0 = blockIdx.y * COL_EXP_ROWS, k1 = min(K, k0 + COL_EXP_ROWS);
  int m = INT32_MIN;
  if (c < N)
    for (int k = k0 + rl; k < k1; k += 8) {
      const double2 v = __ldg(X + (int64_t)k * N + c);
      m = max(m, max(exp_bound(v.x), exp_bound(v.y)));
    }
  part[rl][cl] = m;
  __syncthreads();
  if (rl == 0 && c < N) {
    for (int r = 1; r < 8; ++r) m = max(m, part[r][cl]);
    if (m != INT32_MIN) atomicMax(F + c, m);
  }
}

// Slices of one value against exponent bound E: out[p] for p < S.
__device__ __forceinline__ void slice_value(double x, int E, int S, __nv_bfloat16* out, int64_t pstride) {
  const uint64_t bits = (uint64_t)__double_as_longlong(x);
  const int e = (int)((bits >> 52) & 0x7ff);
  const uint64_t frac = bits & ((1ull << 52) - 1);
  const bool neg = (bits >> 63) != 0;
  uint64_t a = 0;
  if (E != INT32_MIN && (e != 0 || frac != 0)) {
    const uint64_t mant = e ? (frac | (1ull << 52)) : frac;
    const int ex = e ? e - 1075 : -1074;
    const int shift = ex + 54 - E;  // <= 1 because |x| < 2^E
    if (shift >= 0) a = mant << shift;
    else if (shift > -64) a = mant >> (-shift);
  }
  for (int p = 0; p < S; ++p) {
    const int v = (int)((a >> (54 - OZ_BETA * (p + 1))) & ((1u << OZ_BETA) - 1));
    out[p * pstride] = __float2bfloat16_rn((float)(neg ? -v : v));
  }
}

// U (M x K) -> Us[p][comp][M][Kp] (comp 0 = re, 1 = im); zero padding for k >= K.
__global__ void __launch_bounds__(256) split_u_kernel(const double2* __restrict__ U, int M, int K, int Kp, int S,
                                                      const int* __restrict__ E, __nv_bfloat16* __restrict__ Us) {
  const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (int64_t)M * Kp) return;
  const int r = (int)(idx / Kp), k = (int)(idx - (int64_t)r * Kp);
  const int64_t plane = (int64_t)M * Kp;  // one (p, comp) plane
  double2 v = cmk(0.0, 0.0);
  if (k < K) v = __ldg(U + (int64_t)r * K + k);
  const int Er = E[r];
  slice_value(v.x, Er, S, Us + idx, 2 * plane);
  slice_value(v.y, Er, S, Us + plane + idx, 2 * plane);
}

// X (K x N) -> Xs[q][comp][N][Kp] (transposed: each column's K values contiguous).
__global__ void __launch_bounds__(256) split_x_kernel(const double2* __restrict__ X, int K, int N, int Kp, int S,
                                                      const int* __restrict__ F, __nv_bfloat16* __restrict__ Xs) {
  const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (int64_t)N * Kp) return;
  const int c = (int)(idx / Kp), k = (int)(idx - (int64_t)c * Kp);
  const int64_t plane = (int64_t)N * Kp;
  double2 v = cmk(0.0, 0.0);
  if (k < K) v = __ldg(X + (int64_t)k * N + c);
  const int Fc = F[c];
  slice_value(v.x, Fc, S, Xs + idx, 2 * plane);
  slice_value(v.y, Fc, S, Xs + plane + idx, 2 * plane);
}

// t * 2^s for an integer |t| < 2^53 as a double, built with integer operations only (exact: a
// power-of-two scale of an exactly representable integer), so the FP64 pipe -- 1/64 rate on
// this part -- is not spent on conversions and scalings.  Falls back to FP64 arithmetic when the
// result would leave the normal range.
__device__ __forceinline__ double pow2(int e);
__device__ __forceinline__ double scaled_i2d(long long t, int s) {
  if (t == 0) return 0.0;
  const unsigned long long a = t < 0 ? 0ull - (unsigned long long)t : (unsigned long long)t;
  const int e = 63 - __clzll((long long)a);  // a = 1.f * 2^e
  const int ex = e + s + 1023;
  if (e > 52 || ex <= 0 || ex >= 2047) return (double)t * pow2(s);
  const unsigned long long mant = (a << (52 - e)) & ((1ull << 52) - 1);
  return __longlong_as_double((long long)(((t < 0 ? 1ull : 0ull) << 63) | ((unsigned long long)ex << 52) | mant));
}

__device__ __forceinline__ double pow2(int e) {
  if (e >= -1022 && e <= 1023) return __longlong_as_double((long long)(e + 1023) << 52);
  return ldexp(1.0, e);
}

// ---------------------------------------------------------------- tcgen05 path
// Warp-specialised Blackwell kernel for the slice products.  One CTA owns a
// 128-row x 40-complex-column tile of Y (a 2500 x 256 product is 20 x 7 = 140
// tiles: one wave on 152 SMs).  For every slice pair (p, q) and every chunk of
// at most 4096 K values (one "unit"), the tensor cores compute two M = 128,
// N = 80 products into TMEM:
//     acc_r = U_re,p [X_re,q | X_im,q]   (columns 0..39: rr, 40..79: ri)
//     acc_i = U_im,p [X_re,q | X_im,q]   (columns 0..39: ir, 40..79: ii)
// The kernel is bound by the latency of its TMA ring (bytes in flight per SM),
// not by L2 bandwidth: sharing the U tiles of a row of CTAs through cluster
// multicast was measured and gained nothing, so every CTA loads its own.
// with FP32 accumulation that is exact for 6-bit slices.  Roles:
//   warp 0, lane 0: TMA producer (3-stage ring of [U_re | U_im | X_re ; X_im] K-blocks of 64),
//   warp 1, lane 0: MMA issuer (tcgen05.mma, tcgen05.commit into mbarriers),
//   warps 2..5:      epilogue (tcgen05.ld of a finished unit, exact integer sums per slice order,
//                    one FP64 scaling per order into Y).
// Accumulators are double-buffered (TMEM columns 0 and 256) so the epilogue of one
// unit overlaps the MMAs of the next.  Every mbarrier wait is bounded; on a
// timeout the CTA records MM_ERR_WAIT_TIMEOUT, lets its in-flight copies land,
// frees its TMEM and returns.
constexpr int TC_BM = 128;                                // Y rows per CTA (MMA M)
constexpr int TC_NC = 40;                                 // Y complex columns per CTA (MMA N = 80)
constexpr int TC_BK = 64;                                 // K per stage: one 128-byte swizzled row of BF16
constexpr int TC_A_BYTES = TC_BM * TC_BK * 2;             // 16 KB per U component
constexpr int TC_B_BYTES = 2 * TC_NC * TC_BK * 2;         // 10 KB ([X_re; X_im] rows)
constexpr int TC_STAGE_BYTES = 2 * TC_A_BYTES + TC_B_BYTES;  // 42 KB (a multiple of 1 KB: swizzle atoms stay aligned)
// Slice-order sums [comp][col][row]: int32 while 9 pairs x Kp x 2 x 63^2 < 2^31,
// held in TMEM columns TC_T_COL.. (free between the two accumulator buffers), so
// five stages fit in shared memory; int64 beyond, in shared memory (three stages).
constexpr int TC_KP_INT32_MAX = 30000;
// tbytes: bytes per shared-memory order sum (0: sums in TMEM)
constexpr int tc_smem_bytes(int tbytes, int stages) {
  return 1024 + stages * TC_STAGE_BYTES + 2 * TC_NC * TC_BM * tbytes + 256;
}
constexpr int TC_TMEM_COLS = 512;
constexpr int TC_ACC_STRIDE = 256;                        // TMEM columns between the two accumulator buffers
constexpr int TC_T_COL = 4 * TC_NC;                       // int32 order sums: [re cols | im cols] after buffer 0
static_assert(TC_NC % 8 == 0 && 6 * TC_NC <= TC_ACC_STRIDE, "accumulator and order-sum layout");
static_assert(TC_STAGE_BYTES % 1024 == 0 && (TC_B_BYTES / 2) % 1024 == 0, "swizzle atoms");
constexpr int TC_THREADS = 192;
// kind::f16 instruction descriptor: D = F32, A = B = BF16, both K-major, N = 2 * TC_NC, M = 128.
constexpr uint32_t TC_IDESC = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)((2 * TC_NC) >> 3) << 17) |
                              ((uint32_t)(128 >> 4) << 24);

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(bar), "r"(parity)
      : "memory");
  return ok != 0;
}
// Bounded wait: false when another role gave up or the budget ran out (then records the error).
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, volatile int* abort_flag, mm::WsHeader* h,
                                          uint64_t budget_ns) {
  const uint64_t t0 = mm::globaltimer_ns();
  for (uint32_t it = 0;; ++it) {
    if (mbar_try_wait(bar, parity)) return true;
    if ((it & 63) == 63) {
      if (*abort_flag) return false;
      if (mm::globaltimer_ns() - t0 > budget_ns) {
        *abort_flag = 1;
        if (h) mm::set_status(h, MM_ERR_WAIT_TIMEOUT);
        return false;
      }
    }
  }
}
__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap* map, int x, int y, uint32_t bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];"
      ::"r"(dst), "l"((uint64_t)map), "r"(x), "r"(y), "r"(bar)
      : "memory");
}
// K-major, 128-byte swizzle smem descriptor (sm_100 format): start >> 4, LBO 16 B, SBO 1024 B, version 1.
__device__ __forceinline__ uint64_t sw128_desc(uint32_t addr) {
  return (uint64_t)((addr & 0x3FFFF) >> 4) | ((uint64_t)1 << 16) | ((uint64_t)(1024 >> 4) << 32) |
         ((uint64_t)1 << 46) | ((uint64_t)2 << 61);
}
__device__ __forceinline__ void tc_mma(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
      "l"(adesc), "l"(bdesc), "r"(TC_IDESC), "r"(accumulate)
      : "memory");
}
__device__ __forceinline__ void tc_commit(uint32_t bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_ld8(uint32_t taddr, uint32_t (&r)[8]) {
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
               : "r"(taddr));
}
__device__ __forceinline__ void tc_st8(uint32_t taddr, const uint32_t (&r)[8]) {
  asm volatile("tcgen05.st.sync.aligned.32x32b.x8.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8};" ::"r"(taddr), "r"(r[0]),
               "r"(r[1]), "r"(r[2]), "r"(r[3]), "r"(r[4]), "r"(r[5]), "r"(r[6]), "r"(r[7])
               : "memory");
}
__device__ __forceinline__ void tc_wait_st() { asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory"); }
__device__ __forceinline__ void tc_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

// Units of a CTA, in order: slice order d = 2 .. S+1; within an order the
// pairs p in [max(1, d-S), min(S, d-1)], ascending for even d and descending
// for odd d (consecutive units then reuse the U slices still in L2); K chunks
// of at most 4096.  Every role walks the same sequence.
struct UnitIter {
  int S, nkb, chunk_kb;
  int d, p, c;  // current unit
  __device__ int plo() const { return d - S > 1 ? d - S : 1; }
  __device__ int phi() const { return d - 1 < S ? d - 1 : S; }
  __device__ bool desc() const { return (d & 1) != 0; }
  __device__ void start(int S_, int nkb_, int chunk_kb_) {
    S = S_;
    nkb = nkb_;
    chunk_kb = chunk_kb_;
    d = 2;
    p = 1;
    c = 0;
  }
  __device__ bool valid() const { return d <= S + 1; }
  __device__ int q() const { return d - p; }
  __device__ int kb_begin() const { return c * chunk_kb; }
  __device__ int kb_end() const { return min(nkb, (c + 1) * chunk_kb); }
  __device__ bool last_of_order() const { return p == (desc() ? plo() : phi()) && kb_end() >= nkb; }
  __device__ void next() {
    if (kb_end() < nkb) {
      ++c;
      return;
    }
    c = 0;
    if (desc() ? p > plo() : p < phi()) {
      p += desc() ? -1 : 1;
      return;
    }
    ++d;
    p = desc() ? phi() : plo();
  }
};

// TT: type of the slice-order sums; TMEM_T: they live in TMEM (int32 only).
template <typename TT, int TC_STAGES, bool TMEM_T>
__global__ void __launch_bounds__(TC_THREADS, 1)
    ozaki_tc_kernel(const __grid_constant__ CUtensorMap tmap_u, const __grid_constant__ CUtensorMap tmap_x,
                    const int* __restrict__ E, const int* __restrict__ F, double2* __restrict__ Y, int M, int N,
                    int Kp, int S, mm::WsHeader* h, uint64_t budget_ns) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  unsigned char* smem = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  unsigned char* stages = smem;
  static_assert(!TMEM_T || sizeof(TT) == 4, "TMEM sums are 32-bit");
  constexpr int t_bytes = TMEM_T ? 0 : 2 * TC_NC * TC_BM * (int)sizeof(TT);
  TT* T = reinterpret_cast<TT*>(smem + TC_STAGES * TC_STAGE_BYTES);  // [2][TC_NC][TC_BM] (shared-memory sums)
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem + TC_STAGES * TC_STAGE_BYTES + t_bytes);
  // bars: full[STAGES], empty[STAGES], accf[2], acce[2], drain
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars + 2 * TC_STAGES + 5);
  volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_slot + 1);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int m0 = blockIdx.y * TC_BM, n0 = blockIdx.x * TC_NC;
  const int nkb = Kp / TC_BK;
  const int chunk_kb = 4096 / TC_BK;
  auto full = [&](int s) { return smem_u32(bars + s); };
  auto empty = [&](int s) { return smem_u32(bars + TC_STAGES + s); };
  auto accf = [&](int b) { return smem_u32(bars + 2 * TC_STAGES + b); };
  auto acce = [&](int b) { return smem_u32(bars + 2 * TC_STAGES + 2 + b); };
  const uint32_t drain = smem_u32(bars + 2 * TC_STAGES + 4);

  if (threadIdx.x == 0) {
    for (int s = 0; s < TC_STAGES; ++s) {
      mbar_init(full(s), 1);
      mbar_init(empty(s), 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(accf(b), 1);
      mbar_init(acce(b), 128);
    }
    mbar_init(drain, 1);
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {  // whole warp: TMEM allocation
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"(TC_TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;

  if (warp == 0 && lane == 0) {
    // ------------------------------------------------------------ TMA producer
    int stage = 0;
    uint32_t phase = 0;
    uint32_t armed_parity[TC_STAGES];
    bool armed[TC_STAGES];
    for (int s = 0; s < TC_STAGES; ++s) armed[s] = false;
    UnitIter u;
    u.start(S, nkb, chunk_kb);
    bool ok = true;
    for (; ok && u.valid(); u.next()) {
      const int yu = (u.p - 1) * 2 * M + m0, yx = (u.q() - 1) * 2 * N + n0;
      for (int kb = u.kb_begin(); kb < u.kb_end(); ++kb) {
        if (!mbar_wait(empty(stage), phase ^ 1, abort_flag, h, budget_ns)) {
          ok = false;
          break;
        }
        unsigned char* st = stages + stage * TC_STAGE_BYTES;
        mbar_expect_tx(full(stage), TC_STAGE_BYTES);
        armed[stage] = true;
        armed_parity[stage] = phase;
        const int x = kb * TC_BK;
        tma_load_2d(smem_u32(st), &tmap_u, x, yu, full(stage));
        tma_load_2d(smem_u32(st + TC_A_BYTES), &tmap_u, x, yu + M, full(stage));
        tma_load_2d(smem_u32(st + 2 * TC_A_BYTES), &tmap_x, x, yx, full(stage));
        tma_load_2d(smem_u32(st + 2 * TC_A_BYTES + TC_B_BYTES / 2), &tmap_x, x, yx + N, full(stage));
        if (++stage == TC_STAGES) {
          stage = 0;
          phase ^= 1;
        }
      }
    }
    if (!ok) {  // let copies in flight land before the CTA's shared memory goes away
      for (int s = 0; s < TC_STAGES; ++s)
        if (armed[s]) {
          const uint64_t t0 = mm::globaltimer_ns();
          while (!mbar_try_wait(full(s), armed_parity[s]) && mm::globaltimer_ns() - t0 < budget_ns) {
          }
        }
    }
  } else if (warp == 1 && lane == 0) {
    // ------------------------------------------------------------ MMA issuer
    int stage = 0;
    uint32_t phase = 0;
    int abuf = 0;
    uint32_t aphase = 0;
    UnitIter u;
    u.start(S, nkb, chunk_kb);
    bool ok = true;
    for (; ok && u.valid(); u.next()) {
      if (!mbar_wait(acce(abuf), aphase ^ 1, abort_flag, h, budget_ns)) break;
      tc_fence_after();
      const uint32_t d_r = tmem + (uint32_t)(abuf * TC_ACC_STRIDE), d_i = d_r + 2 * TC_NC;
      for (int kb = u.kb_begin(); kb < u.kb_end(); ++kb) {
        if (!mbar_wait(full(stage), phase, abort_flag, h, budget_ns)) {
          ok = false;
          break;
        }
        tc_fence_after();
        const uint32_t st = smem_u32(stages + stage * TC_STAGE_BYTES);
#pragma unroll
        for (int k16 = 0; k16 < TC_BK / 16; ++k16) {
          const uint32_t koff = (uint32_t)k16 * 32;
          const uint32_t acc = (kb > u.kb_begin() || k16 > 0) ? 1u : 0u;
          const uint64_t bdesc = sw128_desc(st + 2 * TC_A_BYTES + koff);
          tc_mma(d_r, sw128_desc(st + koff), bdesc, acc);
          tc_mma(d_i, sw128_desc(st + TC_A_BYTES + koff), bdesc, acc);
        }
        tc_commit(empty(stage));  // frees the stage once these MMAs have read it
        if (++stage == TC_STAGES) {
          stage = 0;
          phase ^= 1;
        }
      }
      if (!ok) break;
      tc_commit(accf(abuf));  // the unit's accumulators are complete
      if (++abuf == 2) {
        abuf = 0;
        aphase ^= 1;
      }
    }
    // every MMA issued above has completed before TMEM can be freed
    tc_commit(drain);
    const uint64_t t0 = mm::globaltimer_ns();
    while (!mbar_try_wait(drain, 0) && mm::globaltimer_ns() - t0 < budget_ns) {
    }
  } else if (warp >= 2) {
    // ------------------------------------------------------------ epilogue
    const int lane_base = 32 * (warp & 3);
    const int row = lane_base + lane;
    const int gm = m0 + row;
    const uint32_t trow = tmem + ((uint32_t)lane_base << 16);  // this warp's 32 TMEM lanes
    const uint32_t zeros[8] = {0u, 0u, 0u, 0u, 0u, 0u, 0u, 0u};
    if constexpr (TMEM_T) {
#pragma unroll
      for (int c8 = 0; c8 < 2 * TC_NC / 8; ++c8) tc_st8(trow + TC_T_COL + c8 * 8, zeros);
      tc_wait_st();
    } else {
      for (int c = 0; c < TC_NC; ++c) T[(0 * TC_NC + c) * TC_BM + row] = T[(1 * TC_NC + c) * TC_BM + row] = 0;
    }
    int abuf = 0;
    uint32_t aphase = 0;
    UnitIter u;
    u.start(S, nkb, chunk_kb);
    for (; u.valid(); u.next()) {
      // one lane waits, the warp follows it, so the warp-wide tcgen05.ld stays convergent
      int okw = lane == 0 ? (int)mbar_wait(accf(abuf), aphase, abort_flag, h, budget_ns) : 0;
      okw = __shfl_sync(0xffffffffu, okw, 0);
      if (!okw) break;
      tc_fence_after();
      const uint32_t base = trow + (uint32_t)(abuf * TC_ACC_STRIDE);
#pragma unroll
      for (int c8 = 0; c8 < TC_NC / 8; ++c8) {
        uint32_t rr[8], ri[8], ir[8], ii[8], tr[8], ti[8];
        tc_ld8(base + c8 * 8, rr);
        tc_ld8(base + TC_NC + c8 * 8, ri);
        tc_ld8(base + 2 * TC_NC + c8 * 8, ir);
        tc_ld8(base + 3 * TC_NC + c8 * 8, ii);
        if constexpr (TMEM_T) {
          tc_ld8(trow + TC_T_COL + c8 * 8, tr);
          tc_ld8(trow + TC_T_COL + TC_NC + c8 * 8, ti);
        }
        tc_wait_ld();
#pragma unroll
        for (int j = 0; j < 8; ++j) {
          const int c = c8 * 8 + j;
          const TT re = (TT)__float2int_rn(__uint_as_float(rr[j])) - (TT)__float2int_rn(__uint_as_float(ii[j]));
          const TT im = (TT)__float2int_rn(__uint_as_float(ri[j])) + (TT)__float2int_rn(__uint_as_float(ir[j]));
          if constexpr (TMEM_T) {
            tr[j] = (uint32_t)((int)tr[j] + (int)re);
            ti[j] = (uint32_t)((int)ti[j] + (int)im);
          } else {
            T[(0 * TC_NC + c) * TC_BM + row] += re;
            T[(1 * TC_NC + c) * TC_BM + row] += im;
          }
        }
        if constexpr (TMEM_T) {
          tc_st8(trow + TC_T_COL + c8 * 8, tr);
          tc_st8(trow + TC_T_COL + TC_NC + c8 * 8, ti);
        }
      }
      if constexpr (TMEM_T) tc_wait_st();
      tc_fence_before();
      mbar_arrive(acce(abuf));
      if (++abuf == 2) {
        abuf = 0;
        aphase ^= 1;
      }
      if (u.last_of_order()) {  // add this slice order's sums to Y in FP64, then clear them
        const int er = gm < M ? E[gm] : INT32_MIN;
#pragma unroll
        for (int c8 = 0; c8 < TC_NC / 8; ++c8) {
          long long vre[8], vim[8];
          if constexpr (TMEM_T) {
            uint32_t tr[8], ti[8];
            tc_ld8(trow + TC_T_COL + c8 * 8, tr);
            tc_ld8(trow + TC_T_COL + TC_NC + c8 * 8, ti);
            tc_wait_ld();
#pragma unroll
            for (int j = 0; j < 8; ++j) {
              vre[j] = (int)tr[j];
              vim[j] = (int)ti[j];
            }
            tc_st8(trow + TC_T_COL + c8 * 8, zeros);
            tc_st8(trow + TC_T_COL + TC_NC + c8 * 8, zeros);
          } else {
#pragma unroll
            for (int j = 0; j < 8; ++j) {
              TT& tre = T[(0 * TC_NC + c8 * 8 + j) * TC_BM + row];
              TT& tim = T[(1 * TC_NC + c8 * 8 + j) * TC_BM + row];
              vre[j] = (long long)tre;
              vim[j] = (long long)tim;
              tre = 0;
              tim = 0;
            }
          }
          // every load of the group is issued before its stores, so the read-modify-writes of a row
          // overlap instead of forming one chain of memory latencies
          double2 y[8], o[8];
          double2* yrow = Y + (int64_t)gm * N + n0 + c8 * 8;
#pragma unroll
          for (int j = 0; j < 8; ++j) {
            const int gn = n0 + c8 * 8 + j;
            y[j] = cmk(0.0, 0.0);
            o[j] = cmk(0.0, 0.0);
            if (gm < M && gn < N) {
              const int fc = F[gn];
              if (er != INT32_MIN && fc != INT32_MIN) {
                const int sh = er + fc - OZ_BETA * u.d;
                y[j] = cmk(scaled_i2d(vre[j], sh), scaled_i2d(vim[j], sh));
              }
              if (u.d != 2) o[j] = yrow[j];
            }
          }
#pragma unroll
          for (int j = 0; j < 8; ++j) {
            const int gn = n0 + c8 * 8 + j;
            if (gm < M && gn < N) yrow[j] = u.d == 2 ? y[j] : cmk(o[j].x + y[j].x, o[j].y + y[j].y);
          }
        }
        if constexpr (TMEM_T) tc_wait_st();
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TC_TMEM_COLS) : "memory");
  }
}

}  // namespace

namespace {
int64_t round_up(int64_t x, int64_t a) { return (x + a - 1) / a * a; }

struct OzLayout {
  int64_t Kp = 0;
  size_t us = 0, xs = 0, e = 0, f = 0, total = 0;
};

// Workspace: 512-byte status header, U slices, X slices, row / column exponents.
OzLayout oz_layout(int64_t M, int64_t N, int64_t K, int S) {
  OzLayout L;
  L.Kp = round_up(K, OZ_KALIGN);
  size_t off = sizeof(mm::WsHeader);
  L.us = off;
  off = round_up(off + (size_t)S * 2 * M * L.Kp * sizeof(__nv_bfloat16), 256);
  L.xs = off;
  off = round_up(off + (size_t)S * 2 * N * L.Kp * sizeof(__nv_bfloat16), 256);
  L.e = off;
  off = round_up(off + (size_t)M * sizeof(int), 256);
  L.f = off;
  off = round_up(off + (size_t)N * sizeof(int), 256);
  L.total = off;
  return L;
}
PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    cudaGetLastError();
  });
  return fn;
}

// 2-D BF16 tensor map over `rows` x `cols` (row-major, cols contiguous), box {64, box_rows}, 128-byte swizzle.
bool make_map(CUtensorMap* map, void* base, uint64_t rows, uint64_t cols, uint32_t box_rows) {
  auto enc = tensor_map_encoder();
  if (!enc) return false;
  const cuuint64_t dims[2] = {cols, rows};
  const cuuint64_t strides[1] = {cols * 2};
  const cuuint32_t box[2] = {64, box_rows};
  const cuuint32_t estr[2] = {1, 1};
  return enc(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, base, dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
             CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
             CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

uint64_t tc_budget_ns() {
  static uint64_t v = [] {
    const char* e = getenv("MM_WAIT_BUDGET_NS");
    return e ? strtoull(e, nullptr, 10) : 2000000000ull;
  }();
  return v;
}
}  // namespace

extern "C" {

MM_API size_t mm_fock_gemm_workspace_bytes(int mode, int64_t M, int64_t N, int64_t K, int slices) {
  if (M < 1 || N < 1 || K < 1) return 0;
  if (mode == 0 || mode == 2) return 256;
  if (mode != 1 || slices < 2 || slices > OZ_MAX_SLICES) return 0;
  return oz_layout(M, N, K, slices).total;
}

MM_API int mm_fock_gemm(int mode, int64_t M, int64_t N, int64_t K, const mm_c128* U, const mm_c128* X, mm_c128* Y,
                        int slices, void* ws, size_t ws_bytes, mm_stream_t stream) {
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    return MM_ERR_NO_DEVICE;
  }
  if (M < 1 || N < 1 || K < 1 || !U || !X || !Y) return MM_ERR_INVALID_ARG;
  if (M > INT32_MAX / 2 || N > INT32_MAX / 2 || K > INT32_MAX / 2) return MM_ERR_TOO_LARGE;
  cudaStream_t st = (cudaStream_t)stream;
  if (mode == 0) {
    dim3 grid((unsigned)((N + FG_BN - 1) / FG_BN), (unsigned)((M + FG_BM - 1) / FG_BM));
    if (grid.y > 65535) return MM_ERR_TOO_LARGE;
    zgemm_fp64_kernel<<<grid, 256, 0, st>>>((const double2*)U, (const double2*)X, (double2*)Y, (int)M, (int)N, (int)K);
    mm::note_launches(1);
    return cudaGetLastError() == cudaSuccess ? MM_OK : MM_ERR_CUDA;
  }
  if (mode == 2) {
    dim3 grid((unsigned)((N + DM_BN - 1) / DM_BN), (unsigned)((M + DM_BM - 1) / DM_BM));
    if (grid.y > 65535) return MM_ERR_TOO_LARGE;
    zgemm_dmma_kernel<<<grid, 128, 0, st>>>((const double2*)U, (const double2*)X, (double2*)Y, (int)M, (int)N, (int)K);
    mm::note_launches(1);
    return cudaGetLastError() == cudaSuccess ? MM_OK : MM_ERR_CUDA;
  }
  if (mode != 1) return MM_ERR_INVALID_ARG;
  if (slices < 2 || slices > OZ_MAX_SLICES) return MM_ERR_INVALID_ARG;
  const OzLayout L = oz_layout(M, N, K, slices);
  if (ws == nullptr || ((uintptr_t)ws % 256) != 0 || ws_bytes < L.total) return MM_ERR_WORKSPACE;
  char* w = static_cast<char*>(ws);
  __nv_bfloat16* Us = reinterpret_cast<__nv_bfloat16*>(w + L.us);
  __nv_bfloat16* Xs = reinterpret_cast<__nv_bfloat16*>(w + L.xs);
  int* E = reinterpret_cast<int*>(w + L.e);
  int* F = reinterpret_cast<int*>(w + L.f);
  const int Kp = (int)L.Kp;
  row_exp_kernel<<<(unsigned)((M * 32 + 255) / 256), 256, 0, st>>>((const double2*)U, (int)M, (int)K, E, (int)N, F);
  col_exp_kernel<<<dim3((unsigned)((N + 31) / 32), (unsigned)((K + COL_EXP_ROWS - 1) / COL_EXP_ROWS)), 256, 0, st>>>(
      (const double2*)X, (int)K, (int)N, F);
  split_u_kernel<<<(unsigned)((M * Kp + 255) / 256), 256, 0, st>>>((const double2*)U, (int)M, (int)K, Kp, slices, E, Us);
  split_x_kernel<<<(unsigned)((N * Kp + 255) / 256), 256, 0, st>>>((const double2*)X, (int)K, (int)N, Kp, slices, F, Xs);
  CUtensorMap tu, tx;
  if (!make_map(&tu, Us, (uint64_t)slices * 2 * M, (uint64_t)Kp, TC_BM) ||
      !make_map(&tx, Xs, (uint64_t)slices * 2 * N, (uint64_t)Kp, TC_NC))
    return MM_ERR_UNSUPPORTED;
  static std::once_flag attr_once;
  std::call_once(attr_once, [] {
    cudaFuncSetAttribute(ozaki_tc_kernel<int, 5, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         tc_smem_bytes(0, 5));
    cudaFuncSetAttribute(ozaki_tc_kernel<long long, 3, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         tc_smem_bytes(8, 3));
  });
  dim3 grid((unsigned)((N + TC_NC - 1) / TC_NC), (unsigned)((M + TC_BM - 1) / TC_BM));
  if (grid.y > 65535) return MM_ERR_TOO_LARGE;
  mm::WsHeader* h = reinterpret_cast<mm::WsHeader*>(w);
  if (Kp <= TC_KP_INT32_MAX)
    ozaki_tc_kernel<int, 5, true><<<grid, TC_THREADS, tc_smem_bytes(0, 5), st>>>(
        tu, tx, E, F, (double2*)Y, (int)M, (int)N, Kp, slices, h, tc_budget_ns());
  else
    ozaki_tc_kernel<long long, 3, false><<<grid, TC_THREADS, tc_smem_bytes(8, 3), st>>>(
        tu, tx, E, F, (double2*)Y, (int)M, (int)N, Kp, slices, h, tc_budget_ns());
  mm::note_launches(5);  // exponents, slices, products
  return cudaGetLastError() == cudaSuccess ? MM_OK : MM_ERR_CUDA;
}

}  // extern "C"
