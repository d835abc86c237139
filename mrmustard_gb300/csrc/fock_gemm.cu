// Fock-space contraction Y = U X (complex128, row-major), the dense step that
// follows the recurrence when a gate tensor is applied to a batch of kets
// (reference: ArrayAnsatz.contract, mrmustard/physics/ansatz/array_ansatz.py:159-226,
// via math.einsum -> opt_einsum -> tensordot -> zgemm, backend_manager.py:526-548).
//
// Two paths:
//  * MM_GEMM_FP64: complex DFMA GEMM (4 FP64 FMA per complex multiply-add).
//  * MM_GEMM_OZAKI_BF16: Ozaki-style split.  Each real and imaginary part of U
//    (per row) and of X (per column) is scaled by a power of two 2^E so that
//    |x| < 2^E, truncated to a 55-bit integer a = floor(|x| 2^(55-E)) and
//    written in S balanced base-256 digits s_p (a = sum_p s_p 2^(8(S-1-p)),
//    every digit in [-128, 128]), each an integer exact in BF16.  Digit products
//    accumulate on the tensor cores in FP32, exactly (|s_p s_q| <= 2^14, so 1024
//    terms stay within 2^24), and are flushed into integer sums every 1024 terms.
//    All pairs (p, q) with the same p + q = d share a scale, so they add up in
//    the same integer sum; group d = 2 .. S+1 carries the scale
//    2^(E_row + F_col + 8(2S - d) - 110), so all groups of an element add up
//    exactly in one 128-bit integer, rounded once to double.  Pairs with
//    p + q > S + 1 are dropped (the Ozaki truncation: 28 of the 49 pairs kept at
//    S = 7); the slicing itself truncates below 2^(E-55).  No step uses FP64
//    arithmetic, which matters on a part whose FP64 rate is 1/1000 of BF16.
#include <algorithm>
#include <cstdint>
#include <cstdlib>
#include <mutex>

#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>

#include "common.cuh"
#include "i128_round.cuh"

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
constexpr int OZ_BETA = 8;        // bits per slice (balanced digits in [-128, 128])
constexpr int OZ_MAX_SLICES = 7;  // digits of the 55-bit integer a
constexpr int OZ_TOP = 55;        // a = floor(|x| 2^(OZ_TOP - E)) < 2^OZ_TOP
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

// Digits of one value against exponent bound E: dig[p] for p < OZ_MAX_SLICES, the balanced
// base-256 digits of a = floor(|x| 2^(OZ_TOP - E)) (digit 0 most significant), negated for x < 0:
// digits 1..6 in [-128, 127], digit 0 (a >> 48 < 128, plus a carry) in [0, 128].  Branch-free: with
// u_p = d_p + 128 for p >= 1, a + 0x808080808080 = d_0 2^48 + sum_p u_p 2^(8(6-p)) has the u_p as its
// low bytes (each in [0, 255]) and d_0 above them.  Keeping only the S most significant digits
// (S < OZ_MAX_SLICES) leaves a within half a unit of the last kept digit.
static_assert(OZ_MAX_SLICES == 7 && OZ_BETA == 8 && OZ_TOP == 55, "digit layout of value_digits");
__device__ __forceinline__ void value_digits(double x, int E, int (&dig)[OZ_MAX_SLICES]) {
  const uint64_t bits = (uint64_t)__double_as_longlong(x);
  const int e = (int)((bits >> 52) & 0x7ff);
  const uint64_t frac = bits & ((1ull << 52) - 1);
  const bool neg = (bits >> 63) != 0;
  uint64_t a = 0;
  if (E != INT32_MIN && (e != 0 || frac != 0)) {
    const uint64_t mant = e ? (frac | (1ull << 52)) : frac;
    const int ex = e ? e - 1075 : -1074;
    const int shift = ex + OZ_TOP - E;  // <= 2 because |x| < 2^E
    if (shift >= 0) a = mant << shift;
    else if (shift > -64) a = mant >> (-shift);
  }
  const uint64_t u = a + 0x808080808080ull;
  const int sg = neg ? -1 : 1;
  dig[0] = sg * (int)(u >> 48);
#pragma unroll
  for (int p = 1; p < OZ_MAX_SLICES; ++p) dig[p] = sg * ((int)((u >> (8 * (OZ_MAX_SLICES - 1 - p))) & 0xff) - 128);
}

// Digits p < S of four consecutive values (of one plane row) as four BF16 (exact: |digit| <= 128)
// packed into one 8-byte store per plane.
__device__ __forceinline__ void store_digits4(const int (&d)[4][OZ_MAX_SLICES], int S, __nv_bfloat16* out,
                                              int64_t pstride) {
#pragma unroll
  for (int p = 0; p < OZ_MAX_SLICES; ++p) {
    if (p >= S) break;
    uint2 w;
    w.x = (uint32_t)__bfloat16_as_ushort(__float2bfloat16_rn((float)d[0][p])) |
          ((uint32_t)__bfloat16_as_ushort(__float2bfloat16_rn((float)d[1][p])) << 16);
    w.y = (uint32_t)__bfloat16_as_ushort(__float2bfloat16_rn((float)d[2][p])) |
          ((uint32_t)__bfloat16_as_ushort(__float2bfloat16_rn((float)d[3][p])) << 16);
    *reinterpret_cast<uint2*>(out + p * pstride) = w;
  }
}

// One CTA per row r of U (M x K): E[r] = max over the row's re and im of exp_bound, then the
// row's slices Us[p][comp][r][0 .. Kp) (comp 0 = re, 1 = im; zeros for k >= K), four K values per
// thread (the second pass reads the row from cache).  The CTAs also set every column exponent
// F[c] to INT32_MIN for col_exp_kernel's atomicMax, which runs after this kernel.
__global__ void __launch_bounds__(256) split_u_kernel(const double2* __restrict__ U, int M, int K, int Kp, int S,
                                                      int* __restrict__ E, int N, int* __restrict__ F,
                                                      __nv_bfloat16* __restrict__ Us) {
  __shared__ int wmax[8];
  const int r = blockIdx.x;
  for (int c = r * 256 + (int)threadIdx.x; c < N; c += gridDim.x * 256) F[c] = INT32_MIN;
  const double2* row = U + (int64_t)r * K;
  int m = INT32_MIN;
  for (int k = threadIdx.x; k < K; k += 256) {
    const double2 v = __ldg(row + k);
    m = max(m, max(exp_bound(v.x), exp_bound(v.y)));
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) wmax[threadIdx.x >> 5] = m;
  __syncthreads();
  int Er = wmax[0];
#pragma unroll
  for (int w = 1; w < 8; ++w) Er = max(Er, wmax[w]);
  if (threadIdx.x == 0) E[r] = Er;
  const int64_t plane = (int64_t)M * Kp;  // one (p, comp) plane
  for (int k0 = 4 * (int)threadIdx.x; k0 < Kp; k0 += 1024) {
    int dr[4][OZ_MAX_SLICES], di[4][OZ_MAX_SLICES];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const double2 v = k0 + j < K ? __ldg(row + k0 + j) : cmk(0.0, 0.0);
      value_digits(v.x, Er, dr[j]);
      value_digits(v.y, Er, di[j]);
    }
    __nv_bfloat16* o = Us + (int64_t)r * Kp + k0;
    store_digits4(dr, S, o, 2 * plane);
    store_digits4(di, S, o + plane, 2 * plane);
  }
}

// X (K x N) -> Xs[q][comp][N][Kp] (transposed: each column's K values contiguous).  CTA (x, y):
// 32 columns x 64 K values through shared memory, read along the rows of X, written along K
// (four values per thread, one 8-byte store per plane).
__global__ void __launch_bounds__(256) split_x_kernel(const double2* __restrict__ X, int K, int N, int Kp, int S,
                                                      const int* __restrict__ F, __nv_bfloat16* __restrict__ Xs) {
  __shared__ double2 tile[64][33];
  const int lane = threadIdx.x & 31;
  const int c0 = blockIdx.x * 32, k0 = blockIdx.y * 64;
  for (int rr = threadIdx.x >> 5; rr < 64; rr += 8) {
    const int k = k0 + rr, c = c0 + lane;
    tile[rr][lane] = (k < K && c < N) ? __ldg(X + (int64_t)k * N + c) : cmk(0.0, 0.0);
  }
  __syncthreads();
  const int64_t plane = (int64_t)N * Kp;
  for (int it = threadIdx.x; it < 32 * 16; it += 256) {
    const int cl = it >> 4, kg = it & 15;  // 16 consecutive threads write one column's 64 K values
    const int c = c0 + cl;
    if (c >= N) continue;
    const int Fc = F[c];
    int dr[4][OZ_MAX_SLICES], di[4][OZ_MAX_SLICES];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const double2 v = tile[kg * 4 + j][cl];
      value_digits(v.x, Fc, dr[j]);
      value_digits(v.y, Fc, di[j]);
    }
    __nv_bfloat16* o = Xs + (int64_t)c * Kp + k0 + kg * 4;
    store_digits4(dr, S, o, 2 * plane);
    store_digits4(di, S, o + plane, 2 * plane);
  }
}

// ---------------------------------------------------------------- tcgen05 path
// Warp-specialised Blackwell kernel for the slice products.  Y is cut into tiles of
// 128 rows x 128 complex columns.  The work of a tile is one unit per slice pair (p, q),
// component (re or im of U) and chunk of at most TC_UNIT_K K values; in a unit the tensor
// cores compute one M = 128, N = 256 product into TMEM:
//     comp re: acc = U_re,p [X_re,q | X_im,q]   (columns 0..127: rr, 128..255: ri)
//     comp im: acc = U_im,p [X_re,q | X_im,q]   (columns 0..127: ir, 128..255: ii)
// with FP32 accumulation that is exact for digits of at most 128 in magnitude.  The units
// of all tiles form one sequence (OzSeq: tile by tile; within a tile by slice order
// d = p + q ascending, the pairs of an order alternating direction so that consecutive
// units reuse U slices still in L2; then by component and K chunk), cut into contiguous runs
// of equal numbers of K blocks, one per SM, so every SM works for the same time whatever the
// number of tiles (a 2500 x 256 product has 40).  A CTA adds each finished unit, converted to
// integers, to per-thread integer sums of its current tile and order (re += rr - ii,
// im += ri + ir); when the tile or the order changes it adds them to that order's sums in
// global memory with integer atomics (exact and order-independent: the result does not
// depend on the schedule), and oz_recombine_kernel then forms each element from all orders.
// The slice products are bound by the tensor cores' operand reads from shared memory (each
// MMA reads its A and B tiles; measured on this part: M = N = 128 MMAs without any TMA
// traffic reach ~60 % of the BF16 peak), so the MMAs use the widest N: 96 instead of 128
// bytes read per MMA cycle.  Roles:
//   warp 0, lane 0: TMA producer (4-stage ring of [U_comp | X_re ; X_im] K-blocks of 64),
//   warp 1, lane 0: MMA issuer (tcgen05.mma, tcgen05.commit into mbarriers),
//   warps 2..17:     epilogue, four warps per 32-lane TMEM quadrant (tcgen05.ld reaches only
//                    the quadrant warp % 4), 32 of the 128 columns each.
// Accumulators are double-buffered (TMEM columns 0 and 256) so the epilogue of one
// unit overlaps the MMAs of the next.  Every mbarrier wait is bounded; on a
// timeout the CTA records MM_ERR_WAIT_TIMEOUT, lets its in-flight copies land,
// frees its TMEM and returns.
constexpr int TC_BM = 128;                                // Y rows per tile (MMA M)
constexpr int TC_NC = 128;                                // Y complex columns per tile (MMA N = 256)
constexpr int TC_BK = 64;                                 // K per stage: one 128-byte swizzled row of BF16
constexpr int TC_A_BYTES = TC_BM * TC_BK * 2;             // 16 KB (one U component)
constexpr int TC_B_BYTES = 2 * TC_NC * TC_BK * 2;         // 32 KB ([X_re; X_im] rows)
constexpr int TC_STAGE_BYTES = TC_A_BYTES + TC_B_BYTES;   // 48 KB (a multiple of 1 KB: swizzle atoms stay aligned)
constexpr int TC_STAGES = 4;
// K values per unit: 1024 products of at most 2^14 in magnitude keep every FP32 partial sum an
// integer of at most 2^24 (exact).
constexpr int TC_UNIT_K = 1024;
constexpr int TC_UNIT_KB = TC_UNIT_K / TC_BK;
static_assert(TC_UNIT_K * 128 * 128 <= (1 << 24), "exact FP32 unit sums");
// Slice-order sums [tile][order][comp][col][row]: int32 while S pairs x 2 products x Kp x 2^14
// < 2^31 (Kp <= 9362 at S = 7), int64 beyond.
constexpr int TC_KP_INT32_MAX = 9344;
static_assert((long long)OZ_MAX_SLICES * 2 * TC_KP_INT32_MAX * 128 * 128 < (1ll << 31), "int32 order sums");
constexpr int TC_SMEM_BYTES = 1024 + TC_STAGES * TC_STAGE_BYTES + 256;
constexpr int TC_TMEM_COLS = 512;
constexpr int TC_ACC_STRIDE = 256;                        // TMEM columns between the two accumulator buffers
static_assert(2 * TC_NC <= TC_ACC_STRIDE, "accumulator layout");
static_assert(TC_STAGE_BYTES % 1024 == 0 && (TC_B_BYTES / 2) % 1024 == 0, "swizzle atoms");
constexpr int TC_EPI_WARPS = 16;
constexpr int TC_EPI_COLS = TC_NC / 4;                    // complex columns per epilogue warp
constexpr int TC_THREADS = 64 + 32 * TC_EPI_WARPS;
constexpr int TC_TILE_SUMS = 2 * TC_NC * TC_BM;           // order-sum elements per tile and order
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
__device__ __forceinline__ void tc_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

__device__ __forceinline__ void red_add(int* p, int v) {
  if (v) atomicAdd(p, v);
}
__device__ __forceinline__ void red_add(long long* p, long long v) {
  if (v) atomicAdd(reinterpret_cast<unsigned long long*>(p), (unsigned long long)v);
}

// The unit sequence, shared by every role of every CTA and by the host's sizing.  The CTAs
// form `lanes` lanes (lanes = the number of column tiles, or 1): lane l = b % lanes of CTA b
// works on column tile l of every row tile, so the CTAs of one row of lanes read the same U
// slices at the same time (once from DRAM, then from L2).  A lane's sequence runs over groups
// g (row tiles; tiles when lanes = 1; tile t = g * lanes + l), pairs, components and K chunks:
// unit i has pair index pj = i / (2 nch) (group pj / npairs), component (i / nch) % 2 and
// chunk c = i % nch of the pair's nkb K blocks (all chunks but the last have TC_UNIT_KB
// blocks).  Within a group the pairs run by order d = 2 .. S+1 (d - 1 pairs each), p ascending
// for even d and descending for odd d.  Row r = b / lanes of CTAs takes the units whose first
// K block lies in [r W, (r + 1) W), W = total_kb / nrows: contiguous runs of equal work.
struct OzSeq {
  int S, nkb, nch, npairs, n_ct, lanes, nrows;
  long long nunits, total_kb;  // per lane
  struct Unit {
    long long t;
    int d, p, comp, kb0, kb1;
  };
  __device__ long long prefix(long long i) const {
    const long long sj = i / nch;  // (pair, component) index
    return sj * nkb + (i - sj * nch) * TC_UNIT_KB;
  }
  __device__ int row_of(long long i) const { return (int)(prefix(i) * nrows / total_kb); }
  // smallest unit index i with row_of(i) >= r (nunits for r = nrows)
  __device__ long long first_unit(int r) const {
    long long lo = 0, hi = nunits;
    while (lo < hi) {
      const long long mid = (lo + hi) >> 1;
      if (row_of(mid) >= r) hi = mid;
      else lo = mid + 1;
    }
    return lo;
  }
  __device__ Unit unit(long long i, int lane) const {
    Unit u;
    const long long sj = i / nch;
    const int c = (int)(i - sj * nch);
    const long long pj = sj >> 1;
    u.comp = (int)(sj & 1);
    const long long g = pj / npairs;
    u.t = g * lanes + lane;
    int j = (int)(pj - g * npairs);
    int d = 2;
    while (j >= d - 1) {
      j -= d - 1;
      ++d;
    }
    u.d = d;
    u.p = (d & 1) ? d - 1 - j : 1 + j;
    u.kb0 = c * TC_UNIT_KB;
    u.kb1 = min(nkb, u.kb0 + TC_UNIT_KB);
    return u;
  }
};

// TT: type of the slice-order sums in global memory (int or long long).
template <typename TT>
__global__ void __launch_bounds__(TC_THREADS, 1)
    ozaki_tc_kernel(const __grid_constant__ CUtensorMap tmap_u, const __grid_constant__ CUtensorMap tmap_x,
                    TT* __restrict__ sums, OzSeq seq, int M, int N, mm::WsHeader* h, uint64_t budget_ns) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  unsigned char* smem = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  unsigned char* stages = smem;
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem + TC_STAGES * TC_STAGE_BYTES);
  // bars: full[STAGES], empty[STAGES], accf[2], acce[2], drain
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars + 2 * TC_STAGES + 5);
  volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_slot + 1);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int lane_id = (int)blockIdx.x % seq.lanes, crow = (int)blockIdx.x / seq.lanes;
  const long long i_lo = seq.first_unit(crow), i_hi = seq.first_unit(crow + 1);
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
      mbar_init(acce(b), 32 * TC_EPI_WARPS);
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
    bool ok = true;
    for (long long i = i_lo; ok && i < i_hi; ++i) {
      const OzSeq::Unit u = seq.unit(i, lane_id);
      const int m0 = (int)(u.t / seq.n_ct) * TC_BM, n0 = (int)(u.t % seq.n_ct) * TC_NC;
      const int yu = ((u.p - 1) * 2 + u.comp) * M + m0, yx = (u.d - u.p - 1) * 2 * N + n0;
      for (int kb = u.kb0; kb < u.kb1; ++kb) {
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
        tma_load_2d(smem_u32(st + TC_A_BYTES), &tmap_x, x, yx, full(stage));
        tma_load_2d(smem_u32(st + TC_A_BYTES + TC_B_BYTES / 2), &tmap_x, x, yx + N, full(stage));
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
    bool ok = true;
    for (long long i = i_lo; ok && i < i_hi; ++i) {
      const OzSeq::Unit u = seq.unit(i, lane_id);
      if (!mbar_wait(acce(abuf), aphase ^ 1, abort_flag, h, budget_ns)) break;
      tc_fence_after();
      const uint32_t dacc = tmem + (uint32_t)(abuf * TC_ACC_STRIDE);
      for (int kb = u.kb0; kb < u.kb1; ++kb) {
        if (!mbar_wait(full(stage), phase, abort_flag, h, budget_ns)) {
          ok = false;
          break;
        }
        tc_fence_after();
        const uint32_t st = smem_u32(stages + stage * TC_STAGE_BYTES);
#pragma unroll
        for (int k16 = 0; k16 < TC_BK / 16; ++k16) {
          const uint32_t koff = (uint32_t)k16 * 32;
          const uint32_t acc = (kb > u.kb0 || k16 > 0) ? 1u : 0u;
          tc_mma(dacc, sw128_desc(st + koff), sw128_desc(st + TC_A_BYTES + koff), acc);
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
    const int c0 = TC_EPI_COLS * ((warp - 2) >> 2);  // this warp's first complex column of the tile
    const uint32_t trow = tmem + ((uint32_t)lane_base << 16);  // this warp's 32 TMEM lanes
    TT sre[TC_EPI_COLS], sim[TC_EPI_COLS];
#pragma unroll
    for (int j = 0; j < TC_EPI_COLS; ++j) sre[j] = sim[j] = 0;
    int abuf = 0;
    uint32_t aphase = 0;
    for (long long i = i_lo; i < i_hi; ++i) {
      const OzSeq::Unit u = seq.unit(i, lane_id);
      // one lane waits, the warp follows it, so the warp-wide tcgen05.ld stays convergent
      int okw = lane == 0 ? (int)mbar_wait(accf(abuf), aphase, abort_flag, h, budget_ns) : 0;
      okw = __shfl_sync(0xffffffffu, okw, 0);
      if (!okw) break;
      tc_fence_after();
      const uint32_t base = trow + (uint32_t)(abuf * TC_ACC_STRIDE) + (uint32_t)c0;
      // comp re: columns [rr | ri] -> re += rr, im += ri;  comp im: [ir | ii] -> re -= ii, im += ir
      const bool cre = u.comp == 0;
#pragma unroll
      for (int c8 = 0; c8 < TC_EPI_COLS / 8; ++c8) {
        uint32_t a0[8], a1[8];
        tc_ld8(base + c8 * 8, a0);
        tc_ld8(base + TC_NC + c8 * 8, a1);
        tc_wait_ld();
#pragma unroll
        for (int j = 0; j < 8; ++j) {
          const TT x0 = (TT)__float2int_rn(__uint_as_float(a0[j])), x1 = (TT)__float2int_rn(__uint_as_float(a1[j]));
          sre[c8 * 8 + j] += cre ? x0 : -x1;
          sim[c8 * 8 + j] += cre ? x1 : x0;
        }
      }
      tc_fence_before();
      mbar_arrive(acce(abuf));
      if (++abuf == 2) {
        abuf = 0;
        aphase ^= 1;
      }
      bool flush = i + 1 >= i_hi;
      if (!flush) {
        const OzSeq::Unit v = seq.unit(i + 1, lane_id);
        flush = v.t != u.t || v.d != u.d;
      }
      if (flush) {  // this tile's and order's share of the sums: [tile][d - 2][comp][col][row]
        TT* s = sums + (u.t * seq.S + (u.d - 2)) * (long long)TC_TILE_SUMS + (long long)c0 * TC_BM + row;
#pragma unroll
        for (int j = 0; j < TC_EPI_COLS; ++j) {
          red_add(s + j * TC_BM, sre[j]);
          red_add(s + TC_NC * TC_BM + j * TC_BM, sim[j]);
          sre[j] = sim[j] = 0;
        }
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

// Y[m][n] = sum over orders d = 2 .. S+1 of the order's integer sums scaled by
// 2^(E_m + F_n + 8(2 OZ_MAX_SLICES - d) - 2 OZ_TOP), formed exactly in 128-bit integers and
// rounded once to double (no FP64 arithmetic: 1/64 rate on this part).  CTA:
// 128 rows x 8 columns of one tile; the sums are read along rows (their layout), the results
// staged in shared memory and written along the rows of Y.
constexpr int RC_COLS = 8;
template <typename TT>
__global__ void __launch_bounds__(256) oz_recombine_kernel(const TT* __restrict__ sums, const int* __restrict__ E,
                                                           const int* __restrict__ F, double2* __restrict__ Y, int M,
                                                           int N, int S, int n_ct) {
  __shared__ double2 ys[RC_COLS][TC_BM + 1];
  const long long t = blockIdx.x / (TC_NC / RC_COLS);
  const int cb = (int)(blockIdx.x % (TC_NC / RC_COLS)) * RC_COLS;
  const int m0 = (int)(t / n_ct) * TC_BM, n0 = (int)(t % n_ct) * TC_NC + cb;
  const int rl = threadIdx.x & (TC_BM - 1), cg = threadIdx.x >> 7;  // two column groups of 4
  const int m = m0 + rl;
  const int er = m < M ? E[m] : INT32_MIN;
#pragma unroll
  for (int j = 0; j < RC_COLS / 2; ++j) {
    const int cl = cb + cg * (RC_COLS / 2) + j, n = n0 + cg * (RC_COLS / 2) + j;
    const int fc = n < N ? F[n] : INT32_MIN;
    double2 y = cmk(0.0, 0.0);
    if (er != INT32_MIN && fc != INT32_MIN) {
      // exact sum of all orders as one 128-bit integer in units of the last order's scale
      // (|sum| < 2^50 per order times at most 2^48), then one rounding to double
      const TT* s = sums + t * S * (long long)TC_TILE_SUMS + (long long)cl * TC_BM + rl;
      long long vre[OZ_MAX_SLICES], vim[OZ_MAX_SLICES];
#pragma unroll
      for (int o = 0; o < OZ_MAX_SLICES; ++o) {  // every load issued before the first use
        vre[o] = o < S ? (long long)s[(long long)o * TC_TILE_SUMS] : 0;
        vim[o] = o < S ? (long long)s[(long long)o * TC_TILE_SUMS + TC_NC * TC_BM] : 0;
      }
      unsigned __int128 are = 0, aim = 0;
#pragma unroll
      for (int o = 0; o < OZ_MAX_SLICES; ++o) {  // order d = o + 2
        if (o < S) {
          const int w = OZ_BETA * (S - 1 - o);
          are += (unsigned __int128)(__int128)vre[o] << w;
          aim += (unsigned __int128)(__int128)vim[o] << w;
        }
      }
      const int sh = er + fc + OZ_BETA * (2 * OZ_MAX_SLICES - (S + 1)) - 2 * OZ_TOP;
      y = cmk(mm::i128_scaled_to_double((__int128)are, sh), mm::i128_scaled_to_double((__int128)aim, sh));
    }
    ys[cg * (RC_COLS / 2) + j][rl] = y;
  }
  __syncthreads();
  for (int it = threadIdx.x; it < TC_BM * RC_COLS; it += 256) {
    const int r = it / RC_COLS, c = it % RC_COLS;
    if (m0 + r < M && n0 + c < N) Y[(int64_t)(m0 + r) * N + n0 + c] = ys[c][r];
  }
}

}  // namespace

namespace {
int64_t round_up(int64_t x, int64_t a) { return (x + a - 1) / a * a; }

struct OzLayout {
  int64_t Kp = 0, n_rt = 0, n_ct = 0;
  bool sums64 = false;  // slice-order sums in int64 (Kp beyond the int32 bound)
  size_t us = 0, xs = 0, e = 0, f = 0, sums = 0, sums_bytes = 0, total = 0;
};

// Workspace: 512-byte status header, U slices, X slices, row / column exponents, slice-order sums.
OzLayout oz_layout(int64_t M, int64_t N, int64_t K, int S) {
  OzLayout L;
  L.Kp = round_up(K, OZ_KALIGN);
  L.n_rt = (M + TC_BM - 1) / TC_BM;
  L.n_ct = (N + TC_NC - 1) / TC_NC;
  L.sums64 = L.Kp > TC_KP_INT32_MAX;
  size_t off = sizeof(mm::WsHeader);
  L.us = off;
  off = round_up(off + (size_t)S * 2 * M * L.Kp * sizeof(__nv_bfloat16), 256);
  L.xs = off;
  off = round_up(off + (size_t)S * 2 * N * L.Kp * sizeof(__nv_bfloat16), 256);
  L.e = off;
  off = round_up(off + (size_t)M * sizeof(int), 256);
  L.f = off;
  off = round_up(off + (size_t)N * sizeof(int), 256);
  L.sums = off;
  L.sums_bytes = (size_t)(L.n_rt * L.n_ct) * S * TC_TILE_SUMS * (L.sums64 ? sizeof(long long) : sizeof(int));
  off = round_up(off + L.sums_bytes, 256);
  L.total = off;
  return L;
}

int sm_count() {
  static int cache[64] = {};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) {
    cudaGetLastError();
    return 1;
  }
  if (cache[dev] == 0) {
    int n = 0;
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n < 1) {
      cudaGetLastError();
      n = 1;
    }
    cache[dev] = n;
  }
  return cache[dev];
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
  split_u_kernel<<<(unsigned)M, 256, 0, st>>>((const double2*)U, (int)M, (int)K, Kp, slices, E, (int)N, F, Us);
  col_exp_kernel<<<dim3((unsigned)((N + 31) / 32), (unsigned)((K + COL_EXP_ROWS - 1) / COL_EXP_ROWS)), 256, 0, st>>>(
      (const double2*)X, (int)K, (int)N, F);
  split_x_kernel<<<dim3((unsigned)((N + 31) / 32), (unsigned)(Kp / 64)), 256, 0, st>>>((const double2*)X, (int)K,
                                                                                     (int)N, Kp, slices, F, Xs);
  CUtensorMap tu, tx;
  if (!make_map(&tu, Us, (uint64_t)slices * 2 * M, (uint64_t)Kp, TC_BM) ||
      !make_map(&tx, Xs, (uint64_t)slices * 2 * N, (uint64_t)Kp, TC_NC))
    return MM_ERR_UNSUPPORTED;
  static std::once_flag attr_once;
  std::call_once(attr_once, [] {
    cudaFuncSetAttribute(ozaki_tc_kernel<int>, cudaFuncAttributeMaxDynamicSharedMemorySize, TC_SMEM_BYTES);
    cudaFuncSetAttribute(ozaki_tc_kernel<long long>, cudaFuncAttributeMaxDynamicSharedMemorySize, TC_SMEM_BYTES);
  });
  OzSeq seq;
  seq.S = slices;
  seq.nkb = (int)(Kp / TC_BK);
  seq.nch = (seq.nkb + TC_UNIT_KB - 1) / TC_UNIT_KB;
  seq.npairs = slices * (slices + 1) / 2;
  seq.n_ct = (int)L.n_ct;
  const long long ntiles = L.n_rt * L.n_ct;
  // one lane per column tile when the SMs divide into rows of lanes with little left over
  const int sms = sm_count();
  seq.lanes = (L.n_ct <= sms && (sms % L.n_ct) * 16 <= sms) ? (int)L.n_ct : 1;
  const long long groups = ntiles / seq.lanes;
  seq.nunits = groups * seq.npairs * 2 * seq.nch;
  seq.total_kb = groups * seq.npairs * 2 * seq.nkb;
  seq.nrows = (int)std::min<long long>(sms / seq.lanes, seq.nunits);
  const int ncta = seq.nrows * seq.lanes;
  mm::WsHeader* h = reinterpret_cast<mm::WsHeader*>(w);
  if (cudaMemsetAsync(w + L.sums, 0, L.sums_bytes, st) != cudaSuccess) return MM_ERR_CUDA;
  const unsigned rgrid = (unsigned)(ntiles * (TC_NC / RC_COLS));
  if (L.sums64) {
    long long* sums = reinterpret_cast<long long*>(w + L.sums);
    ozaki_tc_kernel<long long><<<ncta, TC_THREADS, TC_SMEM_BYTES, st>>>(tu, tx, sums, seq, (int)M, (int)N, h,
                                                                           tc_budget_ns());
    oz_recombine_kernel<long long><<<rgrid, 256, 0, st>>>(sums, E, F, (double2*)Y, (int)M, (int)N, slices,
                                                          (int)L.n_ct);
  } else {
    int* sums = reinterpret_cast<int*>(w + L.sums);
    ozaki_tc_kernel<int><<<ncta, TC_THREADS, TC_SMEM_BYTES, st>>>(tu, tx, sums, seq, (int)M, (int)N, h,
                                                                     tc_budget_ns());
    oz_recombine_kernel<int><<<rgrid, 256, 0, st>>>(sums, E, F, (double2*)Y, (int)M, (int)N, slices, (int)L.n_ct);
  }
  mm::note_launches(5);  // row exponents and U slices, column exponents, X slices, products, recombination
  return cudaGetLastError() == cudaSuccess ? MM_OK : MM_ERR_CUDA;
}

}  // extern "C"
