// Shared device-side definitions of the GB300 Hermite library.
//
// Data layout in HBM (all complex128 = double2, row-major / C order exactly as
// the reference's flat index, mrmustard/math/lattice/strategies/vanilla/core.py:63-73):
//   G[f], f = sum_i k_i * strides[i], strides[D-1] = 1.
// Ragged batches pack instances back to back (G, dLdG by element offset; A by D*D
// offset; b by D offset; c one per instance).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "mm_gb300.h"

#define MM_MAXD 8          // modes supported per instance (exact templates 1..8)
#define MM_NV_MAX (1 + MM_MAXD + MM_MAXD * (MM_MAXD + 1) / 2)  // VJP accumulators per instance
#define MM_BLOCK 256       // threads per CTA for the recurrence kernels

// Shared-memory declarations of the kernels.  Under nvcc this is plain
// __shared__; the host emulation of the kernels (MM_HOST_EMULATION) supplies
// per-CTA storage instead, so several emulated CTAs can run at once.
#if defined(MM_HOST_EMULATION) && !defined(__CUDA_ARCH__)
template <class T>
T& mm_emu_shared(int key);
#define MM_SHARED(T, name) T& name = mm_emu_shared<T>(__LINE__)
#else
#define MM_SHARED(T, name) __shared__ T name
#endif

namespace mm {

// Adds n to the library's launch counter (mm_launch_count); defined in capi.cu.
void note_launches(int64_t n);

// ---------------------------------------------------------------- complex helpers
__device__ __forceinline__ double2 cmk(double r, double i) { return make_double2(r, i); }
// a * b
__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
  return cmk(fma(a.x, b.x, -a.y * b.y), fma(a.x, b.y, a.y * b.x));
}
// acc + a * b  (four DFMA)
__device__ __forceinline__ double2 cfma(double2 a, double2 b, double2 acc) {
  acc.x = fma(a.x, b.x, acc.x);
  acc.x = fma(-a.y, b.y, acc.x);
  acc.y = fma(a.x, b.y, acc.y);
  acc.y = fma(a.y, b.x, acc.y);
  return acc;
}
// acc + s * a for real s (two DFMA)
__device__ __forceinline__ double2 crfma(double s, double2 a, double2 acc) {
  return cmk(fma(s, a.x, acc.x), fma(s, a.y, acc.y));
}
__device__ __forceinline__ double2 cscale(double s, double2 a) { return cmk(s * a.x, s * a.y); }
__device__ __forceinline__ double2 cadd(double2 a, double2 b) { return cmk(a.x + b.x, a.y + b.y); }

// Complex division with Smith's method, as numpy divides complex128 scalars.
__device__ __forceinline__ double2 cdiv_smith(double2 a, double2 b) {
  if (fabs(b.x) >= fabs(b.y)) {
    double rat = b.y / b.x, scl = 1.0 / (b.x + b.y * rat);
    return cmk((a.x + a.y * rat) * scl, (a.y - a.x * rat) * scl);
  }
  double rat = b.x / b.y, scl = 1.0 / (b.y + b.x * rat);
  return cmk((a.x * rat + a.y) * scl, (a.y * rat - a.x) * scl);
}

// a / b correctly rounded, for b > 0 with y = RN(1/b), by Markstein's theorem
// (P. Markstein, "Computation of elementary functions on the IBM RISC System/6000
// processor", IBM J. Res. Dev. 34(1), 1990): q0 = RN(a y) is within one ulp of
// a/b, so the remainder r = a - q0 b is exact in one FMA, and RN(q0 + r y) is
// RN(a/b).  Three FP64 operations instead of a division sequence.  The theorem
// assumes no underflow or overflow on the way: when q0 is zero, below 2^-959,
// above 2^977 or not finite, the quotient comes from the division itself.
__device__ __forceinline__ double div_by_recip(double a, double b, double y) {
  const double q0 = __dmul_rn(a, y);
  const uint32_t e = (uint32_t)(__double_as_longlong(q0) >> 52) & 0x7ffu;
  if (e < 64u || e > 2000u) return __ddiv_rn(a, b);
  const double r = __fma_rn(-q0, b, a);
  return __fma_rn(r, y, q0);
}

// L2-only load (bypasses L1) for data written by other CTAs of the same launch.
__device__ __forceinline__ double2 ld_cg(const double2* p) { return __ldcg(p); }

// ---------------------------------------------------------------- instance geometry
struct Geom {
  int32_t D;
  int32_t maxC;          // max_i shape[i]
  int64_t n;             // prod(shape)
  int64_t shape[MM_MAXD];
  int64_t strides[MM_MAXD];
  int64_t sumC;          // sum_i shape[i]
  int32_t prefC[MM_MAXD];  // prefix sums of shape (coefficient-table segment offsets)
};

// Per-instance record of a ragged batch (lives in the workspace, uploaded by the plan).
struct InstDesc {
  Geom g;
  int64_t g_off;     // element offset into G / dLdG
  int64_t a_off;     // element offset into A (D*D)
  int64_t b_off;     // element offset into b (D)
  int64_t coef_off;  // double2 offset of this instance's coefficient block
  int64_t item_begin;  // first VJP work item of this instance
  int64_t n_items;     // number of VJP work items
  int64_t fibers_per_item;
};

// Coefficient block of one instance (double2 entries), built on the device per call:
//   cd[i][m]   = A_ii * sqrt(m - 1)          m in [1, C_i)     at  coef + cd_off(i)
//   W[i][j][k] = A_ij * sqrt(k)   (j != i)   k in [0, C_j)     at  coef + w_off(i, j)
// Both tables use the layout index(i, j) = i * sumC + prefC[j]  (with j == i
// holding cd), so the block has D * sumC entries.
__host__ __device__ inline int64_t coef_entries(const Geom& g) { return (int64_t)g.D * g.sumC; }

// Index of the VJP accumulator for dA_ij (i <= j): slot 0 is dc, 1..D are db_i,
// then the upper triangle of dA row by row.
__host__ __device__ constexpr int vjp_nv(int D) { return 1 + D + D * (D + 1) / 2; }
__host__ __device__ constexpr int vjp_slot(int D, int i, int j) { return 1 + D + i * D - i * (i - 1) / 2 + (j - i); }

// Global scalar tables (double), built per call for k in [0, kmax):
//   sq[k] = sqrt(k)  (correctly rounded, as the reference's SQRT table)
//   rs[k] = 1 / sqrt(k)  (rs[0] = 0)
//   hh[k] = 0.5 * sqrt(k) * sqrt(k - 1)  (hh[0] = hh[1] = 0)
struct Tables {
  const double* sq;
  const double* rs;
  const double* hh;
  int64_t kmax;
};

// ---------------------------------------------------------------- status / waits
// Bytes [0, 128) hold the sticky status word; bytes [128, 512) are per-launch
// state that every entry point zeroes (cudaMemsetAsync) before its kernels run.
struct WsHeader {
  int32_t status;       // sticky error word (0 = ok), written with atomicCAS
  int32_t pad0[31];
  uint32_t barrier;     // grid-barrier arrival counter
  uint32_t queue;       // work-queue head
  uint32_t pad1[30];
  uint32_t heartbeat;   // bumped by CTAs that work while others wait (progress signal)
  uint32_t pad2[31];
  int32_t abort;        // set when any CTA of the launch gave up a wait
  int32_t pad3[31];
};
static_assert(sizeof(WsHeader) == 512, "header layout");
#define MM_WS_LAUNCH_STATE_OFFSET 128
#define MM_WS_LAUNCH_STATE_BYTES 384

__device__ __forceinline__ void set_status(WsHeader* h, int code) {
  atomicCAS(&h->status, 0, code);
  atomicExch(&h->abort, 1);
}

#if defined(__CUDA_ARCH__)
__device__ __forceinline__ uint64_t globaltimer_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ uint32_t ld_acquire_u32(const uint32_t* p) {
  uint32_t v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ int32_t ld_relaxed_i32(const int32_t* p) {
  int32_t v;
  asm volatile("ld.relaxed.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ uint32_t ld_relaxed_u32(const uint32_t* p) {
  uint32_t v;
  asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_release_u32(uint32_t* p, uint32_t v) {
  asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ unsigned long long ld_relaxed_u64(const void* p) {
  unsigned long long v;
  asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}
// Both 8-byte halves of a polled amplitude in one access.  No "memory" clobber: the amplitude's own
// bits say whether it has been written, so no other access is ordered by it, and the compiler may
// issue several of these before the first result is needed.
__device__ __forceinline__ void ld_relaxed_v2u64(const void* p, unsigned long long& x, unsigned long long& y) {
  asm volatile("ld.relaxed.gpu.global.v2.u64 {%0, %1}, [%2];" : "=l"(x), "=l"(y) : "l"(p));
}
#else  // host compilation of the device code (CPU emulation of the kernels' indexing)
__device__ __forceinline__ uint64_t globaltimer_ns() { return 0; }
__device__ __forceinline__ uint32_t ld_acquire_u32(const uint32_t* p) { return __atomic_load_n(p, __ATOMIC_ACQUIRE); }
__device__ __forceinline__ int32_t ld_relaxed_i32(const int32_t* p) { return __atomic_load_n(p, __ATOMIC_RELAXED); }
__device__ __forceinline__ uint32_t ld_relaxed_u32(const uint32_t* p) { return __atomic_load_n(p, __ATOMIC_RELAXED); }
__device__ __forceinline__ void st_release_u32(uint32_t* p, uint32_t v) { __atomic_store_n(p, v, __ATOMIC_RELEASE); }
__device__ __forceinline__ unsigned long long ld_relaxed_u64(const void* p) {
  return __atomic_load_n(reinterpret_cast<const unsigned long long*>(p), __ATOMIC_RELAXED);
}
__device__ __forceinline__ void ld_relaxed_v2u64(const void* p, unsigned long long& x, unsigned long long& y) {
  const unsigned long long* q = reinterpret_cast<const unsigned long long*>(p);
  x = __atomic_load_n(q, __ATOMIC_RELAXED);
  y = __atomic_load_n(q + 1, __ATOMIC_RELAXED);
}
#endif

// An amplitude that its producer has not written yet, in a region filled with this bit pattern
// (all ones: a NaN that FP64 arithmetic never produces -- its NaN results are the canonical one).
// A consumer that polls the amplitude itself needs no progress word and no release fence: every
// aligned 8-byte store becomes visible whole.
constexpr unsigned long long kPendingBits = 0xffffffffffffffffull;

// Progress signal for waits: a CTA that works alone while the others wait at a
// barrier bumps the heartbeat, which restarts their timeout.
__device__ __forceinline__ void heartbeat(WsHeader* h) { atomicAdd(&h->heartbeat, 1u); }

// Grid-wide barrier for a cooperative launch.  Arrivals count up monotonically;
// barrier number `epoch` (1, 2, ...) completes when the counter reaches
// epoch * gridDim.x.  Every wait is bounded: if neither the arrival counter nor
// the heartbeat moves for `budget_ns` (or another CTA has already given up) the
// CTA records MM_ERR_WAIT_TIMEOUT and the function returns false, so the kernel
// returns instead of hanging the GPU.
__device__ __forceinline__ bool grid_barrier(WsHeader* h, uint32_t epoch, uint64_t budget_ns, uint32_t extra) {
  MM_SHARED(int, s_ok);
  __syncthreads();
  if (threadIdx.x == 0) {
    int ok = 1;
    __threadfence();
    atomicAdd(&h->barrier, 1u);
    const uint32_t target = epoch * gridDim.x + extra;
    uint64_t t0 = globaltimer_ns();
    uint32_t last_arr = 0, last_hb = ld_relaxed_u32(&h->heartbeat);
    uint32_t arr;
    while ((arr = ld_acquire_u32(&h->barrier)) < target) {
      if (ld_relaxed_i32(&h->abort) != 0) { ok = 0; break; }
      const uint32_t hb = ld_relaxed_u32(&h->heartbeat);
      const uint64_t now = globaltimer_ns();
      if (arr != last_arr || hb != last_hb) {
        last_arr = arr;
        last_hb = hb;
        t0 = now;
      } else if (now - t0 > budget_ns) {
        set_status(h, MM_ERR_WAIT_TIMEOUT);
        ok = 0;
        break;
      }
      __nanosleep(64);
    }
    __threadfence();
    s_ok = ok;
  }
  __syncthreads();
  return s_ok != 0;
}

// ---------------------------------------------------------------- debug checks
// Built with -DMM_DEVICE_CHECKS (MM_DEVICE_CHECKS=1 in the environment of the
// build), every global access of the recurrence kernels first checks its
// address for alignment and for lying inside the buffer it belongs to; the
// first violation is recorded in mm_dbg_word (tag, address, base, elements,
// alignment) and the access is skipped.  Without the define the checks vanish.
#ifdef MM_DEVICE_CHECKS
static __device__ unsigned long long mm_dbg_word[8];
__device__ __forceinline__ bool dbg_ok(const void* p, const void* base, long long n_elems, int esize, int align,
                                       int tag) {
  const unsigned long long a = (unsigned long long)p, b0 = (unsigned long long)base;
  const bool ok = (a % (unsigned long long)align) == 0 && a >= b0 &&
                  a + (unsigned long long)esize <= b0 + (unsigned long long)n_elems * (unsigned long long)esize;
  if (!ok && atomicAdd(&mm_dbg_word[0], 1ull) == 0ull) {
    mm_dbg_word[1] = (unsigned long long)tag;
    mm_dbg_word[2] = a;
    mm_dbg_word[3] = b0;
    mm_dbg_word[4] = (unsigned long long)n_elems;
    mm_dbg_word[5] = (unsigned long long)align;
  }
  return ok;
}
#define MM_CHK(p, base, n, T, tag) (::mm::dbg_ok((const void*)(p), (const void*)(base), (long long)(n), (int)sizeof(T), (int)alignof(T), (tag)))
#else
#define MM_CHK(p, base, n, T, tag) (true)
#endif

// Row-major multi-index decomposition helpers (32-bit: chunk sizes are < 2^31).
template <int D>
__device__ __forceinline__ void decompose(uint32_t q, int first, const Geom& g, int32_t (&k)[D]) {
  // k[j] for j >= first from the inner flat index q over axes first..D-1.
#pragma unroll
  for (int j = D - 1; j >= 0; --j) {
    if (j >= first) {
      uint32_t c = (uint32_t)g.shape[j];
      k[j] = (int32_t)(q % c);
      q /= c;
    } else {
      k[j] = 0;
    }
  }
}

}  // namespace mm
