// Device code of the Hermite recurrence, its stable variant and its VJP.
//
// Schedules
// ---------
// vanilla (reference: mrmustard/math/lattice/strategies/vanilla/core.py:25-124).
//   The reference walks the flat C-order index f and takes as pivot axis i the
//   first non-zero coordinate of k (core.py:88-94; i = 0 in the bulk,
//   core.py:108-122).  Group the flat indices by that axis: "level" i holds
//   every k with k_0..k_{i-1} = 0 and k_i >= 1, i.e. f in [strides[i],
//   strides[i-1]); inside a level, "chunk" m = k_i is the contiguous run
//   [m*strides[i], (m+1)*strides[i]).  Every amplitude of chunk (i, m) reads
//   only chunks (i, m-1) and (i, m-2) (pivot f - s_i, neighbours f - s_i - s_j),
//   so a chunk is fully parallel and levels run D-1, ..., 0, chunks m = 1, 2, ...
//   This reproduces the reference's pivot choice and operation order
//   (b_i G_p + A_ii sqrt(m-1) G_{p-1_i} + sum_{j>i} A_ij sqrt(k_j) G_{p-1_j})
//   exactly; the final division by sqrt(m) becomes a multiply by 1/sqrt(m)
//   and products are fused (DFMA), so results agree to rounding.
//   Writes are contiguous (one chunk = one slab of the row-major tensor).
//   One large instance on the whole GPU (fwd_flow_kernel) drops the per-chunk
//   grid barrier: ranges of a chunk wait only for the amplitudes they read
//   (polled in a G pre-filled with a pending bit pattern, or progress words),
//   the smallest levels run in one CTA's shared memory, and
//   latency-bound chains split each amplitude's real and imaginary parts over
//   a lane pair (same terms, products rounded per part).
// stable (core.py:127-213).  Every valid pivot is averaged, so an amplitude also
//   reads amplitudes of its own chunk; the schedule is the |k| anti-diagonal
//   wavefront (all reads sit on wavefronts |k|-1 and |k|-2).
// VJP (gradients.py:25-82).  A reduction: no ordering constraint.  One thread
//   owns a "fiber" (fixed k_1..k_{D-1}) and walks k_0, so the weights
//   sqrt(k_i) sqrt(k_j) of every term not involving axis 0 are constant along
//   the fiber and are applied once per fiber; the axis-0 weights are folded
//   into the cotangent once per amplitude.
#pragma once

#include <algorithm>
#include <cstring>

#include "common.cuh"

namespace mm {

struct InstView {
  Geom g;
  const double2* A;
  const double2* b;
  double2 c;
  double2* G;
  const double2* dLdG;
  const double2* coef;
  double2* Gh;  // optional second destination of the forward's G (e.g. pinned host memory), or null
};

// Field-by-field geometry copy.  Views are never built by whole-struct
// assignment: with nvcc 13.0 for sm_103a, building a view in a local struct
// (geometry memcpy'd from the kernel-parameter struct, pointers stored after
// it) and then assigning the whole struct to shared memory was compiled into a
// byte copy of the parameter struct itself, so the view's pointer fields
// received the parameter struct's unrelated fields.  Writing every field
// straight into its destination avoids that transformation; mm_selftest checks
// the result on the device before any kernel dereferences a view.
__device__ __forceinline__ void copy_geom(Geom& d, const Geom& s) {
  d.D = s.D;
  d.maxC = s.maxC;
  d.n = s.n;
  d.sumC = s.sumC;
#pragma unroll
  for (int j = 0; j < MM_MAXD; ++j) {
    d.shape[j] = s.shape[j];
    d.strides[j] = s.strides[j];
    d.prefC[j] = s.prefC[j];
  }
}

struct VjpItem {
  int32_t inst;
  uint32_t q0;
  uint32_t q1;
  int32_t pad;
};

// One shape, B instances (the unbatched call is B = 1).
struct UniformSrc {
  Geom g;
  int64_t B;
  const double2* A;
  const double2* b;
  const double2* c;
  double2* G;
  const double2* dLdG;
  double2* coef;
  int64_t coef_stride;
  int64_t items_per_inst;
  uint32_t fibers_per_item;
  __device__ __forceinline__ int64_t n_inst() const { return B; }
  __device__ __forceinline__ int64_t sched(int64_t t) const { return t; }
  __device__ __forceinline__ void load(int64_t k, InstView& v) const {
    copy_geom(v.g, g);
    v.A = A + k * g.D * g.D;
    v.b = b + k * g.D;
    v.c = c[k];
    v.G = G + k * g.n;
    v.dLdG = dLdG ? dLdG + k * g.n : nullptr;
    v.coef = coef + k * coef_stride;
    v.Gh = nullptr;
  }
  __device__ __forceinline__ const Geom& geom(int64_t) const { return g; }
  __device__ __forceinline__ double2* coef_of(int64_t k) const { return coef + k * coef_stride; }
  __device__ __forceinline__ double2* gout_of(int64_t) const { return nullptr; }
  __device__ __forceinline__ void item(int64_t it, int64_t& k, uint32_t& q0, uint32_t& q1) const {
    k = it / items_per_inst;
    const int64_t r = it - k * items_per_inst;
    q0 = (uint32_t)(r * fibers_per_item);
    const int64_t e = (r + 1) * (int64_t)fibers_per_item;
    q1 = (uint32_t)(e < g.strides[0] ? e : g.strides[0]);
  }
  __device__ __forceinline__ void items_of(int64_t k, int64_t& begin, int64_t& count) const {
    begin = k * items_per_inst;
    count = items_per_inst;
  }
  __device__ __forceinline__ int64_t a_off(int64_t k) const { return k * g.D * g.D; }
  __device__ __forceinline__ int64_t b_off(int64_t k) const { return k * g.D; }
};

// B instances with their own D and shape; descriptors live in the workspace.
struct RaggedSrc {
  const InstDesc* desc;
  const int32_t* order;  // instances in schedule order (largest first)
  int64_t B;
  const double2* A;
  const double2* b;
  const double2* c;
  double2* G;
  const double2* dLdG;
  double2* coef;
  const VjpItem* items;
  double2* Gout;  // optional copy of G (may be pinned host memory), or null
  // instances k with (k & 7) < fwd_copy_eighths get their copy of G from the
  // forward (InstView::Gh), the others from the VJP (gout_of)
  int32_t fwd_copy_eighths;
  __device__ __forceinline__ int64_t n_inst() const { return B; }
  __device__ __forceinline__ int64_t sched(int64_t t) const { return order[t]; }
  __device__ __forceinline__ bool fwd_copies(int64_t k) const { return (int32_t)(k & 7) < fwd_copy_eighths; }
  __device__ __forceinline__ double2* gout_of(int64_t k) const {
    return (Gout && !fwd_copies(k)) ? Gout + desc[k].g_off : nullptr;
  }
  __device__ __forceinline__ void load(int64_t k, InstView& v) const {
    const InstDesc& d = desc[k];
    copy_geom(v.g, d.g);
    v.A = A + d.a_off;
    v.b = b + d.b_off;
    v.c = c[k];
    v.G = G + d.g_off;
    v.dLdG = dLdG ? dLdG + d.g_off : nullptr;
    v.coef = coef + d.coef_off;
    v.Gh = (Gout && fwd_copies(k)) ? Gout + d.g_off : nullptr;
  }
  __device__ __forceinline__ const Geom& geom(int64_t k) const { return desc[k].g; }
  __device__ __forceinline__ double2* coef_of(int64_t k) const { return coef + desc[k].coef_off; }
  __device__ __forceinline__ void item(int64_t it, int64_t& k, uint32_t& q0, uint32_t& q1) const {
    const VjpItem x = items[it];
    k = x.inst;
    q0 = x.q0;
    q1 = x.q1;
  }
  __device__ __forceinline__ void items_of(int64_t k, int64_t& begin, int64_t& count) const {
    begin = desc[k].item_begin;
    count = desc[k].n_items;
  }
  __device__ __forceinline__ int64_t a_off(int64_t k) const { return desc[k].a_off; }
  __device__ __forceinline__ int64_t b_off(int64_t k) const { return desc[k].b_off; }
};

template <bool CG>
__device__ __forceinline__ double2 ldG(const double2* p) {
  if constexpr (CG) return __ldcg(p);
  else return *p;
}

// Checked forms of the recurrence's accesses (plain accesses unless MM_DEVICE_CHECKS).
template <bool CG>
__device__ __forceinline__ double2 ldGc(const InstView& v, const double2* p, int tag) {
  if (!MM_CHK(p, v.G, v.g.n, double2, tag)) return cmk(0.0, 0.0);
  return ldG<CG>(p);
}
__device__ __forceinline__ double2 ldCoef(const InstView& v, const double2* p, int tag) {
  if (!MM_CHK(p, v.coef, coef_entries(v.g), double2, tag)) return cmk(0.0, 0.0);
  return *p;
}
__device__ __forceinline__ void stG(const InstView& v, int64_t f, double2 x, int tag) {
  if (MM_CHK(v.G + f, v.G, v.g.n, double2, tag)) {
    v.G[f] = x;
    if (v.Gh) v.Gh[f] = x;
  }
}

// ============================================================== setup kernel
// Scalar tables (grid-strided) and each instance's coefficient block (one CTA
// per instance, grid-strided over instances).
template <class Src>
__global__ void __launch_bounds__(256) setup_kernel(Src src, double* sq, double* rs, double* hh, int64_t kmax,
                                                    int do_coef) {
  const int64_t gtid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t gstride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t k = gtid; k < kmax; k += gstride) {
    if (!MM_CHK(hh + k, sq, 3 * kmax, double, 11)) continue;
    const double s = sqrt((double)k);
    sq[k] = s;
    rs[k] = k > 0 ? 1.0 / s : 0.0;
    hh[k] = k > 1 ? (0.5 * s) * sqrt((double)(k - 1)) : 0.0;
  }
  if (!do_coef) return;
  for (int64_t k = blockIdx.x; k < src.n_inst(); k += gridDim.x) {
    const Geom& g = src.geom(k);
    InstView v;
    src.load(k, v);
    double2* coef = src.coef_of(k);
    const int64_t total = coef_entries(g);
    for (int64_t e = threadIdx.x; e < total; e += blockDim.x) {
      const int i = (int)(e / g.sumC);
      const int32_t r = (int32_t)(e - (int64_t)i * g.sumC);
      int j = 0;
      while (j + 1 < g.D && g.prefC[j + 1] <= r) ++j;
      const int32_t kk = r - g.prefC[j];
      const double2 a = MM_CHK(v.A + i * g.D + j, v.A, g.D * g.D, double2, 9) ? v.A[i * g.D + j] : cmk(0.0, 0.0);
      double2 val;
      if (j == i) {  // cd[i][m] = A_ii * sqrt(m - 1) (zero at m = 0, 1)
        const double s = kk >= 1 ? sqrt((double)(kk - 1)) : 0.0;
        val = cmk(a.x * s, a.y * s);
      } else {  // W[i][j][k] = A_ij * sqrt(k)
        const double s = sqrt((double)kk);
        val = cmk(a.x * s, a.y * s);
      }
      if (MM_CHK(coef + e, coef, total, double2, 10)) coef[e] = val;
    }
  }
}

// ============================================================== vanilla forward
// Chunk (level i, index m), amplitudes q in [q_begin, q_end) stepping by q_step
// from thread rank t.
template <int D, bool CG>
__device__ __forceinline__ void fwd_chunk(const InstView& v, const double* __restrict__ rs, int i, int m,
                                          uint32_t q_begin, uint32_t q_end, uint32_t q_step, uint32_t t) {
  const Geom& g = v.g;
  const int64_t si = g.strides[i];
  const double2 bi = MM_CHK(v.b + i, v.b, g.D, double2, 1) ? __ldg(v.b + i) : cmk(0.0, 0.0);
  const double2* __restrict__ crow = v.coef + (int64_t)i * g.sumC;
  const double2 cd = (m >= 2) ? ldCoef(v, crow + g.prefC[i] + m, 2) : cmk(0.0, 0.0);
  const double rsm = MM_CHK(rs + m, rs, g.maxC + 1, double, 3) ? rs[m] : 0.0;
  const double2* G = v.G;
  const int64_t base = (int64_t)m * si;
  int64_t sj[D];
  int32_t pj[D];
#pragma unroll
  for (int j = 0; j < D; ++j) {
    sj[j] = g.strides[j];
    pj[j] = g.prefC[j];
  }
  for (uint32_t q = q_begin + t; q < q_end; q += q_step) {
    int32_t k[D];
    decompose<D>(q, i + 1, g, k);
    const int64_t f = base + q;
    const int64_t p = f - si;
    double2 acc = cmul(bi, ldGc<CG>(v, G + p, 4));
    if (m >= 2) acc = cfma(cd, ldGc<CG>(v, G + p - si, 4), acc);
#pragma unroll
    for (int j = 1; j < D; ++j) {
      if (j > i && k[j] > 0) acc = cfma(ldCoef(v, crow + pj[j] + k[j], 5), ldGc<CG>(v, G + p - sj[j], 4), acc);
    }
    stG(v, f, cscale(rsm, acc), 6);
  }
}

// Chunk (i, m) with the pivot row of the coefficient block and b_i already
// multiplied by 1/sqrt(m) (`row`, built by build_scaled_row): the amplitude is
// the sum of the terms itself, without the final scaling of fwd_chunk (two FP64
// instructions fewer per amplitude; each term is rounded once more instead of
// the sum).  Rows of at most kScaledRow entries (sumC) fit the shared buffers.
constexpr int kScaledRow = 320;
struct ScaledRow {
  double2 c[kScaledRow];
  double2 b;
};

// The two row buffers of a CTA (one static shared array for every caller).
__device__ __forceinline__ ScaledRow* scaled_rows() {
  __shared__ ScaledRow rows[2];
  return rows;
}

__device__ __forceinline__ void build_scaled_row(const InstView& v, const double* __restrict__ rs, int i, int m,
                                                 ScaledRow& row) {
  const double r = MM_CHK(rs + m, rs, v.g.maxC + 1, double, 3) ? rs[m] : 0.0;
  const double2* __restrict__ crow = v.coef + (int64_t)i * v.g.sumC;
  for (int e = (int)threadIdx.x; e < (int)v.g.sumC; e += (int)blockDim.x) row.c[e] = cscale(r, ldCoef(v, crow + e, 5));
  if (threadIdx.x == blockDim.x - 1)
    row.b = cscale(r, MM_CHK(v.b + i, v.b, v.g.D, double2, 1) ? __ldg(v.b + i) : cmk(0.0, 0.0));
}

template <int D, bool CG>
__device__ __forceinline__ void fwd_chunk_scaled(const InstView& v, const ScaledRow& row, int i, int m,
                                                 uint32_t q_begin, uint32_t q_end, uint32_t q_step, uint32_t t) {
  const Geom& g = v.g;
  const int64_t si = g.strides[i];
  const double2 bi = row.b;
  const double2 cd = (m >= 2) ? row.c[g.prefC[i] + m] : cmk(0.0, 0.0);
  const double2* G = v.G;
  const int64_t base = (int64_t)m * si;
  int64_t sj[D];
  int32_t pj[D], shp[D];
#pragma unroll
  for (int j = 0; j < D; ++j) {
    sj[j] = g.strides[j];
    pj[j] = g.prefC[j];
    shp[j] = (int32_t)g.shape[j];
  }
  // k of the thread's first amplitude, then advanced by the digits of q_step (mixed-radix addition over
  // axes i+1..D-1; q < strides[i] for every amplitude used, so the carry out of axis i+1 is dropped)
  int32_t k[D], dk[D];
  {
    uint32_t q0 = q_begin + t < q_end ? q_begin + t : q_begin, st = q_step;
#pragma unroll
    for (int j = D - 1; j >= 0; --j) {
      k[j] = dk[j] = 0;
      if (j > i) {
        const uint32_t c = (uint32_t)shp[j];
        k[j] = (int32_t)(q0 % c);
        q0 /= c;
        dk[j] = (int32_t)(st % c);
        st /= c;
      }
    }
  }
  for (uint32_t q = q_begin + t; q < q_end; q += q_step) {
    const int64_t f = base + q;
    const int64_t p = f - si;
    double2 acc = cmul(bi, ldGc<CG>(v, G + p, 4));
    if (m >= 2) acc = cfma(cd, ldGc<CG>(v, G + p - si, 4), acc);
#pragma unroll
    for (int j = 1; j < D; ++j) {
      if (j > i && k[j] > 0) acc = cfma(row.c[pj[j] + k[j]], ldGc<CG>(v, G + p - sj[j], 4), acc);
    }
    stG(v, f, acc, 6);
    int32_t carry = 0;
#pragma unroll
    for (int j = D - 1; j >= 0; --j) {
      if (j > i) {
        k[j] += dk[j] + carry;
        carry = k[j] >= shp[j] ? 1 : 0;
        if (carry) k[j] -= shp[j];
      }
    }
  }
}

// The chunk after (i, m) in the forward's order (levels D-1 .. 0, m = 1 .. C_i - 1); i < 0 at the end.
__device__ __forceinline__ void next_chunk(const Geom& g, int& i, int& m) {
  ++m;
  while (i >= 0 && m >= (int)g.shape[i]) {
    --i;
    m = 1;
  }
}

// Whole instance on one CTA (chunks separated by __syncthreads).  With a short
// enough pivot row, the next chunk's scaled row is built while the CTA
// finishes the current chunk (double buffer), so it costs no extra barrier.
template <int D>
__device__ void fwd_instance_cta(const InstView& v, const double* rs) {
  if (v.g.sumC <= kScaledRow) {
    ScaledRow* rows = scaled_rows();
    if (threadIdx.x == 0) stG(v, 0, v.c, 7);
    int i = D - 1, m = 0;
    next_chunk(v.g, i, m);
    if (i >= 0) build_scaled_row(v, rs, i, m, rows[0]);
    __syncthreads();
    for (int buf = 0; i >= 0; buf ^= 1) {
      int ni = i, nm = m;
      next_chunk(v.g, ni, nm);
      fwd_chunk_scaled<D, false>(v, rows[buf], i, m, 0u, (uint32_t)v.g.strides[i], blockDim.x, threadIdx.x);
      if (ni >= 0) build_scaled_row(v, rs, ni, nm, rows[buf ^ 1]);
      __syncthreads();
      i = ni;
      m = nm;
    }
    return;
  }
  if (threadIdx.x == 0) stG(v, 0, v.c, 7);
  __syncthreads();
  for (int i = D - 1; i >= 0; --i) {
    const int Ci = (int)v.g.shape[i];
    const uint32_t si = (uint32_t)v.g.strides[i];
    for (int m = 1; m < Ci; ++m) {
      fwd_chunk<D, false>(v, rs, i, m, 0u, si, blockDim.x, threadIdx.x);
      __syncthreads();
    }
  }
}

// ============================================================== stable forward
static __constant__ double c_inv_n[MM_MAXD + 1] = {0.0,       1.0,       1.0 / 2.0, 1.0 / 3.0, 1.0 / 4.0,
                                            1.0 / 5.0, 1.0 / 6.0, 1.0 / 7.0, 1.0 / 8.0};

// One amplitude k (flat index f) of the stable recurrence: the average over the
// pivots i with k_i > 0 of (b_i G[k-1_i] + sum_j A_ij sqrt(k_j) G[k-1_i-1_j]
// (k_j > 0, j != i) + A_ii sqrt(k_i - 1) G[k-2_i]) / sqrt(k_i) (core.py:182-211).
template <int D, bool CG>
__device__ __forceinline__ void stable_point(const InstView& v, const double* __restrict__ rs, const int32_t (&k)[D],
                                             int64_t f, const int64_t (&sj)[D], const int32_t (&pj)[D]) {
  const Geom& g = v.g;
  double2* G = v.G;
  double2 vals = cmk(0.0, 0.0);
  int npiv = 0;
#pragma unroll
  for (int i = 0; i < D; ++i) {
    if (k[i] > 0) {
      ++npiv;
      const double2* __restrict__ crow = v.coef + (int64_t)i * g.sumC;
      const int64_t pv = f - sj[i];
      double2 acc = cmul(__ldg(v.b + i), ldG<CG>(G + pv));
#pragma unroll
      for (int j = 0; j < i; ++j)
        if (k[j] > 0) acc = cfma(crow[pj[j] + k[j]], ldG<CG>(G + pv - sj[j]), acc);
      if (k[i] >= 2) acc = cfma(crow[pj[i] + k[i]], ldG<CG>(G + pv - sj[i]), acc);
#pragma unroll
      for (int j = i + 1; j < D; ++j)
        if (k[j] > 0) acc = cfma(crow[pj[j] + k[j]], ldG<CG>(G + pv - sj[j]), acc);
      vals = crfma(rs[k[i]], acc, vals);
    }
  }
  stG(v, f, cscale(c_inv_n[npiv], vals), 6);
}

// Wavefront |k| = w; prefixes p over axes 0..D-2 in [p_begin, p_end) by p_step.
template <int D, bool CG>
__device__ __forceinline__ void stable_wave(const InstView& v, const double* __restrict__ rs, int w, uint32_t p_begin,
                                            uint32_t p_end, uint32_t p_step, uint32_t t) {
  const Geom& g = v.g;
  const int32_t CL = (int32_t)g.shape[D - 1];
  int64_t sj[D];
  int32_t pj[D];
#pragma unroll
  for (int j = 0; j < D; ++j) {
    sj[j] = g.strides[j];
    pj[j] = g.prefC[j];
  }
  for (uint32_t p = p_begin + t; p < p_end; p += p_step) {
    int32_t k[D];
    int32_t sum = 0;
    uint32_t q = p;
#pragma unroll
    for (int j = D - 2; j >= 0; --j) {
      const uint32_t c = (uint32_t)g.shape[j];
      k[j] = (int32_t)(q % c);
      q /= c;
      sum += k[j];
    }
    const int32_t kl = w - sum;
    if (kl < 0 || kl >= CL) continue;
    k[D - 1] = kl;
    stable_point<D, CG>(v, rs, k, (int64_t)p * CL + kl, sj, pj);
  }
}

template <int D>
__device__ void stable_instance_cta(const InstView& v, const double* rs) {
  if (threadIdx.x == 0) stG(v, 0, v.c, 7);
  __syncthreads();
  int wmax = 0;
  for (int i = 0; i < D; ++i) wmax += (int)v.g.shape[i] - 1;
  const uint32_t P = (uint32_t)(v.g.n / v.g.shape[D - 1]);
  for (int w = 1; w <= wmax; ++w) {
    stable_wave<D, false>(v, rs, w, 0u, P, blockDim.x, threadIdx.x);
    __syncthreads();
  }
}

// One CTA per instance, instances taken in schedule order (largest first).
template <int DLO, int DHI, class Src>
__global__ void __launch_bounds__(MM_BLOCK) fwd_cta_kernel(Src src, const double* __restrict__ rs, int stable) {
  MM_SHARED(InstView, sv);
  const int64_t k = src.sched(blockIdx.x);
  if (threadIdx.x == 0) src.load(k, sv);
  __syncthreads();
  const int D = sv.g.D;
#define MM_FWD_CASE(DD)                                        \
  if constexpr (DLO <= DD && DD <= DHI) {                      \
    if (D == DD) {                                             \
      if (stable) stable_instance_cta<DD>(sv, rs);             \
      else fwd_instance_cta<DD>(sv, rs);                       \
      return;                                                  \
    }                                                          \
  }
  MM_FWD_CASE(1)
  MM_FWD_CASE(2)
  MM_FWD_CASE(3)
  MM_FWD_CASE(4)
  MM_FWD_CASE(5)
  MM_FWD_CASE(6)
  MM_FWD_CASE(7)
  MM_FWD_CASE(8)
#undef MM_FWD_CASE
}

// ------------------------------------------------ ragged batch with cluster teams
// Thread-block cluster helpers (sm_90+ PTX special registers and barrier).
#if defined(__CUDA_ARCH__)
__device__ __forceinline__ uint32_t cluster_rank() {
  uint32_t r;
  asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
  return r;
}
__device__ __forceinline__ uint32_t cluster_size() {
  uint32_t r;
  asm volatile("mov.u32 %0, %%cluster_nctarank;" : "=r"(r));
  return r;
}
__device__ __forceinline__ uint32_t cluster_index() {
  uint32_t r;
  asm volatile("mov.u32 %0, %%clusterid.x;" : "=r"(r));
  return r;
}
__device__ __forceinline__ uint32_t cluster_count() {
  uint32_t r;
  asm volatile("mov.u32 %0, %%nclusterid.x;" : "=r"(r));
  return r;
}
// All threads of all CTAs of the cluster; release/acquire orders the chunk's
// global writes before the next chunk's reads (which go through L2: ldG<true>).
__device__ __forceinline__ void cluster_sync() {
  asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}
#else  // host compilation of the device code (CPU emulation): provided by the emulator
uint32_t cluster_rank();
uint32_t cluster_size();
uint32_t cluster_index();
uint32_t cluster_count();
void cluster_sync();
#endif

// One instance on a whole cluster: every chunk is split over the cluster's
// CTAs in contiguous ranges, with a cluster barrier after it.  Control flow is
// identical in every CTA of the cluster, so every barrier is reached by all.
template <int D>
__device__ void fwd_instance_team(const InstView& v, const double* rs, uint32_t rank, uint32_t nranks) {
  if (v.g.sumC <= kScaledRow) {
    // as fwd_instance_cta: every CTA builds its own copy of the next chunk's scaled row
    ScaledRow* rows = scaled_rows();
    if (rank == 0 && threadIdx.x == 0) stG(v, 0, v.c, 7);
    int i = D - 1, m = 0;
    next_chunk(v.g, i, m);
    if (i >= 0) build_scaled_row(v, rs, i, m, rows[0]);
    cluster_sync();
    for (int buf = 0; i >= 0; buf ^= 1) {
      int ni = i, nm = m;
      next_chunk(v.g, ni, nm);
      const uint32_t si = (uint32_t)v.g.strides[i];
      const uint32_t per = (si + nranks - 1) / nranks;
      const uint32_t lo = min(si, per * rank), hi = min(si, lo + per);
      fwd_chunk_scaled<D, true>(v, rows[buf], i, m, lo, hi, blockDim.x, threadIdx.x);
      if (ni >= 0) build_scaled_row(v, rs, ni, nm, rows[buf ^ 1]);
      cluster_sync();
      i = ni;
      m = nm;
    }
    return;
  }
  if (rank == 0 && threadIdx.x == 0) stG(v, 0, v.c, 7);
  cluster_sync();
  for (int i = D - 1; i >= 0; --i) {
    const uint32_t si = (uint32_t)v.g.strides[i];
    const uint32_t per = (si + nranks - 1) / nranks;
    const uint32_t lo = min(si, per * rank), hi = min(si, lo + per);
    for (int m = 1; m < (int)v.g.shape[i]; ++m) {
      fwd_chunk<D, true>(v, rs, i, m, lo, hi, blockDim.x, threadIdx.x);
      cluster_sync();
    }
  }
}

template <int D>
__device__ void stable_instance_team(const InstView& v, const double* rs, uint32_t rank, uint32_t nranks) {
  if (rank == 0 && threadIdx.x == 0) stG(v, 0, v.c, 7);
  cluster_sync();
  int wmax = 0;
  for (int i = 0; i < D; ++i) wmax += (int)v.g.shape[i] - 1;
  const uint32_t P = (uint32_t)(v.g.n / v.g.shape[D - 1]);
  const uint32_t per = (P + nranks - 1) / nranks;
  const uint32_t lo = min(P, per * rank), hi = min(P, lo + per);
  for (int w = 1; w <= wmax; ++w) {
    stable_wave<D, true>(v, rs, w, lo, hi, blockDim.x, threadIdx.x);
    cluster_sync();
  }
}

// Persistent launch with cluster dimensions (CL, 1, 1).  Phase 1: cluster c
// takes the large instances big[c], big[c + nclusters], ... (largest first) and
// runs each on all its CTAs.  Phase 2: every CTA pulls the remaining instances
// (largest first) one at a time from an atomic queue and runs each alone.
// No CTA ever waits for another cluster, so the launch needs no co-residency
// guarantee beyond the cluster's own.  Four CTAs per SM up to D = 4 (64
// registers; unbounded, the chunk loop's incremental multi-index takes 76 and
// three CTAs per SM were measured slower), two above.
template <int DLO, int DHI>
__global__ void __launch_bounds__(MM_BLOCK, DHI <= 4 ? 4 : 2)
    fwd_ragged_team_kernel(RaggedSrc src, const double* __restrict__ rs, int stable, const int32_t* __restrict__ big,
                           int n_big, const int32_t* __restrict__ small, int n_small, WsHeader* h) {
  MM_SHARED(InstView, sv);
  MM_SHARED(int, s_next);
  const uint32_t rank = cluster_rank(), nranks = cluster_size();
  const uint32_t cid = cluster_index(), ncl = cluster_count();
  for (int bi = (int)cid; bi < n_big; bi += (int)ncl) {
    if (threadIdx.x == 0) src.load(big[bi], sv);
    __syncthreads();
    const int D = sv.g.D;
#define MM_TEAM_CASE(DD)                                          \
  if constexpr (DLO <= DD && DD <= DHI) {                         \
    if (D == DD) {                                                \
      if (stable) stable_instance_team<DD>(sv, rs, rank, nranks); \
      else fwd_instance_team<DD>(sv, rs, rank, nranks);           \
    }                                                             \
  }
    MM_TEAM_CASE(1)
    MM_TEAM_CASE(2)
    MM_TEAM_CASE(3)
    MM_TEAM_CASE(4)
    MM_TEAM_CASE(5)
    MM_TEAM_CASE(6)
    MM_TEAM_CASE(7)
    MM_TEAM_CASE(8)
#undef MM_TEAM_CASE
    __syncthreads();
  }
  for (;;) {
    if (threadIdx.x == 0) s_next = (int)atomicAdd(&h->queue, 1u);
    __syncthreads();
    const int idx = s_next;
    if (idx >= n_small) break;
    if (threadIdx.x == 0) src.load(small[idx], sv);
    __syncthreads();
    const int D = sv.g.D;
#define MM_SOLO_CASE(DD)                                \
  if constexpr (DLO <= DD && DD <= DHI) {               \
    if (D == DD) {                                      \
      if (stable) stable_instance_cta<DD>(sv, rs);      \
      else fwd_instance_cta<DD>(sv, rs);                \
    }                                                   \
  }
    MM_SOLO_CASE(1)
    MM_SOLO_CASE(2)
    MM_SOLO_CASE(3)
    MM_SOLO_CASE(4)
    MM_SOLO_CASE(5)
    MM_SOLO_CASE(6)
    MM_SOLO_CASE(7)
    MM_SOLO_CASE(8)
#undef MM_SOLO_CASE
    __syncthreads();
  }
}

// ------------------------------------------------ single large instance, whole grid
// Stable recurrence of one large instance: every anti-diagonal |k| = w is split
// over all CTAs (cooperative launch) with a bounded grid barrier after it.
template <int D>
__global__ void __launch_bounds__(512) stable_grid_kernel(UniformSrc src, const double* __restrict__ rs, WsHeader* h,
                                                          uint64_t budget_ns) {
  MM_SHARED(InstView, sv);
  if (threadIdx.x == 0) src.load(0, sv);
  __syncthreads();
  const Geom& g = sv.g;
  uint32_t epoch = 0;
  if (blockIdx.x == 0 && threadIdx.x == 0) sv.G[0] = sv.c;
  if (!grid_barrier(h, ++epoch, budget_ns, 0)) return;
  int wmax = 0;
  for (int i = 0; i < D; ++i) wmax += (int)g.shape[i] - 1;
  const uint32_t P = (uint32_t)(g.n / g.shape[D - 1]);
  const uint32_t per = (P + gridDim.x - 1) / gridDim.x;
  const uint32_t lo = min(P, per * blockIdx.x), hi = min(P, lo + per);
  for (int w = 1; w <= wmax; ++w) {
    stable_wave<D, true>(sv, rs, w, lo, hi, blockDim.x, threadIdx.x);
    if (!grid_barrier(h, ++epoch, budget_ns, 0)) return;
  }
}

// ------------------------------------------------ dataflow forward of one large instance
// Level i's chunk m (the slab k_0..k_{i-1} = 0, k_i = m) is split into ctas[i]
// contiguous ranges of per[i] amplitudes; range v is computed by one CTA, which
// then publishes prog[flag0[i] + v] = m.  Amplitude q of chunk m reads chunk
// m-1 at q and at q - strides[j] (j > i), and chunk m-2 at q, so before chunk
// m >= 2 a CTA waits only for the ranges of chunk m-1 that overlap
// [lo - strides[i+1], hi); before chunk 1 it waits until the lower levels hold
// every amplitude below its `hi`.  There is no grid-wide barrier per chunk.
//
// Levels >= small_lvl (positions [0, small_amps)) are latency-bound chains of
// tiny chunks: one CTA computes them in shared memory, writes them out and
// publishes them at once.  Levels 1 .. small_lvl-1 run on `face` CTAs, one per
// SM; level 0 runs on the rest.  Roles come from the SM each CTA landed on
// (%smid, registered once with one grid barrier): with `exclusive`, the other
// CTAs on a face CTA's SM stay idle so the face's latency-bound chain owns its
// SM's FP64 pipes, the face CTAs take the last level-0 ranges (they finish the
// face last) and run them one per SM, consecutive level-0 ranges go to
// different SMs, and the two CTAs of a shared SM hold one early and one late
// range (serpentine_range).
struct FlowPlan {
  uint32_t ctas[MM_MAXD];
  uint32_t per[MM_MAXD];
  uint32_t flag0[MM_MAXD];
  uint32_t face;        // CTAs holding the ranges of levels 1 .. small_lvl-1 (at least 1)
  uint32_t sms;         // SMs of the device
  uint32_t per_sm;      // CTAs per SM of the launch (gridDim.x = per_sm * sms)
  uint32_t exclusive;   // see above
  uint32_t small_lvl;   // levels >= small_lvl live in shared memory (D: none)
  uint32_t small_amps;  // strides[small_lvl - 1]: amplitudes of that region
  uint32_t poll_halo;   // G pre-filled with kPendingBits (but G[0]): every input of another CTA is polled
  uint64_t budget_ns;
};

constexpr uint32_t kFlowSmemAmps = 2560;  // shared-memory region of the small levels (40 KiB)
constexpr uint32_t kFlowMaxSmid = 1024;   // SM-id registration words after the progress words
constexpr uint32_t kFlowNone = 0xffffffffu;

// Host planning.  min_amps: fewest amplitudes of a range (>= 2).  Returns the
// number of progress words (word 0 = the shared-memory region or G[0]).
inline int64_t flow_plan(const Geom& g, int sms, int per_sm, uint32_t min_amps, int exclusive, uint64_t budget,
                         FlowPlan& fp) {
  memset(&fp, 0, sizeof(fp));
  fp.sms = (uint32_t)sms;
  fp.per_sm = (uint32_t)per_sm;
  fp.budget_ns = budget;
  const int D = g.D;
  int L = D;
  while (L > 1 && (uint64_t)g.strides[L - 2] <= kFlowSmemAmps) --L;
  fp.small_lvl = (uint32_t)L;
  fp.small_amps = (L < D) ? (uint32_t)g.strides[L - 1] : 0u;
  auto split = [&](uint32_t s, uint32_t cap, uint32_t& P, uint32_t& per) {
    P = std::max(1u, std::min(cap, (s + min_amps - 1) / min_amps));
    per = (s + P - 1) / P;
    P = (s + per - 1) / per;
  };
  uint32_t flag = 1, F = 1;
  for (int i = D - 1; i >= 1; --i) {
    if (i >= L) {
      fp.ctas[i] = 1;
      fp.per[i] = (uint32_t)g.strides[i];
    } else {
      split((uint32_t)g.strides[i], (uint32_t)sms, fp.ctas[i], fp.per[i]);
    }
    fp.flag0[i] = flag;
    flag += fp.ctas[i];
    F = std::max(F, fp.ctas[i]);
  }
  fp.face = F;
  fp.exclusive = (exclusive && F <= (uint32_t)sms / 2) ? 1u : 0u;
  const uint32_t total = (uint32_t)(per_sm * sms);
  const uint32_t avail = fp.exclusive ? (uint32_t)per_sm * ((uint32_t)sms - F) + F : total;
  split((uint32_t)g.strides[0], avail, fp.ctas[0], fp.per[0]);
  fp.flag0[0] = flag;
  flag += fp.ctas[0];
  return flag;
}

#if defined(__CUDA_ARCH__)
__device__ __forceinline__ uint32_t sm_id() {
  uint32_t r;
  asm volatile("mov.u32 %0, %%smid;" : "=r"(r));
  return r;
}
__device__ __forceinline__ uint32_t sm_id_count() {
  uint32_t r;
  asm volatile("mov.u32 %0, %%nsmid;" : "=r"(r));
  return r;
}
#else  // provided by the emulator
uint32_t sm_id();
uint32_t sm_id_count();
#endif

struct FlowSmem {
  double2 g[kFlowSmemAmps];
};
// flow_level's double buffer (2 chunks of at most 2 amplitudes per thread, 256 threads) reuses it
static_assert(2 * 2 * 256 <= kFlowSmemAmps, "flow_level buffer");

struct FlowRole {
  uint32_t smid, slot, below, present, odd;
  uint32_t face_v;  // range of levels 1 .. small_lvl-1 (kFlowNone: none)
  uint32_t v0;      // level-0 range (kFlowNone: none)
};

// Role of this CTA.  Every CTA registers its SM (reg[smid] counts the CTAs of
// that SM; the slot is the CTA's arrival order on it), one grid barrier, then
// each CTA ranks its SM among the SMs present.  If the launch did not land as
// per_sm CTAs on each of `sms` SMs (or an SM id is out of range), every CTA
// falls back to the same blockIdx-based mapping.  The n = S - F shared SMs take
// the level-0 ranges in serpentine order (serpentine_range): slot 0 of the x-th
// such SM takes range x and slot 1 range 2n - 1 - x, so a range that starts
// late shares its SM with one that started early (and finishes early) rather
// than with one that starts mid-way and runs as long as it does.
__device__ __forceinline__ uint32_t serpentine_range(uint32_t slot, uint32_t x, uint32_t n) {
  return (slot & 1u) ? (slot + 1u) * n - 1u - x : slot * n + x;
}
__device__ bool flow_roles(const FlowPlan& fp, WsHeader* h, uint32_t* reg, FlowRole& r) {
  const uint32_t b = blockIdx.x;
  const uint32_t nsm = sm_id_count();
  if (threadIdx.x == 0) {
    r.smid = sm_id();
    r.slot = (nsm <= kFlowMaxSmid && r.smid < kFlowMaxSmid) ? atomicAdd(reg + r.smid, 1u) : kFlowNone;
    r.below = r.present = r.odd = 0;
  }
  if (!grid_barrier(h, 1, fp.budget_ns, 0)) return false;
  if (nsm <= kFlowMaxSmid) {
    uint32_t below = 0, present = 0, odd = 0;
    for (uint32_t s = threadIdx.x; s < nsm; s += blockDim.x) {
      const uint32_t c = ld_relaxed_u32(reg + s);
      if (c) {
        ++present;
        below += (s < r.smid);
        odd += (c != fp.per_sm);
      }
    }
    if (present) atomicAdd(&r.present, present);
    if (below) atomicAdd(&r.below, below);
    if (odd) atomicAdd(&r.odd, odd);
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    const uint32_t F = fp.face, S = fp.sms, total = fp.per_sm * S;
    uint32_t fv = kFlowNone, v0 = kFlowNone;
    if (!fp.exclusive) {  // face CTAs b < F take the last ranges
      fv = b < F ? b : kFlowNone;
      v0 = b >= F ? b - F : total - F + b;
    } else if (nsm > kFlowMaxSmid || r.odd != 0 || r.present != S) {  // blockIdx-based: b and b + S share an SM
      const uint32_t sm = b % S, slot = b / S;
      if (sm < F) {
        if (slot == 0) {
          fv = sm;
          v0 = fp.per_sm * (S - F) + sm;
        }
      } else {
        v0 = serpentine_range(slot, sm - F, S - F);
      }
    } else if (r.below < F) {
      if (r.slot == 0) {
        fv = r.below;
        v0 = fp.per_sm * (S - F) + r.below;
      }
    } else {
      v0 = serpentine_range(r.slot, r.below - F, S - F);
    }
    r.face_v = fv;
    r.v0 = v0 < fp.ctas[0] ? v0 : kFlowNone;
  }
  __syncthreads();
  return true;
}

// Bounded wait until prog[w] >= target for all w in [w_lo, w_hi) except
// `skip`, the CTA's threads polling the words in parallel.  A word that does
// not move for budget_ns records MM_ERR_WAIT_TIMEOUT; any CTA that gives up
// sets the abort word, which ends every other wait.  Returns false on give-up.
__device__ __forceinline__ bool flow_wait(WsHeader* h, const uint32_t* prog, uint32_t w_lo, uint32_t w_hi,
                                          uint32_t skip, uint32_t target, uint64_t budget_ns, int* s_fail) {
  bool fail = false;
  for (uint32_t w = w_lo + threadIdx.x; w < w_hi && !fail; w += blockDim.x) {
    if (w == skip) continue;
    uint32_t v = ld_acquire_u32(prog + w);
    if (v >= target) continue;
    uint64_t t0 = globaltimer_ns();
    uint32_t last = v;
    while (v < target) {
      if (ld_relaxed_i32(&h->abort) != 0) {
        fail = true;
        break;
      }
      const uint64_t now = globaltimer_ns();
      if (v != last) {
        last = v;
        t0 = now;
      } else if (now - t0 > budget_ns) {
        set_status(h, MM_ERR_WAIT_TIMEOUT);
        fail = true;
        break;
      }
      v = ld_acquire_u32(prog + w);
    }
  }
  if (fail) *s_fail = 1;
  __syncthreads();
  return *s_fail == 0;
}

// Lane pairs: lane 2a computes the real part and lane 2a+1 the imaginary part
// of amplitude a, as one chain of FMAs per part.  A GB300 FP64 warp
// instruction costs the same for 1 or 32 active lanes, so this halves the FP64
// instructions on the latency-bound chains.  The terms are those of fwd_chunk
// (b_i G_p, A_ii sqrt(m-1) G_pp, A_ij sqrt(k_j) G_{p-1_j}, then the 1/sqrt(m)
// scale); only the rounding of the complex products differs.
__device__ __forceinline__ double flip_sign_if(double x, bool neg) {
  return __longlong_as_double(__double_as_longlong(x) ^ (neg ? (long long)0x8000000000000000ull : 0ll));
}
// acc + (re or im part of x*y): re = x.x y.x - x.y y.y, im = x.x y.y + x.y y.x
__device__ __forceinline__ double part_fma(double2 x, double2 y, bool im, double acc) {
  return fma(x.x, im ? y.y : y.x, fma(flip_sign_if(x.y, !im), im ? y.x : y.y, acc));
}

// One halo amplitude of the previous chunk whose bits (x, y) were loaded from p, polled again until
// its producer has written both parts (see kPendingBits); bounded: after budget_ns, or when another
// CTA has given up, records the failure (MM_ERR_WAIT_TIMEOUT on a timeout) and returns what it read.
__device__ __forceinline__ double2 halo_wait(const double2* p, unsigned long long x, unsigned long long y, WsHeader* h,
                                             uint64_t budget_ns, int* s_fail) {
  if (x == kPendingBits || y == kPendingBits) {
    const uint64_t t0 = globaltimer_ns();
    while (x == kPendingBits || y == kPendingBits) {
      if (ld_relaxed_i32(&h->abort) != 0) {
        *s_fail = 1;
        break;
      }
      if (globaltimer_ns() - t0 > budget_ns) {
        set_status(h, MM_ERR_WAIT_TIMEOUT);
        *s_fail = 1;
        break;
      }
      ld_relaxed_v2u64(p, x, y);
    }
  }
  return cmk(__longlong_as_double((long long)x), __longlong_as_double((long long)y));
}

// A value as stored where other CTAs poll it: never the pending pattern (a NaN that arithmetic on a
// NaN input carrying those bits might propagate becomes a plain quiet NaN).
__device__ __forceinline__ double not_pending(double x) {
  return (unsigned long long)__double_as_longlong(x) == kPendingBits ? __longlong_as_double(0x7ff8000000000000ll) : x;
}

// Barrier over the first n threads of the CTA (n a multiple of 32), id != 0.
#if defined(__CUDA_ARCH__)
__device__ __forceinline__ void bar_sync_n(uint32_t id, uint32_t n) {
  asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(n) : "memory");
}
#else  // provided by the emulator
void bar_sync_n(uint32_t id, uint32_t n);
#endif

// Small level i of the shared-memory region, all its chunks, on the first
// `lanes` threads (lane pairs, see part_fma), synchronised by a named
// barrier over those threads only.  With one amplitude per lane pair its
// indices and coefficients are loaded once; the per-chunk coefficients
// (A_ii sqrt(m), 1/sqrt(m)) are fetched one chunk ahead.  `crow` is level i's
// row of the coefficient block and `coff` the column it starts at (entry
// prefC[j] + k is crow[prefC[j] + k - coff]), so a caller may stage only the
// columns j >= 1 of a row in shared memory; `bi` is b_i.
template <int D>
__device__ void small_level(const InstView& v, const double* __restrict__ rs, int i, double2* Gs, uint32_t lanes,
                            const double2* crow, int32_t coff, double2 bi) {
  const Geom& g = v.g;
  const uint32_t si = (uint32_t)g.strides[i];
  const int Ci = (int)g.shape[i];
  const bool im = (threadIdx.x & 1u) != 0;
  const uint32_t pairs = lanes >> 1, a0 = threadIdx.x >> 1;
  const int32_t pci = g.prefC[i] - coff;
  double* Gd = reinterpret_cast<double*>(Gs);
  const bool one = si <= pairs;
  uint32_t str[D];  // strides in registers: the barrier at each chunk's end would force them to be re-read
#pragma unroll
  for (int j = 0; j < D; ++j) str[j] = (uint32_t)g.strides[j];
  int32_t k1[D];
  double2 w1[D];
  decompose<D>(a0 < si ? a0 : 0u, i + 1, g, k1);
#pragma unroll
  for (int j = 0; j < D; ++j)
    w1[j] = (one && j > i && k1[j] > 0) ? crow[g.prefC[j] - coff + k1[j]] : cmk(0.0, 0.0);
  double rs_c = rs[1];
  double2 cd_c = cmk(0.0, 0.0);
  for (int m = 1; m < Ci; ++m) {
    const double rsm = rs_c;
    const double2 cd = cd_c;
    if (m + 1 < Ci) {
      rs_c = rs[m + 1];
      cd_c = crow[pci + m + 1];
    }
    const uint32_t base = (uint32_t)m * si;
    if (one) {
      if (a0 < si) {
        const uint32_t f = base + a0, p = f - si;
        double acc = part_fma(bi, Gs[p], im, 0.0);
        if (m >= 2) acc = part_fma(cd, Gs[p - si], im, acc);
#pragma unroll
        for (int j = 1; j < D; ++j)
          if (j > i && k1[j] > 0) acc = part_fma(w1[j], Gs[p - str[j]], im, acc);
        Gd[2 * f + (im ? 1 : 0)] = rsm * acc;
      }
    } else {
      for (uint32_t a = a0; a < si; a += pairs) {
        int32_t k[D];
        decompose<D>(a, i + 1, g, k);
        const uint32_t f = base + a, p = f - si;
        double acc = part_fma(bi, Gs[p], im, 0.0);
        if (m >= 2) acc = part_fma(cd, Gs[p - si], im, acc);
#pragma unroll
        for (int j = 1; j < D; ++j)
          if (j > i && k[j] > 0)
            acc = part_fma(crow[g.prefC[j] - coff + k[j]], Gs[p - str[j]], im, acc);
        Gd[2 * f + (im ? 1 : 0)] = rsm * acc;
      }
    }
    bar_sync_n(1, lanes);
  }
}

// One CTA's range [lo, hi) of a shared level i (ctas[i] > 1) through chunks
// 1..C_i-1, on lane pairs (see part_fma): pair a of the CTA holds
// amplitudes lo + a + u*(blockDim/2) (u < A), lane 2a their real parts and
// lane 2a+1 their imaginary parts.  Each lane keeps its part of the last two
// chunks in registers (gp: m-1, gpp: m-2; the partner's part comes by
// shuffle), and chunk m-1 of the whole range sits in shared memory S
// (double-buffered) for the in-range neighbours q - strides[j].  The terms
// whose inputs lie in the range are summed before the wait for the
// neighbouring ranges; only the halo terms (inputs in another CTA's range) are
// read from global memory after it.
template <int D, int A>
__device__ bool flow_level(const InstView& v, const double* __restrict__ rs, WsHeader* h, uint32_t* prog,
                           const FlowPlan& fp, int i, uint32_t vr, uint32_t fv, double2* S, int* s_fail) {
  const Geom& g = v.g;
  const uint32_t si = (uint32_t)g.strides[i], per = fp.per[i];
  const uint32_t lo = min(si, per * vr), hi = min(si, lo + per);
  const uint32_t snext = (i + 1 < D) ? (uint32_t)g.strides[i + 1] : 0u;
  const int Ci = (int)g.shape[i];
  const bool im = (threadIdx.x & 1u) != 0;
  const uint32_t pairs = blockDim.x >> 1, a0 = threadIdx.x >> 1;
  const double2 bi = __ldg(v.b + i);
  const double2* __restrict__ crow = v.coef + (int64_t)i * g.sumC;
  double2* G = v.G;
  double* Gd = reinterpret_cast<double*>(G);
  double* Sd = reinterpret_cast<double*>(S);
  uint32_t* my = prog + fp.flag0[i] + vr;
  double gp[A], gpp[A];
  int32_t k[A][D];
#pragma unroll
  for (int u = 0; u < A; ++u) {
    const uint32_t q = lo + a0 + (uint32_t)u * pairs;
    decompose<D>(q < hi ? q : lo, i + 1, g, k[u]);
    gp[u] = gpp[u] = 0.0;
  }
  if (Ci < 2) return true;
  // FlowPlan::poll_halo: no progress words; every amplitude another CTA writes is polled in G (G[0],
  // which holds c, is read from c: it may carry the pending bits)
  const bool poll = fp.poll_halo != 0;
  {  // chunk 1: every input is an amplitude of the lower levels
    if (!poll) {
      const uint32_t pos = hi - 1;
      int l = i + 1;
      while (l < D && pos / (uint32_t)g.strides[l] == 0) ++l;
      uint32_t w_lo = 0, w_hi = (fv == 0) ? 0u : 1u, target = 1u, skip = kFlowNone;
      if (l < D) {
        target = pos / (uint32_t)g.strides[l];
        w_lo = fp.flag0[l];
        w_hi = w_lo + fp.ctas[l];
        if (fv < fp.ctas[l]) skip = w_lo + fv;
      }
      if (w_lo < w_hi && !flow_wait(h, prog, w_lo, w_hi, skip, target, fp.budget_ns, s_fail)) return false;
    }
    const double rs1 = rs[1];
    double acc1[A];
    if (poll) {
      // terms (u, j) in batches as in the later chunks; j = 0 is the amplitude q of the level below
      constexpr int T = A * D, NB = T < 6 ? T : 6;
#pragma unroll
      for (int t0 = 0; t0 < T; t0 += NB) {
        unsigned long long hx[NB], hy[NB];
#pragma unroll
        for (int t = 0; t < NB; ++t) {
          hx[t] = hy[t] = 0ull;
          const int u = (t0 + t) / D, j = (t0 + t) % D;
          if (t0 + t >= T) continue;
          const uint32_t q = lo + a0 + (uint32_t)u * pairs;
          const uint32_t idx = j == 0 ? q : q - (uint32_t)g.strides[j];
          if (q < hi && (j == 0 || (j > i && k[u][j] > 0)) && idx != 0) ld_relaxed_v2u64(G + idx, hx[t], hy[t]);
        }
#pragma unroll
        for (int t = 0; t < NB; ++t) {
          const int u = (t0 + t) / D, j = (t0 + t) % D;
          if (t0 + t >= T) continue;
          const uint32_t q = lo + a0 + (uint32_t)u * pairs;
          const uint32_t idx = j == 0 ? q : q - (uint32_t)g.strides[j];
          if (q >= hi || (j != 0 && !(j > i && k[u][j] > 0))) continue;
          const double2 x = idx == 0 ? v.c : halo_wait(G + idx, hx[t], hy[t], h, fp.budget_ns, s_fail);
          if (j == 0) {
            acc1[u] = part_fma(bi, x, im, 0.0);
            gpp[u] = im ? x.y : x.x;
          } else {
            acc1[u] = part_fma(crow[g.prefC[j] + k[u][j]], x, im, acc1[u]);
          }
        }
      }
    } else {
#pragma unroll
      for (int u = 0; u < A; ++u) {
        const uint32_t q = lo + a0 + (uint32_t)u * pairs;
        if (q < hi) {
          const double2 g0 = __ldcg(G + q);
          acc1[u] = part_fma(bi, g0, im, 0.0);
#pragma unroll
          for (int j = 1; j < D; ++j)
            if (j > i && k[u][j] > 0)
              acc1[u] = part_fma(crow[g.prefC[j] + k[u][j]], __ldcg(G + (q - (uint32_t)g.strides[j])), im, acc1[u]);
          gpp[u] = im ? g0.y : g0.x;
        }
      }
    }
#pragma unroll
    for (int u = 0; u < A; ++u) {
      const uint32_t q = lo + a0 + (uint32_t)u * pairs;
      if (q < hi) {
        const double val = not_pending(rs1 * acc1[u]);
        Gd[2 * ((int64_t)si + q) + im] = val;
        Sd[2 * (per + (q - lo)) + im] = val;
        gp[u] = val;
      }
    }
    __syncthreads();
    if (poll) {
      if (*s_fail) return false;
    } else if (threadIdx.x == 0) {
      st_release_u32(my, 1u);
    }
  }
  const uint32_t w_lo = fp.flag0[i] + (lo >= snext ? lo - snext : 0u) / per, w_hi = fp.flag0[i] + vr;
  // Loop-invariant operands of the chunk loop held in registers instead of being re-read from shared
  // memory and L1 every chunk: the axis strides and, with at most two amplitudes per lane pair, the
  // coefficients A_ij sqrt(k_j) (D <= 4, where the registers are free without spills; the indices
  // are in range of the level's coefficient row for every j, so the unused ones are loaded too).
  constexpr bool kRegStrides = D <= 4, kRegCoefs = D <= 4 && A <= 2;
  uint32_t str_r[kRegStrides ? D : 1];
  double2 cf_r[kRegCoefs ? A : 1][kRegCoefs ? D : 1];
  if constexpr (kRegStrides) {
#pragma unroll
    for (int j = 0; j < D; ++j) str_r[j] = (uint32_t)g.strides[j];
  }
  if constexpr (kRegCoefs) {
#pragma unroll
    for (int u = 0; u < A; ++u)
#pragma unroll
      for (int j = 0; j < D; ++j) cf_r[u][j] = (j > i && k[u][j] > 0) ? crow[g.prefC[j] + k[u][j]] : cmk(0.0, 0.0);
  }
  auto stride = [&](int j) -> uint32_t {
    if constexpr (kRegStrides) {
      return str_r[j];
    } else {
      return (uint32_t)g.strides[j];
    }
  };
  auto coef = [&](int u, int j) -> double2 {
    if constexpr (kRegCoefs) {
      return cf_r[u][j];
    } else {
      return crow[g.prefC[j] + k[u][j]];
    }
  };
  for (int m = 2; m < Ci; ++m) {
    const double2 cd = crow[g.prefC[i] + m];
    const double rsm = rs[m];
    const double2* Sp = S + ((m - 1) & 1) * per;
    double* Sn = Sd + 2 * (m & 1) * per;
    double acc[A];
#pragma unroll
    for (int u = 0; u < A; ++u) {
      const uint32_t q = lo + a0 + (uint32_t)u * pairs;
      const double op = __shfl_xor_sync(0xffffffffu, gp[u], 1), opp = __shfl_xor_sync(0xffffffffu, gpp[u], 1);
      const double2 Gp = im ? cmk(op, gp[u]) : cmk(gp[u], op);
      const double2 Gpp = im ? cmk(opp, gpp[u]) : cmk(gpp[u], opp);
      acc[u] = part_fma(cd, Gpp, im, part_fma(bi, Gp, im, 0.0));
      if (q < hi) {
#pragma unroll
        for (int j = 1; j < D; ++j) {
          const uint32_t sj = stride(j);
          if (j > i && k[u][j] > 0 && q - sj >= lo)
            acc[u] = part_fma(coef(u, j), Sp[q - sj - lo], im, acc[u]);
        }
      }
    }
    if (!poll && w_lo < w_hi && !flow_wait(h, prog, w_lo, w_hi, kFlowNone, (uint32_t)(m - 1), fp.budget_ns, s_fail))
      return false;
    const int64_t prev = (int64_t)(m - 1) * si;
    if (poll) {
      // halo terms (u, j) in batches of NB: every load of a batch is issued before the first is
      // waited on, so a thread pays one round trip to L2 per batch instead of one per term; each
      // acc[u] still adds its terms in increasing j
      constexpr int DM = D > 1 ? D - 1 : 1, T = A * (D - 1), NB = T < 6 ? (T > 0 ? T : 1) : 6;
#pragma unroll
      for (int t0 = 0; t0 < T; t0 += NB) {
        unsigned long long hx[NB], hy[NB];
#pragma unroll
        for (int t = 0; t < NB; ++t) {
          hx[t] = hy[t] = 0ull;
          const int u = (t0 + t) / DM, j = 1 + (t0 + t) % DM;
          if (t0 + t >= T) continue;
          const uint32_t q = lo + a0 + (uint32_t)u * pairs, sj = stride(j);
          if (q < hi && j > i && k[u][j] > 0 && q - sj < lo) ld_relaxed_v2u64(G + prev + (q - sj), hx[t], hy[t]);
        }
#pragma unroll
        for (int t = 0; t < NB; ++t) {
          const int u = (t0 + t) / DM, j = 1 + (t0 + t) % DM;
          if (t0 + t >= T) continue;
          const uint32_t q = lo + a0 + (uint32_t)u * pairs, sj = stride(j);
          if (q < hi && j > i && k[u][j] > 0 && q - sj < lo)
            acc[u] = part_fma(coef(u, j),
                              halo_wait(G + prev + (q - sj), hx[t], hy[t], h, fp.budget_ns, s_fail), im, acc[u]);
        }
      }
    }
#pragma unroll
    for (int u = 0; u < A; ++u) {
      const uint32_t q = lo + a0 + (uint32_t)u * pairs;
      if (q < hi) {
        if (!poll) {
#pragma unroll
          for (int j = 1; j < D; ++j) {
            const uint32_t sj = stride(j);
            if (j > i && k[u][j] > 0 && q - sj < lo)
              acc[u] = part_fma(coef(u, j), __ldcg(G + prev + (q - sj)), im, acc[u]);
          }
        }
        const double val = not_pending(rsm * acc[u]);
        Gd[2 * ((int64_t)m * si + q) + im] = val;
        Sn[2 * (q - lo) + im] = val;
        gpp[u] = gp[u];
        gp[u] = val;
      }
    }
    __syncthreads();
    if (poll) {
      if (*s_fail) return false;
    } else if (threadIdx.x == 0) {
      st_release_u32(my, (uint32_t)m);
    }
  }
  return true;
}

template <int D>
__global__ void __launch_bounds__(256, 2) fwd_flow_kernel(UniformSrc src, const double* __restrict__ rs, WsHeader* h,
                                                          uint32_t* prog, FlowPlan fp) {
  MM_SHARED(InstView, sv);
  MM_SHARED(int, s_fail);
  MM_SHARED(FlowRole, role);
  MM_SHARED(FlowSmem, smem);
  double2* Gs = smem.g;
  if (threadIdx.x == 0) {
    src.load(0, sv);
    s_fail = 0;
  }
  if (!flow_roles(fp, h, prog + (fp.flag0[0] + fp.ctas[0]), role)) return;
  const Geom& g = sv.g;
  const uint32_t fv = role.face_v;
  const int L = (int)fp.small_lvl;
  if (fv == 0) {
    if (L < D) {  // the small levels, in shared memory, then written out at once
      if (threadIdx.x == 0) Gs[0] = sv.c;
      __syncthreads();
      for (int i = D - 1; i >= L; --i) {
        const uint32_t lanes = min((2u * (uint32_t)g.strides[i] + 31u) / 32u * 32u, blockDim.x);
        if (threadIdx.x < lanes)
          small_level<D>(sv, rs, i, Gs, lanes, sv.coef + (int64_t)i * g.sumC, 0, __ldg(sv.b + i));
        __syncthreads();
      }
      for (uint32_t f = threadIdx.x; f < fp.small_amps; f += blockDim.x)
        stG(sv, f, cmk(not_pending(Gs[f].x), not_pending(Gs[f].y)), 7);
      __syncthreads();
      if (threadIdx.x == 0) {
        st_release_u32(prog, 1u);
        for (int l = L; l < D; ++l) st_release_u32(prog + fp.flag0[l], (uint32_t)g.shape[l] - 1u);
      }
    } else {
      if (threadIdx.x == 0) {
        stG(sv, 0, sv.c, 7);
        st_release_u32(prog, 1u);
      }
      __syncthreads();
    }
  }
  for (int i = min(L, D) - 1; i >= 0; --i) {
    const uint32_t P = fp.ctas[i];
    const uint32_t v = (i > 0) ? fv : role.v0;
    if (v >= P) continue;
    const uint32_t si = (uint32_t)g.strides[i];
    const uint32_t per = fp.per[i];
    const uint32_t lo = min(si, per * v), hi = min(si, lo + per);
    const uint32_t snext = (i + 1 < D) ? (uint32_t)g.strides[i + 1] : 0u;
    const int Ci = (int)g.shape[i];
    if (P > 1 && per <= 2u * blockDim.x) {  // register/shared-memory form on lane pairs
      const uint32_t pairs = blockDim.x >> 1;
      const bool ok = (per <= pairs)       ? flow_level<D, 1>(sv, rs, h, prog, fp, i, v, fv, Gs, &s_fail)
                      : (per <= 2 * pairs) ? flow_level<D, 2>(sv, rs, h, prog, fp, i, v, fv, Gs, &s_fail)
                                           : flow_level<D, 4>(sv, rs, h, prog, fp, i, v, fv, Gs, &s_fail);
      if (!ok) return;
      continue;
    }
    const bool publish_each = P > 1 || (i > 0 && fp.ctas[i - 1] > 1);
    for (int m = 1; m < Ci; ++m) {
      uint32_t w_lo, w_hi, skip = kFlowNone, target;
      if (m >= 2) {
        target = (uint32_t)(m - 1);
        w_lo = fp.flag0[i] + (lo >= snext ? lo - snext : 0u) / per;
        w_hi = fp.flag0[i] + v;
      } else {
        const uint32_t pos = hi - 1;
        int l = i + 1;
        while (l < D && pos / (uint32_t)g.strides[l] == 0) ++l;
        if (l < D) {
          target = pos / (uint32_t)g.strides[l];
          w_lo = fp.flag0[l];
          w_hi = w_lo + fp.ctas[l];
          if (fv < fp.ctas[l]) skip = w_lo + fv;
        } else {  // only G[0] lies below hi
          target = 1u;
          w_lo = 0u;
          w_hi = (fv == 0) ? 0u : 1u;
        }
      }
      if (w_lo < w_hi && !flow_wait(h, prog, w_lo, w_hi, skip, target, fp.budget_ns, &s_fail)) return;
      // L1-cached loads only where every amplitude read was written by this CTA
      // (a one-range level >= 1 and everything below it belong to face CTA 0)
      if (i > 0 && P == 1)
        fwd_chunk<D, false>(sv, rs, i, m, lo, hi, blockDim.x, threadIdx.x);
      else
        fwd_chunk<D, true>(sv, rs, i, m, lo, hi, blockDim.x, threadIdx.x);
      __syncthreads();
      // the CTA barrier orders every thread's stores before thread 0's release
      if (threadIdx.x == 0 && (publish_each || m == Ci - 1)) st_release_u32(prog + fp.flag0[i] + v, (uint32_t)m);
    }
  }
}

// ------------------------------------------------ one small instance on one cluster
// Instances whose slab 0 (the strides[0] amplitudes with k_0 = 0) fits the face
// region, in ONE launch with no setup kernel: every CTA builds the coefficients
// and 1/sqrt(m) values it needs in its own shared memory with the expressions of
// setup_kernel (A_ii sqrt(m - 1), A_ij sqrt(k), 1 / sqrt(m)), so the values are
// the same.  CTA 0 computes levels 1 .. D-1 in its shared memory (small_level,
// lane pairs), then every chunk m >= 1 of level 0 is split over the cluster's
// CTAs in contiguous ranges [lo, hi), one hardware cluster barrier per chunk.  A
// lane pair keeps the last two values of its amplitudes in registers and a CTA
// its range of the previous chunk in shared memory (S).  The neighbours
// q - strides[j] below `lo` (at most `hmax`, the largest stride of an axis
// j >= 1, away) are PUSHED by the CTAs that own them, right after they compute
// them, into the halo buffer H of every CTA that will read them (remote
// shared-memory stores), so a chunk reads only its own shared memory and the
// push latency is hidden behind the barrier.  Slab 0 is pushed the same way by
// CTA 0 before chunk 1.  The only waits are hardware cluster barriers that every
// CTA reaches the same number of times.
constexpr uint32_t kClusterRangeMax = 512;   // amplitudes of one CTA's level-0 range (A <= 4 at 256 threads)
constexpr uint32_t kClusterHaloMax = 1280;   // hmax <= strides[0] / 2 <= kFlowSmemAmps / 2
constexpr uint32_t kClusterCoefMax = 2560;   // coefficient columns j >= 1 of levels 1 .. D-1
constexpr uint32_t kClusterC0Max = 1024;     // extent of axis 0 (per-chunk tables of level 0)
constexpr uint32_t kClusterRsMax = kFlowSmemAmps + 1;

__host__ __device__ constexpr size_t cluster_fwd_smem_bytes() {
  return (size_t)(kFlowSmemAmps + 2 * kClusterRangeMax + 2 * kClusterHaloMax + kClusterCoefMax + kClusterC0Max +
                  MM_MAXD * MM_MAXD + MM_MAXD + 8) * sizeof(double2) +
         (size_t)(kClusterRsMax + 1 + kClusterC0Max) * sizeof(double);
}

// Largest stride of an axis j >= 1 whose extent is at least 2 (the farthest
// neighbour of level 0); 0 if there is none.
__host__ __device__ inline uint32_t cluster_halo(const Geom& g) {
  uint32_t h = 0;
  for (int j = 1; j < g.D; ++j)
    if (g.shape[j] >= 2 && (uint32_t)g.strides[j] > h) h = (uint32_t)g.strides[j];
  return h;
}

// Coefficient columns j >= 1 (levels 1 .. D-1 read only those).
__host__ __device__ inline uint32_t cluster_coef_cols(const Geom& g) { return (uint32_t)(g.sumC - g.shape[0]); }

// Largest extent of an axis j >= 1.
__host__ __device__ inline uint32_t cluster_face_cmax(const Geom& g) {
  uint32_t c = 1;
  for (int j = 1; j < g.D; ++j) c = max(c, (uint32_t)g.shape[j]);
  return c;
}

// Whether an instance fits fwd_cluster_kernel's shared-memory tables.
__host__ __device__ inline bool cluster_fits(const Geom& g) {
  return g.strides[0] <= (int64_t)kFlowSmemAmps && g.shape[0] <= (int64_t)kClusterC0Max &&
         (uint64_t)(g.D - 1) * cluster_coef_cols(g) <= kClusterCoefMax && cluster_face_cmax(g) < kClusterRsMax;
}

__device__ __forceinline__ uint32_t cluster_addr(const void* local, uint32_t peer) {
#if defined(__CUDA_ARCH__)
  uint32_t a = (uint32_t)__cvta_generic_to_shared(local), r;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(a), "r"(peer));
  return r;
#else
  (void)peer;
  return (uint32_t)(uintptr_t)local;
#endif
}
__device__ __forceinline__ void cluster_st(const double* local, uint32_t peer, double x) {
#if defined(__CUDA_ARCH__)
  asm volatile("st.shared::cluster.f64 [%0], %1;" ::"r"(cluster_addr(local, peer)), "d"(x) : "memory");
#else
  (void)peer;
  *const_cast<double*>(local) = x;
#endif
}
__device__ __forceinline__ void cluster_st2(const double2* local, uint32_t peer, double2 x) {
#if defined(__CUDA_ARCH__)
  asm volatile("st.shared::cluster.v2.f64 [%0], {%1, %2};" ::"r"(cluster_addr(local, peer)), "d"(x.x), "d"(x.y)
               : "memory");
#else
  (void)peer;
  *const_cast<double2*>(local) = x;
#endif
}

// setup_kernel's coefficient of row i, column c (axis j = the one holding c).
__device__ __forceinline__ double2 cluster_coef(const Geom& g, const double2* As, int i, int32_t c) {
  int j = 0;
  while (j + 1 < g.D && g.prefC[j + 1] <= c) ++j;
  const int32_t kk = c - g.prefC[j];
  const double2 a = As[i * g.D + j];
  const double s = (j == i) ? (kk >= 1 ? sqrt((double)(kk - 1)) : 0.0) : sqrt((double)kk);
  return cmk(a.x * s, a.y * s);
}

template <int D, int A>
__global__ void __launch_bounds__(256) fwd_cluster_kernel(UniformSrc src) {
  extern __shared__ __align__(16) unsigned char cluster_smem[];
  double2* face = reinterpret_cast<double2*>(cluster_smem);
  double2* S = face + kFlowSmemAmps;        // [2][kClusterRangeMax]: own range of chunks m - 1, m
  double2* H = S + 2 * kClusterRangeMax;    // [2][kClusterHaloMax]: H[.][t] = amplitude lo - 1 - t
  double2* cst = H + 2 * kClusterHaloMax;   // coefficient columns j >= 1 of levels 1 .. D-1 (CTA 0)
  double2* cd0 = cst + kClusterCoefMax;     // A_00 sqrt(m - 1), m < C0
  double2* As = cd0 + kClusterC0Max;        // A (D x D)
  double2* bs = As + MM_MAXD * MM_MAXD;     // b, then c
  double* rst = reinterpret_cast<double*>(bs + MM_MAXD + 8);  // 1 / sqrt(m), m <= max C_i (i >= 1)
  double* rs0 = rst + kClusterRsMax + 1;                       // 1 / sqrt(m), m < C0
  MM_SHARED(InstView, sv);
  const uint32_t rank = cluster_rank(), nranks = cluster_size();
  // CTA 0 computes slab 0; level 0 is split over the other CTAs ("workers"; CTA 0 too if it is alone),
  // which build their tables and per-amplitude coefficients while CTA 0 works on slab 0
  const uint32_t base = nranks > 1 ? 1u : 0u, nwork = nranks - base;
  const bool worker = rank >= base;
  const uint32_t wr = worker ? rank - base : 0u;
  if (threadIdx.x == 0) src.load(0, sv);
  __syncthreads();
  const Geom& g = sv.g;
  const uint32_t s0 = (uint32_t)g.strides[0];
  const uint32_t per = (s0 + nwork - 1) / nwork;
  const uint32_t lo = worker ? min(s0, per * wr) : 0u, hi = worker ? min(s0, lo + per) : 0u;
  const uint32_t hmax = cluster_halo(g);
  const int C0 = (int)g.shape[0];
  for (uint32_t e = threadIdx.x; e < (uint32_t)(D * D); e += blockDim.x) As[e] = sv.A[e];
  if (threadIdx.x < (uint32_t)D) bs[threadIdx.x] = sv.b[threadIdx.x];
  if (threadIdx.x == (uint32_t)D) bs[D] = sv.c;
  __syncthreads();
  if (worker) {  // level-0 tables
    for (uint32_t m = threadIdx.x; m < (uint32_t)C0; m += blockDim.x) {
      const double sm = sqrt((double)m);
      rs0[m] = m > 0 ? 1.0 / sm : 0.0;
      const double s = m >= 1 ? sqrt((double)(m - 1)) : 0.0;
      cd0[m] = cmk(As[0].x * s, As[0].y * s);
    }
  }
  const bool im = (threadIdx.x & 1u) != 0;
  const uint32_t pairs = blockDim.x >> 1, a0 = threadIdx.x >> 1;
  int32_t k[A][D];
  double2 w[A][D];    // A_0j sqrt(k_j) of each amplitude (j >= 1; zero where k_j = 0): constant along m
  uint32_t ncons[A];  // workers after this one whose halo holds the amplitude
#pragma unroll
  for (int u = 0; u < A; ++u) {
    const uint32_t q = lo + a0 + (uint32_t)u * pairs;
    decompose<D>(q < hi ? q : 0u, 1, g, k[u]);
    uint32_t nc = 0;
    while (q < hi && wr + 1 + nc < nwork && (wr + 1 + nc) * per <= q + hmax) ++nc;
    ncons[u] = nc;
#pragma unroll
    for (int j = 0; j < D; ++j) {
      w[u][j] = cmk(0.0, 0.0);
      if (j >= 1 && q < hi && k[u][j] > 0) {
        const double sk = sqrt((double)k[u][j]);
        w[u][j] = cmk(As[j].x * sk, As[j].y * sk);
      }
    }
  }
  if (rank == 0) {
    const uint32_t R = cluster_coef_cols(g), fc = cluster_face_cmax(g);
    for (uint32_t m = threadIdx.x; m <= fc; m += blockDim.x) rst[m] = m > 0 ? 1.0 / sqrt((double)m) : 0.0;
    for (uint32_t e = threadIdx.x; e < (uint32_t)(D - 1) * R; e += blockDim.x) {
      const uint32_t i = 1 + e / R, col = e - (i - 1) * R;
      cst[e] = cluster_coef(g, As, (int)i, g.prefC[1] + (int32_t)col);
    }
    if (threadIdx.x == 0) face[0] = bs[D];
    __syncthreads();
    for (int i = D - 1; i >= 1; --i) {
      const uint32_t lanes = min((2u * (uint32_t)g.strides[i] + 31u) / 32u * 32u, blockDim.x);
      if (threadIdx.x < lanes) small_level<D>(sv, rst, i, face, lanes, cst + (int64_t)(i - 1) * R, g.prefC[1], bs[i]);
      __syncthreads();
    }
    // slab 0: to G, and pushed to every CTA as its "previous chunk" (S[0]) and halo (H[0])
    for (uint32_t q = threadIdx.x; q < s0; q += blockDim.x) {
      const double2 v = face[q];
      stG(sv, q, v, 7);
      if (C0 >= 2) {
        const uint32_t r = q / per;  // worker owning q
        cluster_st2(S + (q - r * per), r + base, v);
        for (uint32_t r2 = r + 1; r2 < nwork && r2 * per <= q + hmax; ++r2)
          cluster_st2(H + (r2 * per - 1 - q), r2 + base, v);
      }
    }
  }
  cluster_sync();
  if (C0 < 2) return;  // the same in every CTA: no barrier is skipped by some only
  const double2 b0 = bs[0];
  double* Gd = reinterpret_cast<double*>(sv.G);
  double* Sd = reinterpret_cast<double*>(S);
  double* Hd = reinterpret_cast<double*>(H);
  double gp[A], gpp[A];
#pragma unroll
  for (int u = 0; u < A; ++u) {
    const uint32_t q = lo + a0 + (uint32_t)u * pairs;
    gpp[u] = 0.0;
    gp[u] = q < hi ? Sd[2 * (q - lo) + (im ? 1 : 0)] : 0.0;  // slab 0 (pushed by CTA 0)
  }
  uint32_t str[D];  // strides in registers: the cluster barrier at each chunk's end would force them to be re-read
#pragma unroll
  for (int j = 0; j < D; ++j) str[j] = (uint32_t)g.strides[j];
  for (int m = 1; m < C0; ++m) {
    const double2 cd = cd0[m];
    const double rsm = rs0[m];
    const uint32_t pb = ((m - 1) & 1u), nb = (m & 1u);
    const double2* Sp = S + pb * kClusterRangeMax;
    const double2* Hp = H + pb * kClusterHaloMax;
#pragma unroll
    for (int u = 0; u < A; ++u) {
      const uint32_t q = lo + a0 + (uint32_t)u * pairs;
      const double op = __shfl_xor_sync(0xffffffffu, gp[u], 1), opp = __shfl_xor_sync(0xffffffffu, gpp[u], 1);
      if (q < hi) {
        double2 x[D];
#pragma unroll
        for (int j = 1; j < D; ++j) {
          x[j] = cmk(0.0, 0.0);
          if (k[u][j] > 0) {
            const uint32_t qn = q - str[j];
            x[j] = qn >= lo ? Sp[qn - lo] : Hp[lo - 1 - qn];
          }
        }
        const double2 Gp = im ? cmk(op, gp[u]) : cmk(gp[u], op);
        const double2 Gpp = im ? cmk(opp, gpp[u]) : cmk(gpp[u], opp);
        double acc = part_fma(b0, Gp, im, 0.0);
        if (m >= 2) acc = part_fma(cd, Gpp, im, acc);
#pragma unroll
        for (int j = 1; j < D; ++j)
          if (k[u][j] > 0) acc = part_fma(w[u][j], x[j], im, acc);
        const double val = rsm * acc;
        const uint32_t pi = im ? 1u : 0u;
        Gd[2 * ((int64_t)m * s0 + q) + pi] = val;
        Sd[2 * (nb * kClusterRangeMax + (q - lo)) + pi] = val;
        for (uint32_t c = 0; c < ncons[u]; ++c) {
          const uint32_t r2 = wr + 1 + c;  // worker index
          cluster_st(Hd + 2 * (nb * kClusterHaloMax + (r2 * per - 1 - q)) + pi, r2 + base, val);
        }
        gpp[u] = gp[u];
        gp[u] = val;
      }
    }
    cluster_sync();
  }
}

// Device self-test of view construction: load instance k of `src` into a
// shared view exactly as the compute kernels do and compare every field with
// the host's expectation.  Only `src.c[k]` (a valid workspace address) is read.
template <class Src>
__global__ void view_selftest_kernel(Src src, int64_t k, const InstView* __restrict__ expect, int32_t* bad) {
  MM_SHARED(InstView, sv);
  if (threadIdx.x == 0) src.load(k, sv);
  __syncthreads();
  if (threadIdx.x == 0) {
    const InstView& e = *expect;
    int nbad = 0;
    nbad += sv.A != e.A;
    nbad += sv.b != e.b;
    nbad += sv.G != e.G;
    nbad += sv.dLdG != e.dLdG;
    nbad += sv.coef != e.coef;
    nbad += sv.Gh != e.Gh;
    nbad += sv.c.x != e.c.x || sv.c.y != e.c.y;
    nbad += sv.g.D != e.g.D || sv.g.maxC != e.g.maxC || sv.g.n != e.g.n || sv.g.sumC != e.g.sumC;
    for (int j = 0; j < MM_MAXD; ++j)
      nbad += sv.g.shape[j] != e.g.shape[j] || sv.g.strides[j] != e.g.strides[j] || sv.g.prefC[j] != e.g.prefC[j];
    *bad = nbad;
  }
}

// Test kernel: a barrier whose target can never be reached (one extra arrival
// is required), so every CTA gives up after budget_ns.
__global__ void wait_timeout_test_kernel(WsHeader* h, uint64_t budget_ns) { grid_barrier(h, 1, budget_ns, 1); }

// ============================================================== binomial fill
// Binomial strategy (reference: strategies/binomial.py:30-70): the tensor is
// filled wave by wave, wave w holding every amplitude of total photon number
// |k| = w, and the fill stops after the first wave whose running sum of |G|^2
// exceeds max_l2.  Each amplitude obeys the vanilla recurrence with the first
// non-zero axis as pivot (steps.vanilla_step), computed as fwd_chunk does.
//
// Only the waves up to the stop are computed.  Wave w has n_w = S_0[w] -
// S_0[w-1] amplitudes, from cumulative composition counts S_j[x] = number of
// (k_j, ..., k_{D-1}) inside the cutoffs with sum <= x (rows j = 0..D of W1 =
// max weight + 1 entries, S_D[x] = 1).  Its rank r in [0, n_w) maps to an
// index either through the weight-sorted prefix permutation
// (binomial_perm_kernel: one read) or, for very many prefixes, by unranking
// the lexicographic order of paths.binomial_subspace_basis (a binary search
// per axis in S).  The rank order only fixes the order of the norm's sums.
struct BinomialState {
  double norm;      // |c|^2 plus the sums of the waves filled so far
  int32_t stopped;  // 1 once the running norm exceeded max_l2
  int32_t pad;
};

// Rows T_nax .. T_0 of a count table over the axes 0 .. nax-1 (T_j[x] = number
// of (k_j, ..., k_{nax-1}) inside the cutoffs with sum <= x; row j from row j+1:
// the count of weight x is T_{j+1}[x] - T_{j+1}[x - C_j], then an inclusive
// scan).  One CTA: each thread scans a contiguous chunk of a row, warp 0 scans
// the chunk totals with shuffles.
__device__ void binomial_counts(const Geom& g, int nax, int32_t W, int64_t* __restrict__ T, int64_t* s_tot) {
  const int t = (int)threadIdx.x, nt = (int)blockDim.x;
  for (int32_t x = t; x < W; x += nt) T[(int64_t)nax * W + x] = 1;
  __syncthreads();
  const int32_t chunk = (W + nt - 1) / nt;
  const int32_t lo = min(W, t * chunk), hi = min(W, lo + chunk);
  const int per_lane = (nt + 31) / 32;  // chunk totals per lane of warp 0
  for (int j = nax - 1; j >= 0; --j) {
    const int64_t C = g.shape[j];
    const int64_t* nxt = T + (int64_t)(j + 1) * W;
    int64_t* row = T + (int64_t)j * W;
    int64_t sum = 0;
    for (int32_t x = lo; x < hi; ++x) {
      const int64_t cnt = nxt[x] - (x >= C ? nxt[x - C] : 0);
      row[x] = cnt;
      sum += cnt;
    }
    s_tot[t] = sum;
    __syncthreads();
    if (t < 32) {
      // exclusive prefix of the totals: per-lane serial sums, a shuffle scan across lanes
      int64_t part = 0;
      for (int u = t * per_lane; u < min(nt, (t + 1) * per_lane); ++u) part += s_tot[u];
      int64_t inc = part;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int64_t v = __shfl_up_sync(0xffffffffu, inc, o);
        if (t >= o) inc += v;
      }
      int64_t acc = inc - part;
      for (int u = t * per_lane; u < min(nt, (t + 1) * per_lane); ++u) {
        const int64_t v = s_tot[u];
        s_tot[u] = acc;
        acc += v;
      }
    }
    __syncthreads();
    int64_t run = s_tot[t];
    for (int32_t x = lo; x < hi; ++x) {
      run += row[x];
      row[x] = run;
    }
    __syncthreads();
  }
}

// CTA 0: the table S over all D axes (W1 = max weight + 1); CTA 1 (when Sp is
// given): the table Sp over the prefix axes 0 .. D-2 (W1p = their max weight + 1).
__global__ void __launch_bounds__(256) binomial_table_kernel(Geom g, int32_t W1, int64_t* __restrict__ S, int32_t W1p,
                                                             int64_t* __restrict__ Sp) {
  MM_SHARED(int64_t, s_tot[256]);
  if (blockIdx.x == 0) binomial_counts(g, g.D, W1, S, s_tot);
  else if (Sp) binomial_counts(g, g.D - 1, W1p, Sp, s_tot);
}

// The prefixes p (flat index over the axes 0 .. D-2, last of them fastest)
// sorted by their weight s, lexicographic within a weight: perm[pos] = p with
// pos = #{prefixes of weight < s} + the prefix's lexicographic rank among those
// of weight s (sum over its axes of Sp_{j+1}[R_j] - Sp_{j+1}[R_j - k_j]).  The
// indices of wave w are then the prefixes of weights max(0, w - C_{D-1} + 1) ..
// min(w, max prefix weight), a contiguous run of perm, completed by
// k_{D-1} = w - s.
__global__ void __launch_bounds__(256) binomial_perm_kernel(Geom g, const int64_t* __restrict__ Sp, int32_t W1p,
                                                            uint32_t* __restrict__ perm, int64_t P) {
  const int D = g.D;
  auto T = [&](int j, int32_t x) -> int64_t { return x < 0 ? 0 : Sp[(int64_t)j * W1p + min(x, W1p - 1)]; };
  for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < P; p += (int64_t)gridDim.x * blockDim.x) {
    int32_t k[MM_MAXD];
    int64_t q = p;
    int32_t s = 0;
    for (int j = D - 2; j >= 0; --j) {
      const int64_t C = g.shape[j];
      k[j] = (int32_t)(q % C);
      q /= C;
      s += k[j];
    }
    int64_t rank = 0;
    int32_t R = s;
    for (int j = 0; j < D - 1; ++j) {
      rank += T(j + 1, R) - T(j + 1, R - k[j]);
      R -= k[j];
    }
    perm[T(0, s - 1) + rank] = (uint32_t)p;
  }
}

__device__ __forceinline__ int64_t bn_S(const int64_t* S, int32_t W1, int j, int32_t x) {
  return x < 0 ? 0 : S[(int64_t)j * W1 + min(x, W1 - 1)];
}

struct BinomialSmem {
  double warp[MM_BLOCK / 32];
  double sub;
  double mine[2];  // this CTA's wave sums by wave parity (read by the cluster's CTAs)
};

// Read-only operands staged in dynamic shared memory when they fit (0: read
// them from global memory): the count tables, the coefficient block, the
// 1/sqrt table and the prefix permutation.  The barriers' acquire side may
// discard L1 lines, so their dependent reads would otherwise go to L2 on every
// wave.
struct BinomialStage {
  int32_t table_n;  // int64 entries of the count table S, (D + 1) * W1
  int32_t sp_n;     // int64 entries of the prefix count table Sp, D * W1p
  int32_t coef_n;   // double2 entries of the coefficient block, D * sumC
  int32_t rs_n;     // double entries of the 1/sqrt table, maxC + 1
  int32_t perm_n;   // uint32 entries of the prefix permutation
};

// Byte offsets of the staged operands: S | Sp | coefficients (16-byte aligned) | 1/sqrt | permutation.
__host__ __device__ __forceinline__ size_t bn_stage_coef_offset(const BinomialStage& st) {
  return ((size_t)(st.table_n + st.sp_n) * sizeof(int64_t) + 15) & ~(size_t)15;
}
__host__ __device__ __forceinline__ size_t bn_stage_perm_offset(const BinomialStage& st) {
  return bn_stage_coef_offset(st) + (size_t)st.coef_n * sizeof(double2) + (size_t)st.rs_n * sizeof(double);
}
__host__ __device__ __forceinline__ size_t bn_stage_bytes(const BinomialStage& st) {
  return bn_stage_perm_offset(st) + (size_t)st.perm_n * sizeof(uint32_t);
}

__device__ __forceinline__ double bn_cluster_peer_load(const double* local, uint32_t peer) {
#if defined(__CUDA_ARCH__)
  uint32_t a = (uint32_t)__cvta_generic_to_shared(local), r;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(a), "r"(peer));
  double v;
  asm volatile("ld.shared::cluster.f64 %0, [%1];" : "=d"(v) : "r"(r) : "memory");
  return v;
#else
  (void)peer;
  return *local;
#endif
}

// Waves [w_begin, w_end) of one tensor.  MODE 0: one CTA (CTA barriers);
// MODE 1: one thread-block cluster (cluster barriers, wave sums exchanged
// through distributed shared memory); MODE 2: a cooperative grid (bounded
// grid barriers, wave sums through part[(w & 1) * nranks + rank]).  Wave w's
// ranks are strided over the launch's threads; every CTA sums its |G|^2 in a
// fixed order, and after the barrier every CTA adds the wave's per-CTA sums
// in CTA order to its own copy of the norm, so all CTAs take the same stop
// decision.  With w_begin == 1 the launch writes G[0] = c and starts the norm
// at |c|^2; otherwise it continues from *state (left by the previous launch).
template <int D, int MODE>
__global__ void __launch_bounds__(MM_BLOCK) binomial_wave_kernel(UniformSrc src, const double* __restrict__ rs_g,
                                                                 const int64_t* __restrict__ S_g, int32_t W1,
                                                                 const int64_t* __restrict__ Sp_g, int32_t W1p,
                                                                 const uint32_t* __restrict__ perm_g,
                                                                 BinomialStage stage, int32_t w_begin, int32_t w_end,
                                                                 double max_l2, double* __restrict__ part,
                                                                 BinomialState* state, double* __restrict__ norm_out,
                                                                 WsHeader* h, uint64_t budget_ns) {
  MM_SHARED(InstView, sv);
  MM_SHARED(BinomialSmem, sm);
  extern __shared__ __align__(16) unsigned char bn_dyn[];
  // a launch that continues a fill which has already stopped only republishes the norm
  if (w_begin > 1 && state->stopped) {
    if (blockIdx.x == 0 && threadIdx.x == 0 && norm_out) *norm_out = state->norm;
    return;
  }
  if (threadIdx.x == 0) src.load(0, sv);
  __syncthreads();
  const Geom& g = sv.g;
  // staging
  int64_t* s_tab = reinterpret_cast<int64_t*>(bn_dyn);
  int64_t* s_sp = s_tab + stage.table_n;
  double2* s_coef = reinterpret_cast<double2*>(bn_dyn + bn_stage_coef_offset(stage));
  double* s_rs = reinterpret_cast<double*>(s_coef + stage.coef_n);
  uint32_t* s_perm = reinterpret_cast<uint32_t*>(bn_dyn + bn_stage_perm_offset(stage));
  for (int32_t e = threadIdx.x; e < stage.table_n; e += blockDim.x) s_tab[e] = S_g[e];
  for (int32_t e = threadIdx.x; e < stage.sp_n; e += blockDim.x) s_sp[e] = Sp_g[e];
  for (int32_t e = threadIdx.x; e < stage.coef_n; e += blockDim.x) s_coef[e] = ldCoef(sv, sv.coef + e, 5);
  for (int32_t e = threadIdx.x; e < stage.rs_n; e += blockDim.x) s_rs[e] = rs_g[e];
  for (int32_t e = threadIdx.x; e < stage.perm_n; e += blockDim.x) s_perm[e] = perm_g[e];
  __syncthreads();
  const int64_t* S = stage.table_n ? s_tab : S_g;
  const int64_t* Sp = stage.sp_n ? s_sp : Sp_g;
  const double2* coef = stage.coef_n ? s_coef : sv.coef;
  const double* rs = stage.rs_n ? s_rs : rs_g;
  const uint32_t* perm = stage.perm_n ? s_perm : perm_g;  // null: unrank by binary search
  uint32_t rank, nranks;
  if constexpr (MODE == 1) {
    rank = cluster_rank();
    nranks = cluster_size();
  } else {
    rank = blockIdx.x;
    nranks = gridDim.x;
  }
  uint32_t epoch = 0;
  auto sync_all = [&]() -> bool {
    if constexpr (MODE == 0) {
      __syncthreads();
      return true;
    } else if constexpr (MODE == 1) {
      cluster_sync();
      return true;
    } else {
      return grid_barrier(h, ++epoch, budget_ns, 0);
    }
  };
  double2* G = sv.G;
  double norm;
  int32_t stopped;
  if (w_begin == 1) {
    const double hc = hypot(sv.c.x, sv.c.y);
    norm = hc * hc;
    stopped = 0;
    if (rank == 0 && threadIdx.x == 0) stG(sv, 0, sv.c, 7);
    if (!sync_all()) return;
  } else {
    norm = state->norm;
    stopped = 0;
  }
  int64_t sj[D];
  int32_t pj[D], cj[D];
  double2 bj[D];
#pragma unroll
  for (int j = 0; j < D; ++j) {
    sj[j] = g.strides[j];
    pj[j] = g.prefC[j];
    cj[j] = (int32_t)g.shape[j];
    bj[j] = __ldg(sv.b + j);
  }
  const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
  const int64_t T = (int64_t)nranks * blockDim.x;
  const int64_t r0 = (int64_t)rank * blockDim.x + threadIdx.x;
  // rank r of wave w -> index k (lexicographic order)
  auto unrank = [&](int64_t rr, int32_t w, int32_t(&k)[D]) {
    int32_t R = w;
#pragma unroll
    for (int j = 0; j < D - 1; ++j) {
      const int64_t tot = bn_S(S, W1, j + 1, R);
      int32_t lo = 0, hi = min(cj[j] - 1, R);
      while (lo < hi) {
        const int32_t mid = (lo + hi + 1) >> 1;
        if (tot - bn_S(S, W1, j + 1, R - mid) <= rr) lo = mid;
        else hi = mid - 1;
      }
      rr -= tot - bn_S(S, W1, j + 1, R - lo);
      k[j] = lo;
      R -= lo;
    }
    k[D - 1] = R;
  };
  // the same index from the prefix permutation: one table read and the prefix's digits
  auto from_perm = [&](int64_t rr, int32_t w, int32_t(&k)[D]) {
    const int32_t lo_s = max(0, w - (cj[D - 1] - 1));
    uint32_t q = perm[bn_S(Sp, W1p, 0, lo_s - 1) + rr];
    int32_t sum = 0;
#pragma unroll
    for (int j = D - 2; j >= 0; --j) {
      const uint32_t c = (uint32_t)cj[j];
      k[j] = (int32_t)(q % c);
      q /= c;
      sum += k[j];
    }
    k[D - 1] = w - sum;
  };
  auto index_of = [&](int64_t rr, int32_t w, int32_t(&k)[D]) {
    if (perm) from_perm(rr, w, k);
    else unrank(rr, w, k);
  };
  // this thread's first index of the next wave, unranked ahead of the wave's barrier
  int32_t kn[D];
  if (w_begin < w_end && r0 < bn_S(S, W1, 0, w_begin) - bn_S(S, W1, 0, w_begin - 1)) index_of(r0, w_begin, kn);
  for (int32_t w = w_begin; w < w_end && !stopped; ++w) {
    const int64_t nw = bn_S(S, W1, 0, w) - bn_S(S, W1, 0, w - 1);
    double local = 0.0;
    for (int64_t r = r0; r < nw; r += T) {
      int32_t k[D];
      if (r == r0) {
#pragma unroll
        for (int j = 0; j < D; ++j) k[j] = kn[j];
      } else {
        index_of(r, w, k);
      }
      int64_t f = 0;
#pragma unroll
      for (int j = 0; j < D; ++j) f += (int64_t)k[j] * sj[j];
      // pivot: the first non-zero axis
      int piv = 0, kp = 0, pp = 0;
      int64_t sp = 0;
      double2 bp = cmk(0.0, 0.0);
      bool found = false;
#pragma unroll
      for (int j = 0; j < D; ++j) {
        if (!found && k[j] > 0) {
          found = true;
          piv = j;
          kp = k[j];
          pp = pj[j];
          sp = sj[j];
          bp = bj[j];
        }
      }
      const double2* crow = coef + (int64_t)piv * g.sumC;
      const int64_t p = f - sp;
      // one CTA: its own earlier writes, plain (L1) loads; otherwise L2 loads
      constexpr bool kCG = MODE != 0;
      double2 acc = cmul(bp, ldGc<kCG>(sv, G + p, 4));
      if (kp >= 2) acc = cfma(crow[pp + kp], ldGc<kCG>(sv, G + p - sp, 4), acc);
#pragma unroll
      for (int j = 1; j < D; ++j) {
        if (j > piv && k[j] > 0) acc = cfma(crow[pj[j] + k[j]], ldGc<kCG>(sv, G + p - sj[j], 4), acc);
      }
      const double2 val = cscale(rs[kp], acc);
      stG(sv, f, val, 6);
      local += fma(val.x, val.x, val.y * val.y);
    }
    if (w + 1 < w_end && r0 < bn_S(S, W1, 0, w + 1) - bn_S(S, W1, 0, w)) index_of(r0, w + 1, kn);
    // fixed-order CTA sum; warps without ranks in this wave hold exactly 0
    const bool warp_busy = (r0 - lane) < nw;
    if (warp_busy) {
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) local += __shfl_xor_sync(0xffffffffu, local, o);
    }
    if (lane == 0) sm.warp[warp] = local;
    __syncthreads();
    if (warp == 0) {
      const uint32_t nwarps = blockDim.x >> 5;  // a power of two
      double x = lane < nwarps ? sm.warp[lane] : 0.0;
      for (uint32_t o = nwarps >> 1; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
      if (lane == 0) {
        if constexpr (MODE == 0) sm.sub = x;
        else if constexpr (MODE == 1) sm.mine[w & 1] = x;
        else part[(w & 1) * nranks + rank] = x;
      }
    }
    if (!sync_all()) return;
    if constexpr (MODE != 0) {
      if (warp == 0) {
        double x = 0.0;
        for (uint32_t q = lane; q < nranks; q += 32) {
          if constexpr (MODE == 1) x += bn_cluster_peer_load(&sm.mine[w & 1], q);
          else x += __ldcg(part + (w & 1) * nranks + q);
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
        if (lane == 0) sm.sub = x;
      }
      __syncthreads();
    }
    norm += sm.sub;
    if (norm > max_l2) stopped = 1;
  }
  if constexpr (MODE == 1) cluster_sync();  // no CTA leaves while a peer may still read its wave sums
  if (rank == 0 && threadIdx.x == 0) {
    state->norm = norm;
    state->stopped = stopped;
    if (norm_out) *norm_out = norm;
  }
}

// No early stop (max_l2 = +inf): the fill is the vanilla forward's, kept up to
// wave `last`.  Zeroes every amplitude of weight > last and writes each CTA's
// fixed-order sum of |G|^2 over the kept ones to part[blockIdx.x].
template <int D>
__global__ void __launch_bounds__(256) binomial_mask_norm_kernel(double2* __restrict__ G, Geom g, int64_t last,
                                                                 double* __restrict__ part) {
  MM_SHARED(double, s_warp[8]);
  double acc = 0.0;
  for (int64_t f = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; f < g.n; f += (int64_t)gridDim.x * blockDim.x) {
    int64_t q = f, w = 0;
#pragma unroll
    for (int j = D - 1; j >= 0; --j) {
      const int64_t c = g.shape[j];
      w += q % c;
      q /= c;
    }
    if (w > last) {
      G[f] = cmk(0.0, 0.0);
    } else {
      const double2 v = G[f];
      acc += fma(v.x, v.x, v.y * v.y);
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) s_warp[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x < 32) {
    double x = threadIdx.x < (blockDim.x >> 5) ? s_warp[threadIdx.x] : 0.0;
#pragma unroll
    for (int o = 4; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
    if (threadIdx.x == 0) part[blockIdx.x] = x;
  }
}

// One warp: the CTAs' sums in CTA order (lane-strided, then a fixed tree).
__global__ void binomial_norm_final_kernel(const double* __restrict__ part, int n, double* __restrict__ norm_out) {
  double x = 0.0;
  for (int q = (int)threadIdx.x; q < n; q += 32) x += part[q];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
  if (threadIdx.x == 0 && norm_out) *norm_out = x;
}

// ============================================================== VJP
// Per-thread accumulation over the fibers q of [q0, q1) (q = flat index over
// axes 1..D-1) for one instance; results go to tot[] (weights applied).
// gout (optional): receives G[f] for every amplitude of the item's fibers, so a caller that
// needs G elsewhere (pinned host memory) gets it from the loads the VJP makes anyway.
template <int D, bool COPY = false, bool PF = false>
__device__ __forceinline__ void vjp_fibers(const InstView& v, const Tables& T, uint32_t q0, uint32_t q1,
                                           double2 (&tot)[vjp_nv(D)], double2* gout = nullptr) {
  constexpr int NV = vjp_nv(D);
  const Geom& g = v.g;
  const int C0 = (int)g.shape[0];
  const int64_t s0 = g.strides[0];
  int64_t sj[D];
#pragma unroll
  for (int j = 0; j < D; ++j) sj[j] = g.strides[j];
  const double2* __restrict__ G = v.G;
  const double2* __restrict__ gb = v.dLdG;
  const double* __restrict__ sq = T.sq;
  const double* __restrict__ hh = T.hh;
  for (uint32_t q = q0 + threadIdx.x; q < q1; q += blockDim.x) {
    int32_t r[D];
    decompose<D>(q, 1, g, r);
    double2 a[NV];
#pragma unroll
    for (int s = 0; s < NV; ++s) a[s] = cmk(0.0, 0.0);
    // PF (the host-buffer step: the cotangent is read over the host link from pinned host memory):
    // each cotangent value is loaded two steps of k_0 ahead of its use, hiding that latency (one
    // step ahead hid part of it; from device memory an early load measured ~1 % slower, so it is
    // not used there)
    double2 gu_next = PF ? __ldg(gb + q) : cmk(0.0, 0.0);
    double2 gu_next2 = (PF && C0 > 1) ? __ldg(gb + s0 + q) : cmk(0.0, 0.0);
    for (int m = 0; m < C0; ++m) {
      const int64_t f = (int64_t)m * s0 + q;
      double2 gu;
      if constexpr (PF) {
        gu = gu_next;
        gu_next = gu_next2;
        if (m + 2 < C0) gu_next2 = __ldg(gb + f + 2 * s0);
      } else {
        gu = __ldg(gb + f);
      }
      const double2 gf = __ldg(G + f);
      a[0] = cfma(gf, gu, a[0]);
      if constexpr (COPY) gout[f] = gf;
      if (m >= 1) {
        const double2 h0 = cscale(sq[m], gu);
        a[1] = cfma(__ldg(G + f - s0), h0, a[1]);
#pragma unroll
        for (int j = 1; j < D; ++j)
          if (r[j] >= 1) a[vjp_slot(D, 0, j)] = cfma(__ldg(G + f - s0 - sj[j]), h0, a[vjp_slot(D, 0, j)]);
        if (m >= 2) {
          const double2 h00 = cscale(hh[m], gu);
          a[vjp_slot(D, 0, 0)] = cfma(__ldg(G + f - 2 * s0), h00, a[vjp_slot(D, 0, 0)]);
        }
      }
#pragma unroll
      for (int i = 1; i < D; ++i) {
        if (r[i] >= 1) {
          a[1 + i] = cfma(__ldg(G + f - sj[i]), gu, a[1 + i]);
          if (r[i] >= 2) a[vjp_slot(D, i, i)] = cfma(__ldg(G + f - 2 * sj[i]), gu, a[vjp_slot(D, i, i)]);
#pragma unroll
          for (int j = i + 1; j < D; ++j)
            if (r[j] >= 1) a[vjp_slot(D, i, j)] = cfma(__ldg(G + f - sj[i] - sj[j]), gu, a[vjp_slot(D, i, j)]);
        }
      }
    }
    // fold the fiber's sums with the weights that are constant along it
    tot[0] = cadd(tot[0], a[0]);
    tot[1] = cadd(tot[1], a[1]);
    tot[vjp_slot(D, 0, 0)] = cadd(tot[vjp_slot(D, 0, 0)], a[vjp_slot(D, 0, 0)]);
#pragma unroll
    for (int j = 1; j < D; ++j) tot[vjp_slot(D, 0, j)] = crfma(sq[r[j]], a[vjp_slot(D, 0, j)], tot[vjp_slot(D, 0, j)]);
#pragma unroll
    for (int i = 1; i < D; ++i) {
      tot[1 + i] = crfma(sq[r[i]], a[1 + i], tot[1 + i]);
      tot[vjp_slot(D, i, i)] = crfma(hh[r[i]], a[vjp_slot(D, i, i)], tot[vjp_slot(D, i, i)]);
#pragma unroll
      for (int j = i + 1; j < D; ++j)
        tot[vjp_slot(D, i, j)] = crfma(sq[r[i]] * sq[r[j]], a[vjp_slot(D, i, j)], tot[vjp_slot(D, i, j)]);
    }
  }
}

// Deterministic CTA reduction of NV complex values (fixed shuffle tree, then
// warps in order); thread 0..NV-1 end up writing out[s].
template <int NV>
__device__ __forceinline__ void block_reduce_write(double2 (&tot)[NV], double2* out) {
  typedef double2 RedT[MM_BLOCK / 32][MM_NV_MAX];
  MM_SHARED(RedT, red);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int s = 0; s < NV; ++s) {
    double x = tot[s].x, y = tot[s].y;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      x += __shfl_xor_sync(0xffffffffu, x, o);
      y += __shfl_xor_sync(0xffffffffu, y, o);
    }
    if (lane == 0) red[warp][s] = cmk(x, y);
  }
  __syncthreads();
  const int nw = blockDim.x >> 5;
  for (int s = threadIdx.x; s < NV; s += blockDim.x) {
    double2 acc = red[0][s];
    for (int w = 1; w < nw; ++w) acc = cadd(acc, red[w][s]);
    out[s] = acc;
  }
}

// One CTA per work item; partial sums to partials[item * MM_NV_MAX + slot].
template <int DLO, int DHI, class Src, bool COPY = false>
__global__ void __launch_bounds__(MM_BLOCK) vjp_items_kernel(Src src, Tables T, double2* __restrict__ partials,
                                                             int64_t item_base) {
  MM_SHARED(InstView, sv);
  MM_SHARED(uint32_t, sq0);
  MM_SHARED(uint32_t, sq1);
  MM_SHARED(double2*, sgo);
  const int64_t item = item_base + blockIdx.x;
  if (threadIdx.x == 0) {
    int64_t k;
    uint32_t q0, q1;
    src.item(item, k, q0, q1);
    src.load(k, sv);
    sq0 = q0;
    sq1 = q1;
    sgo = COPY ? src.gout_of(k) : nullptr;  // null also when the forward made this instance's copy
  }
  __syncthreads();
  const int D = sv.g.D;
  double2* out = partials + item * MM_NV_MAX;
#define MM_VJP_CASE(DD)                                       \
  if constexpr (DLO <= DD && DD <= DHI) {                     \
    if (D == DD) {                                            \
      double2 tot[vjp_nv(DD)];                                \
      for (int s = 0; s < vjp_nv(DD); ++s) tot[s] = cmk(0, 0); \
      if (COPY && sgo) vjp_fibers<DD, COPY, COPY>(sv, T, sq0, sq1, tot, sgo); \
      else vjp_fibers<DD, false, COPY>(sv, T, sq0, sq1, tot); \
      block_reduce_write<vjp_nv(DD)>(tot, out);               \
      return;                                                 \
    }                                                         \
  }
  MM_VJP_CASE(1)
  MM_VJP_CASE(2)
  MM_VJP_CASE(3)
  MM_VJP_CASE(4)
  MM_VJP_CASE(5)
  MM_VJP_CASE(6)
  MM_VJP_CASE(7)
  MM_VJP_CASE(8)
#undef MM_VJP_CASE
}

// One warp per instance: sum its items' partials in item order, then write
// dA (symmetrised as (X + X^T)/2, gradients.py:82), db, dc = sum(G dLdG) / c.
template <class Src>
__global__ void __launch_bounds__(128) vjp_reduce_kernel(Src src, const double2* __restrict__ partials,
                                                         double2* __restrict__ dA, double2* __restrict__ db,
                                                         double2* __restrict__ dc) {
  const int warps = blockDim.x >> 5;
  const int64_t k = (int64_t)blockIdx.x * warps + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (k >= src.n_inst()) return;
  const Geom& g = src.geom(k);
  const int D = g.D;
  const int NV = vjp_nv(D);
  int64_t it0, nit;
  src.items_of(k, it0, nit);
  double2* dAk = dA + src.a_off(k);
  double2* dbk = db + src.b_off(k);
  for (int s = lane; s < NV; s += 32) {
    double2 acc = cmk(0.0, 0.0);
    for (int64_t it = 0; it < nit; ++it) acc = cadd(acc, partials[(it0 + it) * MM_NV_MAX + s]);
    if (s == 0) {
      dc[k] = cdiv_smith(acc, __ldg(src.c + k));
    } else if (s <= D) {
      dbk[s - 1] = acc;
    } else {
      // locate (i, j) of slot s
      int i = 0, base = 1 + D;
      while (s >= base + (D - i)) {
        base += D - i;
        ++i;
      }
      const int j = i + (s - base);
      if (i == j) {
        dAk[i * D + i] = acc;
      } else {
        const double2 half = cmk(acc.x / 2.0, acc.y / 2.0);
        dAk[i * D + j] = half;
        dAk[j * D + i] = half;
      }
    }
  }
}

// ============================================================== checkpointed VJP
// Backward pass that never holds all of G (the forward keeps only checkpoint
// slabs; reference: vanilla_vjp_numba, gradients.py:25-82, whose stencil
// reads G only at u, u - 1_i, u - 1_i - 1_j, u - 2_i).  Slab m of level 0 (all
// amplitudes with k_0 = m, a contiguous run of strides[0] amplitudes) depends
// only on slabs m - 1 and m - 2, so segment [s, e) of slabs is recomputed into
// a window buffer from the checkpointed slabs s - 2, s - 1 and the VJP stencil
// then runs over the segment's slabs reading G from the window.
//
// Window: slot t holds slab wbase + t.  One launch per slab; one thread per
// amplitude q of the slab; the arithmetic is fwd_chunk's at level 0.
template <int D>
__global__ void __launch_bounds__(256) fwd_slab_kernel(Geom g, const double2* __restrict__ b,
                                                       const double2* __restrict__ coef,
                                                       const double* __restrict__ rs, double2* __restrict__ W,
                                                       int m, int wbase) {
  const int64_t s0 = g.strides[0];
  const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= s0 || m < 1 || m - 1 < wbase) return;
  const double2 b0 = __ldg(b);
  const double2 cd = (m >= 2) ? __ldg(coef + g.prefC[0] + m) : cmk(0.0, 0.0);
  const double rsm = rs[m];
  const double2* Gp = W + (int64_t)(m - 1 - wbase) * s0;
  int32_t k[D];
  decompose<D>((uint32_t)q, 1, g, k);
  double2 acc = cmul(b0, __ldcg(Gp + q));
  if (m >= 2) acc = cfma(cd, __ldcg(Gp - s0 + q), acc);
#pragma unroll
  for (int j = 1; j < D; ++j)
    if (k[j] > 0) acc = cfma(__ldg(coef + g.prefC[j] + k[j]), __ldcg(Gp + q - g.strides[j]), acc);
  W[(int64_t)(m - wbase) * s0 + q] = cscale(rsm, acc);
}

// vjp_fibers over the slabs m in [m_lo, m_hi) only, G read from the window
// (slab m at W + (m - wbase) * strides[0]); the cotangent is the full tensor.
// Same terms and weights as vjp_fibers; per fiber the sum over m is split at the
// segment boundaries, so results agree with the full-G VJP to rounding.
template <int D>
__device__ __forceinline__ void vjp_fibers_window(const InstView& v, const Tables& T, uint32_t q0, uint32_t q1,
                                                  int m_lo, int m_hi, int wbase, double2 (&tot)[vjp_nv(D)]) {
  constexpr int NV = vjp_nv(D);
  const Geom& g = v.g;
  const int64_t s0 = g.strides[0];
  int64_t sj[D];
#pragma unroll
  for (int j = 0; j < D; ++j) sj[j] = g.strides[j];
  const double2* __restrict__ G = v.G;  // the window
  const double2* __restrict__ gb = v.dLdG;
  const double* __restrict__ sq = T.sq;
  const double* __restrict__ hh = T.hh;
  for (uint32_t q = q0 + threadIdx.x; q < q1; q += blockDim.x) {
    int32_t r[D];
    decompose<D>(q, 1, g, r);
    double2 a[NV];
#pragma unroll
    for (int s = 0; s < NV; ++s) a[s] = cmk(0.0, 0.0);
    for (int m = m_lo; m < m_hi; ++m) {
      const int64_t f = (int64_t)m * s0 + q;          // index in the full tensor (cotangent)
      const int64_t w = (int64_t)(m - wbase) * s0 + q;  // index in the window
      const double2 gu = __ldg(gb + f);
      const double2 gf = __ldg(G + w);
      a[0] = cfma(gf, gu, a[0]);
      if (m >= 1) {
        const double2 h0 = cscale(sq[m], gu);
        a[1] = cfma(__ldg(G + w - s0), h0, a[1]);
#pragma unroll
        for (int j = 1; j < D; ++j)
          if (r[j] >= 1) a[vjp_slot(D, 0, j)] = cfma(__ldg(G + w - s0 - sj[j]), h0, a[vjp_slot(D, 0, j)]);
        if (m >= 2) {
          const double2 h00 = cscale(hh[m], gu);
          a[vjp_slot(D, 0, 0)] = cfma(__ldg(G + w - 2 * s0), h00, a[vjp_slot(D, 0, 0)]);
        }
      }
#pragma unroll
      for (int i = 1; i < D; ++i) {
        if (r[i] >= 1) {
          a[1 + i] = cfma(__ldg(G + w - sj[i]), gu, a[1 + i]);
          if (r[i] >= 2) a[vjp_slot(D, i, i)] = cfma(__ldg(G + w - 2 * sj[i]), gu, a[vjp_slot(D, i, i)]);
#pragma unroll
          for (int j = i + 1; j < D; ++j)
            if (r[j] >= 1) a[vjp_slot(D, i, j)] = cfma(__ldg(G + w - sj[i] - sj[j]), gu, a[vjp_slot(D, i, j)]);
        }
      }
    }
    tot[0] = cadd(tot[0], a[0]);
    tot[1] = cadd(tot[1], a[1]);
    tot[vjp_slot(D, 0, 0)] = cadd(tot[vjp_slot(D, 0, 0)], a[vjp_slot(D, 0, 0)]);
#pragma unroll
    for (int j = 1; j < D; ++j) tot[vjp_slot(D, 0, j)] = crfma(sq[r[j]], a[vjp_slot(D, 0, j)], tot[vjp_slot(D, 0, j)]);
#pragma unroll
    for (int i = 1; i < D; ++i) {
      tot[1 + i] = crfma(sq[r[i]], a[1 + i], tot[1 + i]);
      tot[vjp_slot(D, i, i)] = crfma(hh[r[i]], a[vjp_slot(D, i, i)], tot[vjp_slot(D, i, i)]);
#pragma unroll
      for (int j = i + 1; j < D; ++j)
        tot[vjp_slot(D, i, j)] = crfma(sq[r[i]] * sq[r[j]], a[vjp_slot(D, i, j)], tot[vjp_slot(D, i, j)]);
    }
  }
}

// One CTA per work item of one segment (src: one instance, G = the window);
// partial sums to partials[item * MM_NV_MAX + slot].
template <int D>
__global__ void __launch_bounds__(MM_BLOCK) vjp_window_kernel(UniformSrc src, Tables T, double2* __restrict__ partials,
                                                              int m_lo, int m_hi, int wbase) {
  MM_SHARED(InstView, sv);
  MM_SHARED(uint32_t, sq0);
  MM_SHARED(uint32_t, sq1);
  const int64_t item = blockIdx.x;
  if (threadIdx.x == 0) {
    int64_t k;
    uint32_t q0, q1;
    src.item(item, k, q0, q1);
    src.load(k, sv);
    sq0 = q0;
    sq1 = q1;
  }
  __syncthreads();
  double2 tot[vjp_nv(D)];
#pragma unroll
  for (int s = 0; s < vjp_nv(D); ++s) tot[s] = cmk(0.0, 0.0);
  vjp_fibers_window<D>(sv, T, sq0, sq1, m_lo, m_hi, wbase, tot);
  block_reduce_write<vjp_nv(D)>(tot, partials + item * MM_NV_MAX);
}

}  // namespace mm
