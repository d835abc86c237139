// Diagonal strategies of the Fock recurrence: photon-number (PNR) probabilities and
// leftover-mode density matrices without filling the whole tensor.
//
// 1. compactFock diagonal amplitudes (mrmustard/math/lattice/strategies/compactFock/
//    diagonal_amps.py:17-248), called by math.hermite_renormalized_diagonal
//    (backend_manager.py:729-757 -> backend_numpy.py:423-432 / backend_jax.py:513-522).
//    For M modes with cutoffs c_k the recurrence walks the params lattice (a, b, ...)
//    in order of a + b + ...; at each point a "diagonal pivot" fills the 2M
//    neighbours [a+1,a,...] / [a,a+1,...] / ... (array arr1) and "off-diagonal
//    pivots" fill arr0 (the diagonal G[a,a,b,b,...]), arr2, arr1010, arr1001.
//    Points of equal weight are independent, so the kernel runs one weight per
//    step of a cooperative grid, one thread per (point, output row, batch column);
//    an off-diagonal row recomputes the diagonal-pivot value of its own point that
//    it reads (the same expression on the same inputs), so a weight needs one grid
//    barrier.  Storage: the reference's five arrays back to back in one buffer of
//    "slots" (slot 0 = arr0, then arr2[d], arr1010[d][e], arr1001[d][e], arr1[i]),
//    each P x nb values (P = prod c_k, params in C order, batch index last).
// 2. their Jacobians (compactFock/diagonal_grad.py:17-378): the same schedule with
//    one thread per (point, output row, component of d/dA (2M x 2M) and d/dB (2M)).
// 3. fast_diagonal (mrmustard/math/lattice/strategies/fast_diagonal.py:32-200), which
//    backend_numpy.hermite_renormalized_1leftoverMode calls: the recurrence on the
//    detected modes' near-diagonal lattice (pairs |a - b| <= 2, at most one pair at
//    distance 2), every lattice point an (oc+1) x (oc+1) block of mode 0.  Points are
//    stored densely over per-pair states a*5 + (a - b + 2); one thread per (point,
//    block element), one grid barrier per weight.
//
// Points are ordered by weight on the device (counting sort), so every entry point
// is a fixed sequence of launches without host copies (capturable in a CUDA graph).
// Arithmetic is FP64 with fused multiply-adds; parity with the reference is to
// rounding (the reference's own row products are BLAS dots).
#include <algorithm>
#include <cstdint>
#include <cstring>
#include <vector>

#include "common.cuh"

using namespace mm;

namespace {

constexpr int DG_MAXM = 8;          // modes of the diagonal strategy
constexpr int FD_MAXK = 7;          // detected modes of fast_diagonal (L <= 8)
constexpr int DG_BLOCK = 128;       // threads per CTA of the wavefront kernels
constexpr int SORT_BLOCK = 256;
constexpr int kMaxWeights = 1 << 16;
constexpr size_t kWsAlign = 256;

size_t al(size_t x) { return (x + kWsAlign - 1) / kWsAlign * kWsAlign; }

#ifndef MM_HOST_EMULATION
int cuda_status() { return cudaGetLastError() == cudaSuccess ? MM_OK : MM_ERR_CUDA; }
#endif

uint64_t budget_ns() {
  const char* s = getenv("MM_WAIT_BUDGET_NS");
  return s ? strtoull(s, nullptr, 10) : 2000000000ull;
}

// ------------------------------------------------------------------ lattices

struct DiagLat {
  int M;
  int n;  // 2M
  int32_t c[DG_MAXM];
  int32_t st[DG_MAXM];
  int32_t P;
  int32_t nb;
  int32_t W;  // number of weights: sum(c - 1) + 1
};

__host__ __device__ __forceinline__ int64_t slot_arr2(const DiagLat& L, int d) { return 1 + d; }
__host__ __device__ __forceinline__ int64_t slot_1010(const DiagLat& L, int d, int e) {
  return 1 + L.M + (int64_t)d * (L.M - 1) + e;
}
__host__ __device__ __forceinline__ int64_t slot_1001(const DiagLat& L, int d, int e) {
  return 1 + L.M + (int64_t)L.M * (L.M - 1) + (int64_t)d * (L.M - 1) + e;
}
__host__ __device__ __forceinline__ int64_t slot_arr1(const DiagLat& L, int i) {
  return 1 + L.M + 2 * (int64_t)L.M * (L.M - 1) + i;
}
__host__ __device__ __forceinline__ int64_t diag_slots(int M) { return 1 + M + 2 * (int64_t)M * (M - 1) + 2 * M; }

__device__ __forceinline__ int diag_weight(const DiagLat& L, int32_t f, int32_t* p) {
  int w = 0;
  for (int k = 0; k < L.M; ++k) {
    p[k] = f / L.st[k];
    f -= p[k] * L.st[k];
    w += p[k];
  }
  return w;
}

struct FdLat {
  int K;  // detected modes (pairs)
  int q;  // oc + 1
  int32_t pnr[FD_MAXK];
  int32_t rad[FD_MAXK];  // 5 (pnr + 1)
  int32_t pst[FD_MAXK];  // mixed-radix strides of the dense point id
  int32_t npts;
  int32_t ost[FD_MAXK];  // strides of the output's leading (pnr + 1) axes
  int32_t W;             // number of weights of the lattice: 2 sum(pnr) + 1
  int32_t wend;          // the reference's loop bound: weights 1 .. wend - 1 are filled
};

// coordinates of a dense id: returns the weight, or -1 when the id is not a lattice point
__device__ __forceinline__ int fd_decode(const FdLat& F, int32_t id, int32_t* k) {
  int n2 = 0, w = 0;
  for (int j = 0; j < F.K; ++j) {
    const int32_t s = (id / F.pst[j]) % F.rad[j];
    const int32_t a = s / 5, dl = s % 5 - 2, b = a - dl;
    if (b < 0 || b > F.pnr[j]) return -1;
    n2 += (dl == 2 || dl == -2);
    k[2 * j] = a;
    k[2 * j + 1] = b;
    w += a + b;
  }
  return n2 <= 1 ? w : -1;
}

// ------------------------------------------------------------------ weight sort
// Counting sort of the lattice points by weight: histogram, scan, scatter.  The
// order inside one weight depends on atomics and does not matter (the points of one
// weight are independent).

struct SortBufs {
  int32_t* count;   // W
  int32_t* start;   // W + 1
  int32_t* cursor;  // W
  int32_t* order;   // points
};

template <class Lat>
__device__ __forceinline__ int point_weight(const Lat& L, int32_t id);
template <>
__device__ __forceinline__ int point_weight<DiagLat>(const DiagLat& L, int32_t id) {
  int32_t p[DG_MAXM];
  return diag_weight(L, id, p);
}
template <>
__device__ __forceinline__ int point_weight<FdLat>(const FdLat& F, int32_t id) {
  int32_t k[2 * FD_MAXK];
  return fd_decode(F, id, k);
}

template <class Lat>
__global__ void sort_count_kernel(Lat L, int32_t n, SortBufs sb) {
  for (int32_t id = blockIdx.x * blockDim.x + threadIdx.x; id < n; id += gridDim.x * blockDim.x) {
    const int w = point_weight(L, id);
    if (w >= 0) atomicAdd(&sb.count[w], 1);
  }
}

__global__ void sort_scan_kernel(int32_t W, SortBufs sb) {
  // one CTA: a serial scan in chunks by thread 0 is enough for W <= 65536
  if (threadIdx.x == 0) {
    int32_t acc = 0;
    for (int32_t w = 0; w < W; ++w) {
      sb.start[w] = acc;
      sb.cursor[w] = acc;
      acc += sb.count[w];
    }
    sb.start[W] = acc;
  }
}

template <class Lat>
__global__ void sort_scatter_kernel(Lat L, int32_t n, SortBufs sb) {
  for (int32_t id = blockIdx.x * blockDim.x + threadIdx.x; id < n; id += gridDim.x * blockDim.x) {
    const int w = point_weight(L, id);
    if (w >= 0) sb.order[atomicAdd(&sb.cursor[w], 1)] = id;
  }
}

#ifndef MM_HOST_EMULATION  // the host emulation of the kernels runs them without the launch code below
template <class Lat>
int launch_sort(const Lat& L, int32_t n, int32_t W, const SortBufs& sb, int sms, cudaStream_t st) {
  if (cudaMemsetAsync(sb.count, 0, (size_t)W * sizeof(int32_t), st) != cudaSuccess) return MM_ERR_CUDA;
  const unsigned blocks = (unsigned)std::max<int64_t>(1, std::min<int64_t>((n + SORT_BLOCK - 1) / SORT_BLOCK, 4 * sms));
  sort_count_kernel<Lat><<<blocks, SORT_BLOCK, 0, st>>>(L, n, sb);
  sort_scan_kernel<<<1, 32, 0, st>>>(W, sb);
  sort_scatter_kernel<Lat><<<blocks, SORT_BLOCK, 0, st>>>(L, n, sb);
  note_launches(3);
  return cuda_status();
}
#endif

// ------------------------------------------------------------------ grid step barrier
__device__ __forceinline__ bool step_barrier(WsHeader* h, uint32_t& epoch, uint64_t budget) {
  if (gridDim.x == 1) {
    __syncthreads();
    return true;
  }
  return grid_barrier(h, ++epoch, budget, 0);
}

// ------------------------------------------------------------------ square-root tables
// sq[k] = sqrt(k) (correctly rounded, as the reference's SQRT tables) and rs[k] = 1/sqrt(k),
// filled once per call: FP64 square roots and divisions are multi-instruction FP64
// sequences, far too costly to repeat per amplitude on this part.
struct Tabs {
  const double* sq;
  const double* rs;
};

// Per-CTA copies of the read-only operands of a wavefront kernel: the square-root tables
// (when they fit) and the 2M x 2M matrix, so that the per-item reads are shared-memory hits.
constexpr int kSmemTab = 1024;
constexpr int kSmemA = 16 * 16;
struct StageSmem {
  double sq[kSmemTab];
  double rs[kSmemTab];
  double2 A[kSmemA];
  double2 b[16];
};

// Copies tables (first ntab entries) and the n x n matrix A (and the n-vector b when given)
// into shared memory; returns the staged views.
__device__ __forceinline__ void stage_operands(StageSmem& sm, Tabs& t, int32_t ntab, const double2*& A, int n,
                                               const double2** b) {
  if (ntab <= kSmemTab) {
    for (int k = threadIdx.x; k < ntab; k += blockDim.x) {
      sm.sq[k] = t.sq[k];
      sm.rs[k] = t.rs[k];
    }
    t.sq = sm.sq;
    t.rs = sm.rs;
  }
  for (int k = threadIdx.x; k < n * n; k += blockDim.x) sm.A[k] = A[k];
  A = sm.A;
  if (b) {
    for (int k = threadIdx.x; k < n; k += blockDim.x) sm.b[k] = (*b)[k];
    *b = sm.b;
  }
  __syncthreads();
}

__global__ void sqrt_table_kernel(double* sq, double* rs, int32_t n) {
  for (int32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
    const double s = sqrt((double)k);
    sq[k] = s;
    rs[k] = k > 0 ? 1.0 / s : 0.0;
  }
}

// ------------------------------------------------------------------ 1. diagonal amplitudes

struct DiagArgs {
  DiagLat L;
  const double2* A;   // 2M x 2M, interleaved mode order
  const double2* B;   // 2M x nb
  const double2* G0;  // nb
  double2* Wv;        // slots x P x nb
  double2* J;         // Jacobians: slots x P x (4M^2 + 2M) (Jacobian kernel only)
  Tabs t;
  int32_t ntab;
  SortBufs sb;
  WsHeader* h;
  uint64_t budget;
};

__device__ __forceinline__ double2 ldv(const double2* p) { return __ldcg(p); }

template <int M>
__device__ __forceinline__ void decode_params(const DiagLat& L, int32_t f, int32_t* p) {
#pragma unroll
  for (int k = 0; k < M; ++k) {
    p[k] = f / L.st[k];
    f -= p[k] * L.st[k];
  }
}

// Row i of the diagonal pivot at point f (diagonal_amps.py:92-137):
// (arr0[p] B_i + sum_l A_il sqrt(p_{l/2}) arr1[l^1][p - 1_{l/2}]) / sqrt(p_{i/2} + 1).
template <int M>
__device__ __forceinline__ double2 diag_row(const DiagArgs& a, const int32_t* p, int32_t f, int i, int32_t col) {
  constexpr int n = 2 * M;
  const DiagLat& L = a.L;
  const int64_t PN = (int64_t)L.P * L.nb;
  double2 gin[n];
#pragma unroll
  for (int l = 0; l < n; ++l) {
    const int k = l >> 1;
    gin[l] = p[k] > 0 ? ldv(&a.Wv[slot_arr1(L, l ^ 1) * PN + (int64_t)(f - L.st[k]) * L.nb + col]) : cmk(0.0, 0.0);
  }
  double2 acc = cmul(ldv(&a.Wv[(int64_t)f * L.nb + col]), __ldg(&a.B[(int64_t)i * L.nb + col]));
#pragma unroll
  for (int l = 0; l < n; ++l) acc = cfma(a.A[i * n + l], cscale(a.t.sq[p[l >> 1]], gin[l]), acc);
  return cscale(a.t.rs[p[i >> 1] + 1], acc);
}

// Output row `row` of the off-diagonal pivot d at point f (diagonal_amps.py:17-89),
// with g = arr1[2d][f] (the diagonal pivot's row 2d at the same point).
template <int M>
__device__ __forceinline__ double2 offdiag_row(const DiagArgs& a, const int32_t* p, int32_t f, int d, int row,
                                               double2 g, int32_t col) {
  constexpr int n = 2 * M;
  const DiagLat& L = a.L;
  const int64_t PN = (int64_t)L.P * L.nb;
  double2 gin[n];
  double kl[n];
#pragma unroll
  for (int i = 0; i < M; ++i) {
    gin[2 * i] = cmk(0.0, 0.0);
    gin[2 * i + 1] = cmk(0.0, 0.0);
    kl[2 * i] = a.t.sq[p[i]];
    kl[2 * i + 1] = kl[2 * i];
    if (i < d) continue;
    if (i == d) {  // G_in[2d] = arr0[p] with K_l = sqrt(p_d + 1); G_in[2d+1] = arr2[d][p - 1_d]
      kl[2 * i] = a.t.sq[p[i] + 1];
      gin[2 * i] = ldv(&a.Wv[(int64_t)f * L.nb + col]);
      if (p[i] > 0) gin[2 * i + 1] = ldv(&a.Wv[slot_arr2(L, d) * PN + (int64_t)(f - L.st[i]) * L.nb + col]);
    } else if (p[i] > 0) {
      const int64_t o = (int64_t)(f - L.st[i]) * L.nb + col;
      gin[2 * i] = ldv(&a.Wv[slot_1001(L, d, i - d - 1) * PN + o]);
      gin[2 * i + 1] = ldv(&a.Wv[slot_1010(L, d, i - d - 1) * PN + o]);
    }
  }
  double2 acc = cmul(g, __ldg(&a.B[(int64_t)row * L.nb + col]));
#pragma unroll
  for (int l = 0; l < n; ++l)
    if ((l >> 1) >= d) acc = cfma(a.A[row * n + l], cscale(kl[l], gin[l]), acc);
  const int k = row >> 1;
  const int lift = (row & 1) == 0 && k == d;  // K_i[2d] = sqrt(p_d + 2)
  return cscale(a.t.rs[p[k] + lift + 1], acc);
}

// Target of local row r of the off-diagonal pivot d (r = 0: arr0[p + 1_d]; r = 1: arr2[d];
// r >= 2: arr1010 / arr1001 of mode d + 1 + (r - 2) / 2).  False when the reference writes nothing.
__device__ __forceinline__ bool offdiag_target(const DiagLat& L, const int32_t* p, int d, int r, int& row,
                                               int64_t& slot, int32_t& dst, int32_t f) {
  if (!(p[d] < L.c[d] - 1) || r >= L.n - 2 * d) return false;
  if (r == 0) {
    row = 2 * d + 1;
    slot = 0;
    dst = f + L.st[d];
    return true;
  }
  dst = f;
  if (r == 1) {
    if (!(p[d] + 2 < L.c[d])) return false;
    row = 2 * d;
    slot = slot_arr2(L, d);
    return true;
  }
  const int i = d + 1 + (r - 2) / 2;
  if (!(p[i] + 1 < L.c[i])) return false;
  row = 2 * i + ((r - 2) & 1);
  slot = (row & 1) ? slot_1001(L, d, i - d - 1) : slot_1010(L, d, i - d - 1);
  return true;
}

__device__ __forceinline__ bool diag_target(const DiagLat& L, const int32_t* p, int i) {
  return (L.c[0] == 1 || p[0] < L.c[0] - 1) && p[i >> 1] + 1 < L.c[i >> 1] && (i != 1 || p[0] + 2 < L.c[0]);
}

// The off-diagonal pivots d of a point are 0 .. (index of its first non-zero coordinate).
template <int M>
__device__ __forceinline__ int last_pivot(const int32_t* p) {
  int fz = M - 1;
#pragma unroll
  for (int k = M - 1; k >= 0; --k)
    if (p[k] != 0) fz = k;
  return fz;
}

// Items of one weight: (slot r, point, column), column fastest, then point, so that the
// lanes of a warp run the same row of neighbouring points (or columns).  Slots 0 .. 2M-1
// are the diagonal-pivot rows; slots 2M .. 4M-1 the off-diagonal rows r - 2M of every pivot d.
template <int M>
__global__ void __launch_bounds__(DG_BLOCK) diag_amps_kernel(DiagArgs a) {
  constexpr int n = 2 * M;
  MM_SHARED(StageSmem, sm);
  stage_operands(sm, a.t, a.ntab, a.A, n, nullptr);
  const DiagLat& L = a.L;
  const int64_t PN = (int64_t)L.P * L.nb;
  const int64_t t0 = (int64_t)blockIdx.x * blockDim.x + threadIdx.x, stride = (int64_t)gridDim.x * blockDim.x;
  // The point of this thread's first item of the next weight is read before the barrier
  // (the order is fixed), taking two dependent loads off the path after it.
  auto first_point = [&](int w, int32_t& s0, int32_t& cnt) -> int32_t {
    s0 = a.sb.start[w];
    cnt = a.sb.start[w + 1] - s0;
    const int64_t per_slot = (int64_t)cnt * L.nb;
    if (t0 >= per_slot * 2 * n) return -1;
    const int64_t u = t0 - (t0 / per_slot) * per_slot;
    return a.sb.order[s0 + (int32_t)(u / L.nb)];
  };
  int32_t s0, cnt;
  int32_t fnext = first_point(0, s0, cnt);
  uint32_t epoch = 0;
  for (int w = 0; w < L.W; ++w) {
    const int64_t per_slot = (int64_t)cnt * L.nb;
    const int64_t items = per_slot * 2 * n;
    for (int64_t t = t0; t < items; t += stride) {
      const int r = (int)(t / per_slot);
      const int64_t u = t - r * per_slot;
      const int32_t pidx = (int32_t)(u / L.nb);
      const int32_t col = (int32_t)(u - (int64_t)pidx * L.nb);
      const int32_t f = t == t0 ? fnext : a.sb.order[s0 + pidx];
      int32_t p[M];
      decode_params<M>(L, f, p);
      if (r < n) {
        if (diag_target(L, p, r)) a.Wv[slot_arr1(L, r) * PN + (int64_t)f * L.nb + col] = diag_row<M>(a, p, f, r, col);
        continue;
      }
      const int lr = r - n, dl = last_pivot<M>(p);
      for (int d = 0; d <= dl; ++d) {
        int row;
        int64_t slot;
        int32_t dst;
        if (!offdiag_target(L, p, d, lr, row, slot, dst, f)) continue;
        const double2 g = diag_row<M>(a, p, f, 2 * d, col);
        a.Wv[slot * PN + (int64_t)dst * L.nb + col] = offdiag_row<M>(a, p, f, d, row, g, col);
      }
    }
    if (w + 1 < L.W) fnext = first_point(w + 1, s0, cnt);
    if (!step_barrier(a.h, epoch, a.budget)) return;
  }
}

__global__ void diag_init_kernel(DiagArgs a) {
  for (int32_t col = threadIdx.x; col < a.L.nb; col += blockDim.x) a.Wv[col] = a.G0[col];
}

// ------------------------------------------------------------------ 2. Jacobians
// calc_dA_dB (diagonal_grad.py:17-41): for output row i with pivot value g, pivot
// Jacobian Jp and inputs (K_l Gin_l, J_l):
//   d/dA_pq = (Jp_pq B_i + sum_l K_l A_il J_l,pq + [p == i] K_q Gin_q) / K_i
//   d/dB_r  = (Jp_r  B_i + [r == i] g + sum_l K_l A_il J_l,r) / K_i

template <int M>
__device__ __forceinline__ double2 jac_diag_row(const DiagArgs& a, const int32_t* p, int32_t f, int i, int q) {
  constexpr int n = 2 * M, nc = n * n + n;
  const DiagLat& L = a.L;
  const int64_t P = L.P;
  const bool isA = q < n * n;
  const int qa = q / n, qb = q - qa * n;  // (row, column) of a dA component
  double2 jin[n];
#pragma unroll
  for (int l = 0; l < n; ++l)
    jin[l] = p[l >> 1] > 0 ? ldv(&a.J[(slot_arr1(L, l ^ 1) * P + (f - L.st[l >> 1])) * nc + q]) : cmk(0.0, 0.0);
  double2 acc = cmul(ldv(&a.J[(int64_t)f * nc + q]), __ldg(&a.B[i]));
  if (!isA && q - n * n == i) acc = cadd(acc, ldv(&a.Wv[f]));
#pragma unroll
  for (int l = 0; l < n; ++l) acc = cfma(cscale(a.t.sq[p[l >> 1]], a.A[i * n + l]), jin[l], acc);
  if (isA && qa == i && p[qb >> 1] > 0)
    acc = cadd(acc, cscale(a.t.sq[p[qb >> 1]], ldv(&a.Wv[slot_arr1(L, qb ^ 1) * P + (f - L.st[qb >> 1])])));
  return cscale(a.t.rs[p[i >> 1] + 1], acc);
}

template <int M>
__device__ __forceinline__ double2 jac_offdiag_row(const DiagArgs& a, const int32_t* p, int32_t f, int d, int row,
                                                   double2 Jp, int q) {
  constexpr int n = 2 * M, nc = n * n + n;
  const DiagLat& L = a.L;
  const int64_t P = L.P;
  const bool isA = q < n * n;
  const int qa = q / n, qb = q - qa * n;
  int64_t src[n];
  double kl[n];
#pragma unroll
  for (int i = 0; i < M; ++i) {
    src[2 * i] = -1;
    src[2 * i + 1] = -1;
    kl[2 * i] = a.t.sq[p[i]];
    kl[2 * i + 1] = kl[2 * i];
    if (i < d) continue;
    if (i == d) {
      kl[2 * i] = a.t.sq[p[i] + 1];
      src[2 * i] = f;
      if (p[i] > 0) src[2 * i + 1] = slot_arr2(L, d) * P + (f - L.st[i]);
    } else if (p[i] > 0) {
      src[2 * i] = slot_1001(L, d, i - d - 1) * P + (f - L.st[i]);
      src[2 * i + 1] = slot_1010(L, d, i - d - 1) * P + (f - L.st[i]);
    }
  }
  double2 jin[n];
#pragma unroll
  for (int l = 0; l < n; ++l) jin[l] = src[l] >= 0 ? ldv(&a.J[src[l] * nc + q]) : cmk(0.0, 0.0);
  double2 acc = cmul(Jp, __ldg(&a.B[row]));
  if (!isA && q - n * n == row) acc = cadd(acc, ldv(&a.Wv[slot_arr1(L, 2 * d) * P + f]));
#pragma unroll
  for (int l = 0; l < n; ++l) acc = cfma(cscale(kl[l], a.A[row * n + l]), jin[l], acc);
  if (isA && qa == row && src[qb] >= 0) acc = cadd(acc, cscale(kl[qb], ldv(&a.Wv[src[qb]])));
  const int k = row >> 1;
  const int lift = (row & 1) == 0 && k == d;
  return cscale(a.t.rs[p[k] + lift + 1], acc);
}

// Items of one weight: (slot r, point, component q), q fastest (coalesced Jacobian rows).
template <int M>
__global__ void __launch_bounds__(DG_BLOCK) diag_jacobian_kernel(DiagArgs a) {
  constexpr int n = 2 * M, nc = n * n + n;
  MM_SHARED(StageSmem, sm);
  stage_operands(sm, a.t, a.ntab, a.A, n, nullptr);
  const DiagLat& L = a.L;
  const int64_t P = L.P;
  const int64_t t0 = (int64_t)blockIdx.x * blockDim.x + threadIdx.x, stride = (int64_t)gridDim.x * blockDim.x;
  auto first_point = [&](int w, int32_t& s0, int32_t& cnt) -> int32_t {
    s0 = a.sb.start[w];
    cnt = a.sb.start[w + 1] - s0;
    const int64_t per_slot = (int64_t)cnt * nc;
    if (t0 >= per_slot * 2 * n) return -1;
    const int64_t u = t0 - (t0 / per_slot) * per_slot;
    return a.sb.order[s0 + (int32_t)(u / nc)];
  };
  int32_t s0, cnt;
  int32_t fnext = first_point(0, s0, cnt);
  uint32_t epoch = 0;
  for (int w = 0; w < L.W; ++w) {
    const int64_t per_slot = (int64_t)cnt * nc;
    const int64_t items = per_slot * 2 * n;
    for (int64_t t = t0; t < items; t += stride) {
      const int r = (int)(t / per_slot);
      const int64_t u = t - r * per_slot;
      const int32_t pidx = (int32_t)(u / nc);
      const int q = (int)(u - (int64_t)pidx * nc);
      const int32_t f = t == t0 ? fnext : a.sb.order[s0 + pidx];
      int32_t p[M];
      decode_params<M>(L, f, p);
      if (r < n) {
        if (diag_target(L, p, r)) a.J[(slot_arr1(L, r) * P + f) * nc + q] = jac_diag_row<M>(a, p, f, r, q);
        continue;
      }
      const int lr = r - n, dl = last_pivot<M>(p);
      for (int d = 0; d <= dl; ++d) {
        int row;
        int64_t slot;
        int32_t dst;
        if (!offdiag_target(L, p, d, lr, row, slot, dst, f)) continue;
        const double2 Jp = jac_diag_row<M>(a, p, f, 2 * d, q);
        a.J[(slot * P + dst) * nc + q] = jac_offdiag_row<M>(a, p, f, d, row, Jp, q);
      }
    }
    if (w + 1 < L.W) fnext = first_point(w + 1, s0, cnt);
    if (!step_barrier(a.h, epoch, a.budget)) return;
  }
}

// dL/dA_pq = sum_k g_k J0_k,pq ; dL/dB_r = sum_k g_k J0_k,r ; dL/dG0 = sum_k g_k (arr0_k / G0)
// (the contraction of hermite_renormalized_diagonal_jax_bwd, jax_vjps/hermite.py:292-329).
// One CTA per output component, fixed-order reduction.
__global__ void diag_vjp_kernel(DiagLat L, const double2* J, const double2* Wv, const double2* G0, const double2* g,
                                double2* dA, double2* dB, double2* dG0) {
  const int nc = L.n * L.n + L.n;
  const int comp = blockIdx.x;  // 0..nc (nc = dG0)
  double2 acc = cmk(0.0, 0.0);
  const double2 c0 = __ldg(G0);
  for (int32_t k = threadIdx.x; k < L.P; k += blockDim.x) {
    const double2 gk = __ldg(&g[k]);
    const double2 x = comp < nc ? __ldg(&J[(int64_t)k * nc + comp]) : cdiv_smith(__ldg(&Wv[k]), c0);
    acc = cfma(gk, x, acc);
  }
  __shared__ double2 red[256];
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if ((int)threadIdx.x < s) red[threadIdx.x] = cadd(red[threadIdx.x], red[threadIdx.x + s]);
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    if (comp < L.n * L.n)
      dA[comp] = red[0];
    else if (comp < nc)
      dB[comp - L.n * L.n] = red[0];
    else
      *dG0 = red[0];
  }
}

// ------------------------------------------------------------------ 3. fast_diagonal

struct FdArgs {
  FdLat F;
  const double2* A;  // 2L x 2L, caller's order (all first copies, then all second copies)
  const double2* b;
  const double2* c;
  int stable;
  double2* Ap;       // permuted (interleaved) A, 2L x 2L (workspace)
  double2* bp;       // permuted b (workspace)
  double2* G;        // npts x q^2 (workspace)
  double2* out;      // (pnr + 1 ..., q, q)
  Tabs t;
  int32_t ntab;
  SortBufs sb;
  WsHeader* h;
  uint64_t budget;
};

__device__ __forceinline__ int32_t fd_zero_id(const FdLat& F) {
  int32_t id = 0;
  for (int j = 0; j < F.K; ++j) id += 2 * F.pst[j];
  return id;
}

// One CTA: permute A and b (perm = [m, m + L], fast_diagonal.py:56-59) and fill the
// first block, the (q, q) recurrence of mode 0 (vanilla_numba or stable_numba on
// A[:2, :2], b[:2], c; vanilla/core.py:25-213), by anti-diagonals.
__global__ void fd_init_kernel(FdArgs a) {
  const FdLat& F = a.F;
  const int Lm = F.K + 1, n = 2 * Lm, q = F.q;
  const double* sq = a.t.sq;
  const double* rs = a.t.rs;
  for (int t = threadIdx.x; t < n * n; t += blockDim.x) {
    const int r = t / n, s = t % n;
    const int pr = (r & 1) ? (r >> 1) + Lm : (r >> 1), ps = (s & 1) ? (s >> 1) + Lm : (s >> 1);
    a.Ap[t] = a.A[pr * n + ps];
  }
  for (int r = threadIdx.x; r < n; r += blockDim.x) a.bp[r] = a.b[(r & 1) ? (r >> 1) + Lm : (r >> 1)];
  __syncthreads();
  double2* G = a.G + (int64_t)fd_zero_id(F) * q * q;
  const double2 A00 = a.Ap[0], A01 = a.Ap[1], A10 = a.Ap[n], A11 = a.Ap[n + 1], b0 = a.bp[0], b1 = a.bp[1];
  if (threadIdx.x == 0) G[0] = __ldg(a.c);
  __syncthreads();
  auto at = [&](int m, int k) -> double2 { return (m < 0 || k < 0) ? cmk(0.0, 0.0) : G[m * q + k]; };
  for (int s = 1; s <= 2 * (q - 1); ++s) {
    for (int m = max(0, s - (q - 1)) + (int)threadIdx.x; m <= min(s, q - 1); m += blockDim.x) {
      const int k = s - m;
      double2 v;
      if (!a.stable) {
        if (m == 0) {  // face: pivot on axis 1
          double2 acc = cmul(b1, at(0, k - 1));
          acc = cfma(cscale(sq[k - 1], A11), at(0, k - 2), acc);
          v = cscale(rs[k], acc);
        } else {  // bulk: pivot on axis 0
          double2 acc = cmul(b0, at(m - 1, k));
          acc = cfma(cscale(sq[m - 1], A00), at(m - 2, k), acc);
          acc = cfma(cscale(sq[k], A01), at(m - 1, k - 1), acc);
          v = cscale(rs[m], acc);
        }
      } else {  // average over the pivots with k_i > 0
        double2 vals = cmk(0.0, 0.0);
        int npiv = 0;
        if (m > 0) {
          double2 acc = cmul(b0, at(m - 1, k));
          acc = cfma(cscale(sq[m - 1], A00), at(m - 2, k), acc);
          acc = cfma(cscale(sq[k], A01), at(m - 1, k - 1), acc);
          vals = cadd(vals, cscale(rs[m], acc));
          ++npiv;
        }
        if (k > 0) {
          double2 acc = cmul(b1, at(m, k - 1));
          acc = cfma(cscale(sq[m], A10), at(m - 1, k - 1), acc);
          acc = cfma(cscale(sq[k - 1], A11), at(m, k - 2), acc);
          vals = cadd(vals, cscale(rs[k], acc));
          ++npiv;
        }
        v = npiv == 2 ? cscale(0.5, vals) : vals;  // / npiv (exact for 1 and 2)
      }
      G[m * q + k] = v;
    }
    __syncthreads();
  }
  for (int t = threadIdx.x; t < q * q; t += blockDim.x) a.out[t] = G[t];
}

// Items of one weight: (point, block element e), e fastest: the lanes of a warp share the
// point (and its pivot) and read consecutive block elements.
template <int K>
__global__ void __launch_bounds__(DG_BLOCK) fd_kernel(FdArgs a) {
  constexpr int n = 2 * (K + 1);
  MM_SHARED(StageSmem, sm);
  const double2* Ap = a.Ap;
  const double2* bp = a.bp;
  stage_operands(sm, a.t, a.ntab, Ap, n, &bp);
  const FdLat& F = a.F;
  const int q = F.q, qq = q * q;
  const double* sq = a.t.sq;
  const int64_t t0 = (int64_t)blockIdx.x * blockDim.x + threadIdx.x, stride = (int64_t)gridDim.x * blockDim.x;
  auto first_point = [&](int w, int32_t& s0, int32_t& cnt) -> int32_t {
    s0 = a.sb.start[w];
    cnt = a.sb.start[w + 1] - s0;
    if (t0 >= (int64_t)cnt * qq) return -1;
    return a.sb.order[s0 + (int32_t)(t0 / qq)];
  };
  uint32_t epoch = 0;
  const int wlast = min(F.W - 1, F.wend - 1);
  int32_t s0 = 0, cnt = 0, idnext = -1;
  if (wlast >= 1) idnext = first_point(1, s0, cnt);
  for (int w = 1; w <= wlast; ++w) {
    const int64_t items = (int64_t)cnt * qq;
    for (int64_t t = t0; t < items; t += stride) {
      const int32_t pi = (int32_t)(t / qq);
      const int e = (int)(t - (int64_t)pi * qq);
      const int32_t id = t == t0 ? idnext : a.sb.order[s0 + pi];
      const int m = e / q, kk = e - m * q;
      int32_t k[2 * K];
#pragma unroll
      for (int j = 0; j < K; ++j) {
        const int32_t s = (id / F.pst[j]) % F.rad[j];
        k[2 * j] = s / 5;
        k[2 * j + 1] = s / 5 - (s % 5 - 2);
      }
      // get_pivot (fast_diagonal.py:80-99)
      int mbest = 0, dbest = -1;
#pragma unroll
      for (int j = 0; j < K; ++j) {
        const int dl = abs(k[2 * j] - k[2 * j + 1]);
        if (dl > dbest) {
          dbest = dl;
          mbest = j;
        }
      }
      int i;
      if (dbest == 0) {
        i = 0;
#pragma unroll
        for (int j = 1; j < 2 * K; ++j)
          if (k[j] > k[i]) i = j;
      } else {
        i = k[2 * mbest] > k[2 * mbest + 1] ? 2 * mbest : 2 * mbest + 1;
      }
      // pivot id: lowering a (even coordinate) moves the pair state by -6, lowering b by +1
      const int32_t pid = id + ((i & 1) ? 1 : -6) * F.pst[i >> 1];
      int32_t kp[2 * K];
#pragma unroll
      for (int j = 0; j < 2 * K; ++j) kp[j] = k[j] - (j == i);
      const double2* mat = a.G + (int64_t)pid * qq;
      const double2* Arow = Ap + (i + 2) * n;
      double2 low[2 * K];
#pragma unroll
      for (int j = 0; j < 2 * K; ++j)
        low[j] = kp[j] > 0 ? ldv(&a.G[(int64_t)(pid + ((j & 1) ? 1 : -6) * F.pst[j >> 1]) * qq + e]) : cmk(0.0, 0.0);
      // single_step (fast_diagonal.py:102-124)
      double2 acc = cmul(bp[i + 2], ldv(&mat[e]));
      if (m > 0) acc = cfma(cscale(sq[m], Arow[0]), ldv(&mat[e - q]), acc);
      if (kk > 0) acc = cfma(cscale(sq[kk], Arow[1]), ldv(&mat[e - 1]), acc);
#pragma unroll
      for (int j = 0; j < 2 * K; ++j) acc = cfma(cscale(sq[kp[j]], Arow[j + 2]), low[j], acc);
      const double2 v = cscale(a.t.rs[k[i]], acc);
      a.G[(int64_t)id * qq + e] = v;
      bool diag = true;
      int32_t o = 0;
#pragma unroll
      for (int j = 0; j < K; ++j) {
        diag &= k[2 * j] == k[2 * j + 1];
        o += k[2 * j] * F.ost[j];
      }
      if (diag) a.out[(int64_t)o * qq + e] = v;
    }
    if (w + 1 <= wlast) idnext = first_point(w + 1, s0, cnt);
    if (!step_barrier(a.h, epoch, a.budget)) return;
  }
}

// ------------------------------------------------------------------ 4. leftover mode
// compactFock's leftover-mode strategy (compactFock/singleLeftoverMode_amps.py:18-421 and
// singleLeftoverMode_grad.py:18-724): mode 0 is left over, its q x q block is carried by every
// point of the detected modes' params lattice.  Block entry (m, n) of an output row i (full
// index) reads the pivot block at (m, n), (m-1, n), (m, n-1) and the inputs at (m, n):
//   (pivot[m,n] B_i + A_i0 sqrt(m) pivot[m-1,n] + A_i1 sqrt(n) pivot[m,n-1]
//    + sum_l A_i,l+2 K_l G_l[m,n]) / K_i.
// The first block (every detected mode at 0) is a 2-D recurrence filled by one CTA by
// anti-diagonals.  Storage W[slot][m][n][P'] (the diagonal strategy's slots over the detected
// modes), J[slot][m][n][P'][4M^2 + 2M].  Two phases per weight: diagonal pivots, then
// off-diagonal pivots (which read three entries of a diagonal pivot's block).

struct LoArgs {
  DiagLat L;  // detected modes' lattice (M' modes; L.n = 2M')
  int q;      // leftover cutoff
  int N;      // 2M (rows of A)
  const double2* A;
  const double2* B;
  const double2* G0;
  double2* Wv;
  double2* J;
  Tabs t;
  int32_t ntab;
  SortBufs sb;
  WsHeader* h;
  uint64_t budget;
};

__device__ __forceinline__ int64_t lo_at(const LoArgs& a, int64_t slot, int m, int n, int32_t f) {
  return ((slot * a.q + m) * a.q + n) * (int64_t)a.L.P + f;
}

// Block entry (m, n) of full row `row`; gin[l] are the scaled inputs K_l G_l[m, n].
template <int MT>
__device__ __forceinline__ double2 lo_value(const LoArgs& a, int row, int64_t ps, int32_t f, int m, int n,
                                            const double2* gin, double kinv) {
  const double2* W = a.Wv;
  double2 acc = cmul(ldv(&W[lo_at(a, ps, m, n, f)]), a.B[row]);
  if (m > 0) acc = cfma(a.A[row * a.N + 0], cscale(a.t.sq[m], ldv(&W[lo_at(a, ps, m - 1, n, f)])), acc);
  if (n > 0) acc = cfma(a.A[row * a.N + 1], cscale(a.t.sq[n], ldv(&W[lo_at(a, ps, m, n - 1, f)])), acc);
#pragma unroll
  for (int l = 0; l < 2 * MT; ++l) acc = cfma(a.A[row * a.N + l + 2], gin[l], acc);
  return cscale(kinv, acc);
}

// Inputs of the diagonal pivot at (m, n): arr1[l^1] at p - 1_{l/2}, scaled by sqrt(p_{l/2}).
template <int MT>
__device__ __forceinline__ void lo_diag_inputs(const LoArgs& a, const int32_t* p, int32_t f, int m, int n,
                                               int64_t* src, double* kl) {
#pragma unroll
  for (int l = 0; l < 2 * MT; ++l) {
    const int k = l >> 1;
    kl[l] = a.t.sq[p[k]];
    src[l] = p[k] > 0 ? lo_at(a, slot_arr1(a.L, l ^ 1), m, n, f - a.L.st[k]) : -1;
  }
}

// Inputs of the off-diagonal pivot d at (m, n).
template <int MT>
__device__ __forceinline__ void lo_offdiag_inputs(const LoArgs& a, const int32_t* p, int32_t f, int d, int m, int n,
                                                  int64_t* src, double* kl) {
#pragma unroll
  for (int i = 0; i < MT; ++i) {
    src[2 * i] = -1;
    src[2 * i + 1] = -1;
    kl[2 * i] = a.t.sq[p[i]];
    kl[2 * i + 1] = kl[2 * i];
    if (i < d) continue;
    if (i == d) {
      kl[2 * i] = a.t.sq[p[i] + 1];
      src[2 * i] = lo_at(a, 0, m, n, f);
      if (p[i] > 0) src[2 * i + 1] = lo_at(a, slot_arr2(a.L, d), m, n, f - a.L.st[i]);
    } else if (p[i] > 0) {
      src[2 * i] = lo_at(a, slot_1001(a.L, d, i - d - 1), m, n, f - a.L.st[i]);
      src[2 * i + 1] = lo_at(a, slot_1010(a.L, d, i - d - 1), m, n, f - a.L.st[i]);
    }
  }
}

template <int MT>
__device__ __forceinline__ void lo_gather(const LoArgs& a, const int64_t* src, const double* kl, double2* gin) {
#pragma unroll
  for (int l = 0; l < 2 * MT; ++l) gin[l] = src[l] >= 0 ? cscale(kl[l], ldv(&a.Wv[src[l]])) : cmk(0.0, 0.0);
}

// First block (singleLeftoverMode_amps.py:339-352): anti-diagonals s = m + k of the q x q block.
__global__ void lo_fill_kernel(LoArgs a) {
  const int q = a.q, N = a.N;
  double2* W = a.Wv;
  if (threadIdx.x == 0) W[lo_at(a, 0, 0, 0, 0)] = __ldg(a.G0);
  __syncthreads();
  auto at = [&](int m, int k) -> double2 { return (m < 0 || k < 0) ? cmk(0.0, 0.0) : W[lo_at(a, 0, m, k, 0)]; };
  for (int s = 1; s <= 2 * (q - 1); ++s) {
    for (int m = max(0, s - (q - 1)) + (int)threadIdx.x; m <= min(s, q - 1); m += blockDim.x) {
      const int k = s - m;
      double2 acc;
      if (k == 0) {  // column 0, from (m - 1, 0) and (m - 2, 0)
        acc = cmul(at(m - 1, 0), a.B[0]);
        acc = cfma(cscale(a.t.sq[m - 1], a.A[0]), at(m - 2, 0), acc);
        acc = cscale(a.t.rs[m], acc);
      } else {  // from (m, k - 1), (m - 1, k - 1), (m, k - 2)
        acc = cmul(at(m, k - 1), a.B[1]);
        acc = cfma(cscale(a.t.sq[m], a.A[N + 0]), at(m - 1, k - 1), acc);
        acc = cfma(cscale(a.t.sq[k - 1], a.A[N + 1]), at(m, k - 2), acc);
        acc = cscale(a.t.rs[k], acc);
      }
      W[lo_at(a, 0, m, k, 0)] = acc;
    }
    __syncthreads();
  }
}

template <int MT>
__global__ void __launch_bounds__(DG_BLOCK) lo_amps_kernel(LoArgs a) {
  MM_SHARED(StageSmem, sm);
  const double2* Bs = a.B;
  stage_operands(sm, a.t, a.ntab, a.A, a.N, &Bs);
  a.B = Bs;
  const DiagLat& L = a.L;
  const int q = a.q, qq = q * q;
  const int64_t t0 = (int64_t)blockIdx.x * blockDim.x + threadIdx.x, stride = (int64_t)gridDim.x * blockDim.x;
  uint32_t epoch = 0;
  for (int w = 0; w < L.W; ++w) {
    const int32_t s0 = a.sb.start[w], cnt = a.sb.start[w + 1] - s0;
    const int64_t per_row = (int64_t)cnt * qq;
    for (int phase = 0; phase < 2; ++phase) {
      for (int64_t t = t0; t < per_row * 2 * MT; t += stride) {
        const int r = (int)(t / per_row);
        const int64_t u = t - r * per_row;
        const int mn = (int)(u / cnt);
        const int32_t f = a.sb.order[s0 + (int32_t)(u - (int64_t)mn * cnt)];
        const int m = mn / q, n = mn - m * q;
        int32_t p[MT];
        decode_params<MT>(L, f, p);
        int64_t src[2 * MT];
        double kl[2 * MT];
        double2 gin[2 * MT];
        if (phase == 0) {
          if (!diag_target(L, p, r)) continue;
          lo_diag_inputs<MT>(a, p, f, m, n, src, kl);
          lo_gather<MT>(a, src, kl, gin);
          a.Wv[lo_at(a, slot_arr1(L, r), m, n, f)] = lo_value<MT>(a, r + 2, 0, f, m, n, gin, a.t.rs[p[r >> 1] + 1]);
          continue;
        }
        const int dl = last_pivot<MT>(p);
        for (int d = 0; d <= dl; ++d) {
          int row;
          int64_t slot;
          int32_t dst;
          if (!offdiag_target(L, p, d, r, row, slot, dst, f)) continue;
          lo_offdiag_inputs<MT>(a, p, f, d, m, n, src, kl);
          lo_gather<MT>(a, src, kl, gin);
          const int k = row >> 1;
          const int lift = (row & 1) == 0 && k == d;
          a.Wv[lo_at(a, slot, m, n, dst)] =
              lo_value<MT>(a, row + 2, slot_arr1(L, 2 * d), f, m, n, gin, a.t.rs[p[k] + lift + 1]);
        }
      }
      if (!step_barrier(a.h, epoch, a.budget)) return;
    }
  }
}

// ---- Jacobians

template <int MT>
__device__ __forceinline__ double2 lo_jac_value(const LoArgs& a, int row, int64_t ps, int32_t f, int m, int n,
                                                const int64_t* src, const double* kl, int qc, double kinv) {
  const int N = a.N, nA = N * N, nc = nA + N;
  const bool isA = qc < nA;
  const int qa = qc / N, qb = qc - qa * N;
  const double2* W = a.Wv;
  const double2* J = a.J;
  const int64_t pv = lo_at(a, ps, m, n, f);
  double2 acc = cmul(ldv(&J[pv * nc + qc]), a.B[row]);
  if (!isA && qc - nA == row) acc = cadd(acc, ldv(&W[pv]));
  if (m > 0) {
    const int64_t o = lo_at(a, ps, m - 1, n, f);
    acc = cfma(cscale(a.t.sq[m], a.A[row * N + 0]), ldv(&J[o * nc + qc]), acc);
    if (isA && qa == row && qb == 0) acc = cadd(acc, cscale(a.t.sq[m], ldv(&W[o])));
  }
  if (n > 0) {
    const int64_t o = lo_at(a, ps, m, n - 1, f);
    acc = cfma(cscale(a.t.sq[n], a.A[row * N + 1]), ldv(&J[o * nc + qc]), acc);
    if (isA && qa == row && qb == 1) acc = cadd(acc, cscale(a.t.sq[n], ldv(&W[o])));
  }
#pragma unroll
  for (int l = 0; l < 2 * MT; ++l) {
    if (src[l] < 0) continue;
    acc = cfma(cscale(kl[l], a.A[row * N + l + 2]), ldv(&J[src[l] * nc + qc]), acc);
    if (isA && qa == row && qb == l + 2) acc = cadd(acc, cscale(kl[l], ldv(&W[src[l]])));
  }
  return cscale(kinv, acc);
}

// First block's Jacobians (singleLeftoverMode_grad.py:606-650), one thread per component.
__global__ void lo_fill_jacobian_kernel(LoArgs a) {
  const int q = a.q, N = a.N, nA = N * N, nc = nA + N;
  const double2* W = a.Wv;
  double2* J = a.J;
  auto jat = [&](int m, int k, int c) -> double2 {
    return (m < 0 || k < 0) ? cmk(0.0, 0.0) : J[lo_at(a, 0, m, k, 0) * nc + c];
  };
  auto wat = [&](int m, int k) -> double2 { return (m < 0 || k < 0) ? cmk(0.0, 0.0) : W[lo_at(a, 0, m, k, 0)]; };
  for (int s = 1; s <= 2 * (q - 1); ++s) {
    const int m_lo = max(0, s - (q - 1)), m_hi = min(s, q - 1);
    const int items = (m_hi - m_lo + 1) * nc;
    for (int it = threadIdx.x; it < items; it += blockDim.x) {
      const int m = m_lo + it / nc, c = it % nc, k = s - m;
      double2 acc;
      if (k == 0) {
        acc = cmul(jat(m - 1, 0, c), a.B[0]);
        acc = cfma(cscale(a.t.sq[m - 1], a.A[0]), jat(m - 2, 0, c), acc);
        if (c == 0) acc = cadd(acc, cscale(a.t.sq[m - 1], wat(m - 2, 0)));
        if (c == nA) acc = cadd(acc, wat(m - 1, 0));
        acc = cscale(a.t.rs[m], acc);
      } else {
        acc = cmul(jat(m, k - 1, c), a.B[1]);
        acc = cfma(cscale(a.t.sq[m], a.A[N + 0]), jat(m - 1, k - 1, c), acc);
        acc = cfma(cscale(a.t.sq[k - 1], a.A[N + 1]), jat(m, k - 2, c), acc);
        if (c == N) acc = cadd(acc, cscale(a.t.sq[m], wat(m - 1, k - 1)));
        if (c == N + 1) acc = cadd(acc, cscale(a.t.sq[k - 1], wat(m, k - 2)));
        if (c == nA + 1) acc = cadd(acc, wat(m, k - 1));
        acc = cscale(a.t.rs[k], acc);
      }
      J[lo_at(a, 0, m, k, 0) * nc + c] = acc;
    }
    __syncthreads();
  }
}

template <int MT>
__global__ void __launch_bounds__(DG_BLOCK) lo_jacobian_kernel(LoArgs a) {
  MM_SHARED(StageSmem, sm);
  const double2* Bs = a.B;
  stage_operands(sm, a.t, a.ntab, a.A, a.N, &Bs);
  a.B = Bs;
  const DiagLat& L = a.L;
  const int q = a.q, qq = q * q, nc = a.N * a.N + a.N;
  const int64_t t0 = (int64_t)blockIdx.x * blockDim.x + threadIdx.x, stride = (int64_t)gridDim.x * blockDim.x;
  uint32_t epoch = 0;
  for (int w = 0; w < L.W; ++w) {
    const int32_t s0 = a.sb.start[w], cnt = a.sb.start[w + 1] - s0;
    const int64_t per_row = (int64_t)cnt * qq * nc;
    for (int phase = 0; phase < 2; ++phase) {
      for (int64_t t = t0; t < per_row * 2 * MT; t += stride) {
        const int r = (int)(t / per_row);
        const int64_t u = t - r * per_row;
        const int64_t v = u / nc;
        const int qc = (int)(u - v * nc);
        const int mn = (int)(v / cnt);
        const int32_t f = a.sb.order[s0 + (int32_t)(v - (int64_t)mn * cnt)];
        const int m = mn / q, n = mn - m * q;
        int32_t p[MT];
        decode_params<MT>(L, f, p);
        int64_t src[2 * MT];
        double kl[2 * MT];
        if (phase == 0) {
          if (!diag_target(L, p, r)) continue;
          lo_diag_inputs<MT>(a, p, f, m, n, src, kl);
          a.J[lo_at(a, slot_arr1(L, r), m, n, f) * nc + qc] =
              lo_jac_value<MT>(a, r + 2, 0, f, m, n, src, kl, qc, a.t.rs[p[r >> 1] + 1]);
          continue;
        }
        const int dl = last_pivot<MT>(p);
        for (int d = 0; d <= dl; ++d) {
          int row;
          int64_t slot;
          int32_t dst;
          if (!offdiag_target(L, p, d, r, row, slot, dst, f)) continue;
          lo_offdiag_inputs<MT>(a, p, f, d, m, n, src, kl);
          const int k = row >> 1;
          const int lift = (row & 1) == 0 && k == d;
          a.J[lo_at(a, slot, m, n, dst) * nc + qc] =
              lo_jac_value<MT>(a, row + 2, slot_arr1(L, 2 * d), f, m, n, src, kl, qc, a.t.rs[p[k] + lift + 1]);
        }
      }
      if (!step_barrier(a.h, epoch, a.budget)) return;
    }
  }
}

// ------------------------------------------------------------------ host planning

#ifndef MM_HOST_EMULATION
struct DevCfg {
  int sms = 0;
  int occ = 0;
};

int dev_cfg(const void* kernel, DevCfg& dc) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return MM_ERR_NO_DEVICE;
  if (cudaDeviceGetAttribute(&dc.sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return MM_ERR_CUDA;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&dc.occ, kernel, DG_BLOCK, 0) != cudaSuccess) return MM_ERR_CUDA;
  if (dc.occ < 1) return MM_ERR_UNSUPPORTED;
  return MM_OK;
}

#endif

int diag_lat(int M, const int64_t* cutoffs, int64_t nb, DiagLat& L) {
  if (M < 1 || cutoffs == nullptr || nb < 1) return MM_ERR_INVALID_ARG;
  if (M > DG_MAXM) return MM_ERR_UNSUPPORTED;
  memset(&L, 0, sizeof(L));
  L.M = M;
  L.n = 2 * M;
  int64_t P = 1, W = 1;
  for (int k = M - 1; k >= 0; --k) {
    if (cutoffs[k] < 1) return MM_ERR_INVALID_ARG;
    if (cutoffs[k] > 99999) return MM_ERR_TOO_LARGE;
    L.c[k] = (int32_t)cutoffs[k];
    L.st[k] = (int32_t)P;
    P *= cutoffs[k];
    W += cutoffs[k] - 1;
    if (P * nb * diag_slots(M) > ((int64_t)1 << 40) || P > INT32_MAX / 64) return MM_ERR_TOO_LARGE;
  }
  if (W > kMaxWeights || nb > INT32_MAX) return MM_ERR_TOO_LARGE;
  L.P = (int32_t)P;
  L.nb = (int32_t)nb;
  L.W = (int32_t)W;
  return MM_OK;
}

// points per weight: coefficients of prod_k (1 + x + ... + x^{c_k - 1})
std::vector<int64_t> diag_counts(const DiagLat& L) {
  std::vector<int64_t> cnt(1, 1);
  for (int k = 0; k < L.M; ++k) {
    std::vector<int64_t> nx(cnt.size() + L.c[k] - 1, 0);
    for (size_t s = 0; s < cnt.size(); ++s)
      for (int v = 0; v < L.c[k]; ++v) nx[s + v] += cnt[s];
    cnt.swap(nx);
  }
  return cnt;
}

struct DiagWs {
  size_t header, count, start, cursor, order, tabs, total;
  int32_t ntab;
};
// header | weight counts | starts | cursors | point order | sqrt and 1/sqrt tables (ntab each)
DiagWs diag_ws(int32_t W, int32_t npts, int32_t ntab) {
  DiagWs w;
  w.header = 0;
  w.ntab = ntab;
  w.count = al(sizeof(WsHeader));
  w.start = w.count + al((size_t)W * sizeof(int32_t));
  w.cursor = w.start + al((size_t)(W + 1) * sizeof(int32_t));
  w.order = w.cursor + al((size_t)W * sizeof(int32_t));
  w.tabs = w.order + al((size_t)npts * sizeof(int32_t));
  w.total = w.tabs + al(2 * (size_t)ntab * sizeof(double));
  return w;
}
Tabs tabs_of(char* ws, const DiagWs& w) {
  Tabs t;
  t.sq = reinterpret_cast<const double*>(ws + w.tabs);
  t.rs = t.sq + w.ntab;
  return t;
}
#ifndef MM_HOST_EMULATION
int launch_tables(char* ws, const DiagWs& w, cudaStream_t st) {
  double* sq = reinterpret_cast<double*>(ws + w.tabs);
  sqrt_table_kernel<<<(unsigned)std::max<int64_t>(1, std::min<int64_t>((w.ntab + 255) / 256, 64)), 256, 0, st>>>(
      sq, sq + w.ntab, w.ntab);
  note_launches(1);
  return cuda_status();
}
#endif
int32_t diag_ntab(const DiagLat& L) {
  int32_t mc = 1;
  for (int k = 0; k < L.M; ++k) mc = std::max(mc, L.c[k]);
  return mc + 3;  // sqrt(p + 2) with p <= c - 1
}
SortBufs sort_bufs(char* ws, const DiagWs& w) {
  SortBufs sb;
  sb.count = reinterpret_cast<int32_t*>(ws + w.count);
  sb.start = reinterpret_cast<int32_t*>(ws + w.start);
  sb.cursor = reinterpret_cast<int32_t*>(ws + w.cursor);
  sb.order = reinterpret_cast<int32_t*>(ws + w.order);
  return sb;
}

#ifndef MM_HOST_EMULATION
int check_ws(void* ws, size_t ws_bytes, size_t need) {
  if (ws == nullptr || ((uintptr_t)ws % kWsAlign) != 0 || ws_bytes < need) return MM_ERR_WORKSPACE;
  return MM_OK;
}

// CTAs of a wavefront launch: one per DG_BLOCK items of the widest weight, at most what fits
// co-resident (and at most MM_DIAG_MAX_CTAS when that is set).
int64_t max_ctas_env() {
  static const int64_t v = [] {
    const char* s = getenv("MM_DIAG_MAX_CTAS");
    return s ? (int64_t)strtoll(s, nullptr, 10) : (int64_t)0;
  }();
  return v;
}

int launch_wavefront(void* kern, void* arg, int64_t max_items, int sms, int occ, cudaStream_t st) {
  int64_t cap = (int64_t)sms * occ;
  if (max_ctas_env() > 0) cap = std::min(cap, max_ctas_env());
  const unsigned blocks = (unsigned)std::max<int64_t>(1, std::min<int64_t>((max_items + DG_BLOCK - 1) / DG_BLOCK, cap));
  void* args[] = {arg};
  if (cudaLaunchCooperativeKernel(kern, dim3(blocks), dim3(DG_BLOCK), args, 0, st) != cudaSuccess) return MM_ERR_CUDA;
  note_launches(1);
  return MM_OK;
}

#endif

int fd_lat(int Lm, const int64_t* pnr, int64_t oc, FdLat& F) {
  if (Lm < 2 || pnr == nullptr || oc < 0) return Lm == 1 ? MM_ERR_UNSUPPORTED : MM_ERR_INVALID_ARG;
  if (Lm - 1 > FD_MAXK) return MM_ERR_UNSUPPORTED;
  if (oc > 4096) return MM_ERR_TOO_LARGE;
  memset(&F, 0, sizeof(F));
  F.K = Lm - 1;
  F.q = (int)(oc + 1);
  int64_t npts = 1, nout = 1, sum = 0;
  for (int j = F.K - 1; j >= 0; --j) {
    if (pnr[j] < 0) return MM_ERR_INVALID_ARG;
    if (pnr[j] > 9999) return MM_ERR_TOO_LARGE;  // the reference's sqrt table (fast_diagonal.py:29)
    F.pnr[j] = (int32_t)pnr[j];
    F.rad[j] = (int32_t)(5 * (pnr[j] + 1));
    F.pst[j] = (int32_t)npts;
    F.ost[j] = (int32_t)nout;
    npts *= F.rad[j];
    nout *= pnr[j] + 1;
    sum += pnr[j];
    if (npts > INT32_MAX / 8 || npts * F.q * F.q > ((int64_t)1 << 36)) return MM_ERR_TOO_LARGE;
  }
  F.npts = (int32_t)npts;
  F.W = (int32_t)(2 * sum + 1);
  F.wend = (int32_t)std::max<int64_t>(1, std::min<int64_t>(2 * oc + 2 * sum - Lm, (int64_t)F.W));
  return MM_OK;
}

int lo_lat(int M, const int64_t* cutoffs, DiagLat& L, int& q) {
  if (cutoffs == nullptr || M < 2) return M == 1 ? MM_ERR_UNSUPPORTED : MM_ERR_INVALID_ARG;
  if (M > DG_MAXM) return MM_ERR_UNSUPPORTED;
  if (cutoffs[0] < 1) return MM_ERR_INVALID_ARG;
  if (cutoffs[0] > 1000) return MM_ERR_TOO_LARGE;  // the reference's sqrt table (helperFunctions.py:12)
  q = (int)cutoffs[0];
  const int rc = diag_lat(M - 1, cutoffs + 1, 1, L);
  if (rc) return rc;
  if ((int64_t)L.P * q * q * diag_slots(M - 1) > ((int64_t)1 << 36)) return MM_ERR_TOO_LARGE;
  return MM_OK;
}
int32_t lo_ntab(const DiagLat& L, int q) { return std::max(diag_ntab(L), q + 1); }

// lattice points per weight: per pair, states by a + b split into |a-b| < 2 and |a-b| = 2;
// the product keeps at most one pair at distance 2
std::vector<int64_t> fd_counts(const FdLat& F) {
  std::vector<int64_t> c0(1, 1), c1(1, 0);  // no pair at distance 2 / exactly one
  for (int j = 0; j < F.K; ++j) {
    const int p = F.pnr[j];
    std::vector<int64_t> s0(2 * p + 1, 0), s2(2 * p + 1, 0);
    for (int a = 0; a <= p; ++a)
      for (int b = std::max(0, a - 2); b <= std::min(p, a + 2); ++b) (std::abs(a - b) == 2 ? s2 : s0)[a + b] += 1;
    std::vector<int64_t> n0(c0.size() + 2 * p, 0), n1(c0.size() + 2 * p, 0);
    for (size_t s = 0; s < c0.size(); ++s)
      for (int v = 0; v <= 2 * p; ++v) {
        n0[s + v] += c0[s] * s0[v];
        n1[s + v] += c1[s] * s0[v] + c0[s] * s2[v];
      }
    c0.swap(n0);
    c1.swap(n1);
  }
  for (size_t s = 0; s < c0.size(); ++s) c0[s] += c1[s];
  return c0;
}

struct FdWs {
  DiagWs base;
  size_t ap, g, total;
};
int32_t fd_ntab(const FdLat& F) {
  int32_t mx = F.q;
  for (int j = 0; j < F.K; ++j) mx = std::max(mx, F.pnr[j] + 2);
  return mx + 1;
}
FdWs fd_ws(const FdLat& F) {
  FdWs w;
  w.base = diag_ws(F.W, F.npts, fd_ntab(F));
  const int n = 2 * (F.K + 1);
  w.ap = w.base.total;
  w.g = w.ap + al((size_t)(n * n + n) * sizeof(double2));
  w.total = w.g + al((size_t)F.npts * F.q * F.q * sizeof(double2));
  return w;
}

}  // namespace

#ifndef MM_HOST_EMULATION
// =================================================================== C ABI

MM_API int64_t mm_diagonal_slots(int M) { return M < 1 ? 0 : diag_slots(M); }

MM_API size_t mm_diagonal_workspace_bytes(int M, const int64_t* cutoffs, int64_t nb) {
  DiagLat L;
  if (diag_lat(M, cutoffs, nb, L)) return 0;
  return diag_ws(L.W, L.P, diag_ntab(L)).total;
}

void* diag_amps_fn(int M) {
  switch (M) {
    case 1: return (void*)diag_amps_kernel<1>;
    case 2: return (void*)diag_amps_kernel<2>;
    case 3: return (void*)diag_amps_kernel<3>;
    case 4: return (void*)diag_amps_kernel<4>;
    case 5: return (void*)diag_amps_kernel<5>;
    case 6: return (void*)diag_amps_kernel<6>;
    case 7: return (void*)diag_amps_kernel<7>;
    case 8: return (void*)diag_amps_kernel<8>;
  }
  return nullptr;
}
void* diag_jacobian_fn(int M) {
  switch (M) {
    case 1: return (void*)diag_jacobian_kernel<1>;
    case 2: return (void*)diag_jacobian_kernel<2>;
    case 3: return (void*)diag_jacobian_kernel<3>;
    case 4: return (void*)diag_jacobian_kernel<4>;
    case 5: return (void*)diag_jacobian_kernel<5>;
    case 6: return (void*)diag_jacobian_kernel<6>;
    case 7: return (void*)diag_jacobian_kernel<7>;
    case 8: return (void*)diag_jacobian_kernel<8>;
  }
  return nullptr;
}
void* lo_amps_fn(int MT) {
  switch (MT) {
    case 1: return (void*)lo_amps_kernel<1>;
    case 2: return (void*)lo_amps_kernel<2>;
    case 3: return (void*)lo_amps_kernel<3>;
    case 4: return (void*)lo_amps_kernel<4>;
    case 5: return (void*)lo_amps_kernel<5>;
    case 6: return (void*)lo_amps_kernel<6>;
    case 7: return (void*)lo_amps_kernel<7>;
  }
  return nullptr;
}
void* lo_jacobian_fn(int MT) {
  switch (MT) {
    case 1: return (void*)lo_jacobian_kernel<1>;
    case 2: return (void*)lo_jacobian_kernel<2>;
    case 3: return (void*)lo_jacobian_kernel<3>;
    case 4: return (void*)lo_jacobian_kernel<4>;
    case 5: return (void*)lo_jacobian_kernel<5>;
    case 6: return (void*)lo_jacobian_kernel<6>;
    case 7: return (void*)lo_jacobian_kernel<7>;
  }
  return nullptr;
}

void* fd_fn(int K) {
  switch (K) {
    case 1: return (void*)fd_kernel<1>;
    case 2: return (void*)fd_kernel<2>;
    case 3: return (void*)fd_kernel<3>;
    case 4: return (void*)fd_kernel<4>;
    case 5: return (void*)fd_kernel<5>;
    case 6: return (void*)fd_kernel<6>;
    case 7: return (void*)fd_kernel<7>;
  }
  return nullptr;
}

MM_API int mm_diagonal_amps(int M, const int64_t* cutoffs, int64_t nb, const mm_c128* A, const mm_c128* B,
                            const mm_c128* G0, mm_c128* W, void* ws, size_t ws_bytes, mm_stream_t stream) {
  DiagLat L;
  int rc = diag_lat(M, cutoffs, nb, L);
  if (rc) return rc;
  if (!A || !B || !G0 || !W) return MM_ERR_INVALID_ARG;
  const DiagWs lay = diag_ws(L.W, L.P, diag_ntab(L));
  if ((rc = check_ws(ws, ws_bytes, lay.total))) return rc;
  void* kern = diag_amps_fn(M);
  DevCfg dc;
  if ((rc = dev_cfg(kern, dc))) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  char* w = static_cast<char*>(ws);
  DiagArgs a;
  memset(&a, 0, sizeof(a));
  a.L = L;
  a.A = (const double2*)A;
  a.B = (const double2*)B;
  a.G0 = (const double2*)G0;
  a.Wv = (double2*)W;
  a.t = tabs_of(w, lay);
  a.ntab = lay.ntab;
  a.sb = sort_bufs(w, lay);
  a.h = reinterpret_cast<WsHeader*>(w);
  a.budget = budget_ns();
  if (cudaMemsetAsync(w + MM_WS_LAUNCH_STATE_OFFSET, 0, MM_WS_LAUNCH_STATE_BYTES, st) != cudaSuccess) return MM_ERR_CUDA;
  if (cudaMemsetAsync(W, 0, (size_t)diag_slots(M) * L.P * L.nb * sizeof(double2), st) != cudaSuccess)
    return MM_ERR_CUDA;
  if ((rc = launch_sort(L, L.P, L.W, a.sb, dc.sms, st))) return rc;
  if ((rc = launch_tables(w, lay, st))) return rc;
  diag_init_kernel<<<1, 128, 0, st>>>(a);
  note_launches(1);
  if ((rc = cuda_status())) return rc;
  const std::vector<int64_t> cnt = diag_counts(L);
  const int64_t max_items = *std::max_element(cnt.begin(), cnt.end()) * 2 * L.n * L.nb;
  return launch_wavefront(kern, &a, max_items, dc.sms, dc.occ, st);
}

MM_API int mm_diagonal_jacobian(int M, const int64_t* cutoffs, const mm_c128* A, const mm_c128* B, const mm_c128* W,
                                mm_c128* J, void* ws, size_t ws_bytes, mm_stream_t stream) {
  DiagLat L;
  int rc = diag_lat(M, cutoffs, 1, L);
  if (rc) return rc;
  if (!A || !B || !W || !J) return MM_ERR_INVALID_ARG;
  const int64_t nc = (int64_t)L.n * L.n + L.n;
  if ((int64_t)L.P * nc * diag_slots(M) > ((int64_t)1 << 36)) return MM_ERR_TOO_LARGE;
  const DiagWs lay = diag_ws(L.W, L.P, diag_ntab(L));
  if ((rc = check_ws(ws, ws_bytes, lay.total))) return rc;
  void* kern = diag_jacobian_fn(M);
  DevCfg dc;
  if ((rc = dev_cfg(kern, dc))) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  char* w = static_cast<char*>(ws);
  DiagArgs a;
  memset(&a, 0, sizeof(a));
  a.L = L;
  a.A = (const double2*)A;
  a.B = (const double2*)B;
  a.Wv = (double2*)W;
  a.J = (double2*)J;
  a.t = tabs_of(w, lay);
  a.ntab = lay.ntab;
  a.sb = sort_bufs(w, lay);
  a.h = reinterpret_cast<WsHeader*>(w);
  a.budget = budget_ns();
  if (cudaMemsetAsync(w + MM_WS_LAUNCH_STATE_OFFSET, 0, MM_WS_LAUNCH_STATE_BYTES, st) != cudaSuccess) return MM_ERR_CUDA;
  if (cudaMemsetAsync(J, 0, (size_t)diag_slots(M) * L.P * nc * sizeof(double2), st) != cudaSuccess) return MM_ERR_CUDA;
  if ((rc = launch_sort(L, L.P, L.W, a.sb, dc.sms, st))) return rc;
  if ((rc = launch_tables(w, lay, st))) return rc;
  const std::vector<int64_t> cnt = diag_counts(L);
  const int64_t max_items = *std::max_element(cnt.begin(), cnt.end()) * 2 * L.n * nc;
  return launch_wavefront(kern, &a, max_items, dc.sms, dc.occ, st);
}

MM_API int mm_diagonal_vjp(int M, const int64_t* cutoffs, const mm_c128* J, const mm_c128* W, const mm_c128* G0,
                           const mm_c128* g, mm_c128* dA, mm_c128* dB, mm_c128* dG0, mm_stream_t stream) {
  DiagLat L;
  int rc = diag_lat(M, cutoffs, 1, L);
  if (rc) return rc;
  if (!J || !W || !G0 || !g || !dA || !dB || !dG0) return MM_ERR_INVALID_ARG;
  const int nc = L.n * L.n + L.n;
  diag_vjp_kernel<<<nc + 1, 256, 0, (cudaStream_t)stream>>>(L, (const double2*)J, (const double2*)W,
                                                            (const double2*)G0, (const double2*)g, (double2*)dA,
                                                            (double2*)dB, (double2*)dG0);
  note_launches(1);
  return cuda_status();
}

MM_API size_t mm_fast_diagonal_workspace_bytes(int L, const int64_t* pnr_cutoffs, int64_t output_cutoff) {
  FdLat F;
  if (fd_lat(L, pnr_cutoffs, output_cutoff, F)) return 0;
  return fd_ws(F).total;
}

MM_API int mm_fast_diagonal(int L, const int64_t* pnr_cutoffs, int64_t output_cutoff, const mm_c128* A,
                            const mm_c128* b, const mm_c128* c, int stable, mm_c128* out, void* ws, size_t ws_bytes,
                            mm_stream_t stream) {
  FdLat F;
  int rc = fd_lat(L, pnr_cutoffs, output_cutoff, F);
  if (rc) return rc;
  if (!A || !b || !c || !out) return MM_ERR_INVALID_ARG;
  const FdWs lay = fd_ws(F);
  if ((rc = check_ws(ws, ws_bytes, lay.total))) return rc;
  void* kern = fd_fn(F.K);
  DevCfg dc;
  if ((rc = dev_cfg(kern, dc))) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  char* w = static_cast<char*>(ws);
  FdArgs a;
  memset(&a, 0, sizeof(a));
  a.F = F;
  a.A = (const double2*)A;
  a.b = (const double2*)b;
  a.c = (const double2*)c;
  a.stable = stable ? 1 : 0;
  const int n = 2 * L;
  a.Ap = reinterpret_cast<double2*>(w + lay.ap);
  a.bp = a.Ap + n * n;
  a.G = reinterpret_cast<double2*>(w + lay.g);
  a.out = (double2*)out;
  a.t = tabs_of(w, lay.base);
  a.ntab = lay.base.ntab;
  a.sb = sort_bufs(w, lay.base);
  a.h = reinterpret_cast<WsHeader*>(w);
  a.budget = budget_ns();
  int64_t nout = (int64_t)F.q * F.q;
  for (int j = 0; j < F.K; ++j) nout *= F.pnr[j] + 1;
  if (cudaMemsetAsync(w + MM_WS_LAUNCH_STATE_OFFSET, 0, MM_WS_LAUNCH_STATE_BYTES, st) != cudaSuccess) return MM_ERR_CUDA;
  if (cudaMemsetAsync(out, 0, (size_t)nout * sizeof(double2), st) != cudaSuccess) return MM_ERR_CUDA;
  if ((rc = launch_sort(F, F.npts, F.W, a.sb, dc.sms, st))) return rc;
  if ((rc = launch_tables(w, lay.base, st))) return rc;
  fd_init_kernel<<<1, 256, 0, st>>>(a);
  note_launches(1);
  if ((rc = cuda_status())) return rc;
  const std::vector<int64_t> cnt = fd_counts(F);
  int64_t mx = 1;
  for (int wgt = 1; wgt < (int)cnt.size() && wgt < F.wend; ++wgt) mx = std::max(mx, cnt[wgt]);
  return launch_wavefront(kern, &a, mx * F.q * F.q, dc.sms, dc.occ, st);
}

MM_API int64_t mm_leftover_slots(int M) { return M < 2 ? 0 : diag_slots(M - 1); }

MM_API size_t mm_leftover_workspace_bytes(int M, const int64_t* cutoffs) {
  DiagLat L;
  int q;
  if (lo_lat(M, cutoffs, L, q)) return 0;
  return diag_ws(L.W, L.P, lo_ntab(L, q)).total;
}

static int lo_setup(int M, const int64_t* cutoffs, const mm_c128* A, const mm_c128* B, void* ws, size_t ws_bytes,
                    LoArgs& a, DiagWs& lay) {
  int q;
  int rc = lo_lat(M, cutoffs, a.L, q);
  if (rc) return rc;
  if (!A || !B) return MM_ERR_INVALID_ARG;
  lay = diag_ws(a.L.W, a.L.P, lo_ntab(a.L, q));
  if ((rc = check_ws(ws, ws_bytes, lay.total))) return rc;
  char* w = static_cast<char*>(ws);
  a.q = q;
  a.N = 2 * M;
  a.A = (const double2*)A;
  a.B = (const double2*)B;
  a.t = tabs_of(w, lay);
  a.ntab = lay.ntab;
  a.sb = sort_bufs(w, lay);
  a.h = reinterpret_cast<WsHeader*>(w);
  a.budget = budget_ns();
  return MM_OK;
}

MM_API int mm_leftover_amps(int M, const int64_t* cutoffs, const mm_c128* A, const mm_c128* B, const mm_c128* G0,
                            mm_c128* W, void* ws, size_t ws_bytes, mm_stream_t stream) {
  LoArgs a;
  memset(&a, 0, sizeof(a));
  DiagWs lay;
  int rc = lo_setup(M, cutoffs, A, B, ws, ws_bytes, a, lay);
  if (rc) return rc;
  if (!G0 || !W) return MM_ERR_INVALID_ARG;
  a.G0 = (const double2*)G0;
  a.Wv = (double2*)W;
  void* kern = lo_amps_fn(M - 1);
  DevCfg dc;
  if ((rc = dev_cfg(kern, dc))) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  char* w = static_cast<char*>(ws);
  const int64_t qq = (int64_t)a.q * a.q;
  if (cudaMemsetAsync(w + MM_WS_LAUNCH_STATE_OFFSET, 0, MM_WS_LAUNCH_STATE_BYTES, st) != cudaSuccess) return MM_ERR_CUDA;
  if (cudaMemsetAsync(W, 0, (size_t)diag_slots(M - 1) * qq * a.L.P * sizeof(double2), st) != cudaSuccess)
    return MM_ERR_CUDA;
  if ((rc = launch_sort(a.L, a.L.P, a.L.W, a.sb, dc.sms, st))) return rc;
  if ((rc = launch_tables(w, lay, st))) return rc;
  lo_fill_kernel<<<1, 256, 0, st>>>(a);
  note_launches(1);
  if ((rc = cuda_status())) return rc;
  const std::vector<int64_t> cnt = diag_counts(a.L);
  const int64_t max_items = *std::max_element(cnt.begin(), cnt.end()) * qq * a.L.n;
  return launch_wavefront(kern, &a, max_items, dc.sms, dc.occ, st);
}

MM_API int mm_leftover_jacobian(int M, const int64_t* cutoffs, const mm_c128* A, const mm_c128* B, const mm_c128* W,
                                mm_c128* J, void* ws, size_t ws_bytes, mm_stream_t stream) {
  LoArgs a;
  memset(&a, 0, sizeof(a));
  DiagWs lay;
  int rc = lo_setup(M, cutoffs, A, B, ws, ws_bytes, a, lay);
  if (rc) return rc;
  if (!W || !J) return MM_ERR_INVALID_ARG;
  a.Wv = (double2*)W;
  a.J = (double2*)J;
  const int64_t nc = (int64_t)a.N * a.N + a.N, qq = (int64_t)a.q * a.q;
  if ((int64_t)a.L.P * qq * nc * diag_slots(M - 1) > ((int64_t)1 << 36)) return MM_ERR_TOO_LARGE;
  void* kern = lo_jacobian_fn(M - 1);
  DevCfg dc;
  if ((rc = dev_cfg(kern, dc))) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  char* w = static_cast<char*>(ws);
  if (cudaMemsetAsync(w + MM_WS_LAUNCH_STATE_OFFSET, 0, MM_WS_LAUNCH_STATE_BYTES, st) != cudaSuccess) return MM_ERR_CUDA;
  if (cudaMemsetAsync(J, 0, (size_t)diag_slots(M - 1) * qq * a.L.P * nc * sizeof(double2), st) != cudaSuccess)
    return MM_ERR_CUDA;
  if ((rc = launch_sort(a.L, a.L.P, a.L.W, a.sb, dc.sms, st))) return rc;
  if ((rc = launch_tables(w, lay, st))) return rc;
  lo_fill_jacobian_kernel<<<1, 256, 0, st>>>(a);
  note_launches(1);
  if ((rc = cuda_status())) return rc;
  const std::vector<int64_t> cnt = diag_counts(a.L);
  const int64_t max_items = *std::max_element(cnt.begin(), cnt.end()) * qq * nc * a.L.n;
  return launch_wavefront(kern, &a, max_items, dc.sms, dc.occ, st);
}

MM_API int mm_leftover_vjp(int M, const int64_t* cutoffs, const mm_c128* J, const mm_c128* W, const mm_c128* G0,
                           const mm_c128* g, mm_c128* dA, mm_c128* dB, mm_c128* dG0, mm_stream_t stream) {
  DiagLat L;
  int q;
  int rc = lo_lat(M, cutoffs, L, q);
  if (rc) return rc;
  if (!J || !W || !G0 || !g || !dA || !dB || !dG0) return MM_ERR_INVALID_ARG;
  // arr0's Jacobian is [block entry][component] with the entries (m, n, params) flat, the layout
  // the diagonal strategy's VJP contracts: reuse it with 2M rows and q^2 P' entries.
  if ((int64_t)q * q * L.P > INT32_MAX) return MM_ERR_TOO_LARGE;  // arr0 entries are counted in 32 bits
  DiagLat V;
  memset(&V, 0, sizeof(V));
  V.M = M;
  V.n = 2 * M;
  V.P = (int32_t)((int64_t)q * q * L.P);
  const int nc = V.n * V.n + V.n;
  diag_vjp_kernel<<<nc + 1, 256, 0, (cudaStream_t)stream>>>(V, (const double2*)J, (const double2*)W,
                                                            (const double2*)G0, (const double2*)g, (double2*)dA,
                                                            (double2*)dB, (double2*)dG0);
  note_launches(1);
  return cuda_status();
}
#endif  // MM_HOST_EMULATION
