// Per-mode Fock cutoffs of Gaussian density-matrix triples (autoshape).
//
// Reference: autoshape_numba, mrmustard/math/lattice/autoshape.py:23-154,
// called by State.auto_shape (mrmustard/lab/states/base.py:383-430) on the
// triple of ``ansatz.conj & ansatz`` (2M x 2M A, 2M-vector b, scalar c; the
// first M variables are the bra copy, the last M the ket copy).  For every mode
// m the reference reduces the state to mode m,
//     Z = inv(A_nn - X), X = [[0, I], [I, 0]] over the other M-1 modes,
//     A_ = A_mm - (A_mn Z) A_mn^T,  b_ = b_m - (A_mn Z) b_n,
//     c_ = c exp(((-1/2 b_n) Z) b_n) / sqrt(det(A_nn - X))
// (A_nm taken as A_mn^T), then runs a buffered single-mode recurrence over the
// elements around the diagonal, adding |rho_kk| until the sum reaches max_prob
// or k reaches max_shape; the shape is clip(k, min_shape, max_shape).
//
// One thread per (state, mode): the work per pair is a (2M-2)-sized complex LU
// and at most max_shape steps of a 9-element recurrence, independent across
// pairs.  Every product and sum is an explicitly rounded FP64 operation (no
// fused multiply-add), in the reference's order, so the results follow the
// reference's arithmetic term by term; the LU pivots on |re| + |im| as LAPACK
// does.  The recurrence's divisions by sqrt(k) give the correctly rounded
// quotient from a correctly rounded reciprocal (div_by_recip, Markstein's
// theorem; checked bit for bit against the division by mm_probe_division).
// A reduction whose matrix is singular (the reference raises LinAlgError)
// yields shape -1 for every mode of that state.
#include <cstdint>

#include "common.cuh"

namespace {

constexpr int AS_MAXM = 8;
constexpr int AS_MAXN = 2 * (AS_MAXM - 1);

struct cx {
  double r, i;
};
__device__ __forceinline__ cx mk(double r, double i) { return {r, i}; }
__device__ __forceinline__ cx cmul(cx a, cx b) {
  return mk(__dsub_rn(__dmul_rn(a.r, b.r), __dmul_rn(a.i, b.i)), __dadd_rn(__dmul_rn(a.r, b.i), __dmul_rn(a.i, b.r)));
}
__device__ __forceinline__ cx cadd(cx a, cx b) { return mk(__dadd_rn(a.r, b.r), __dadd_rn(a.i, b.i)); }
__device__ __forceinline__ cx csub(cx a, cx b) { return mk(__dsub_rn(a.r, b.r), __dsub_rn(a.i, b.i)); }
// complex * real, the real promoted to (s, 0) as in the reference's mixed arithmetic
__device__ __forceinline__ cx cmulr(cx a, double s) {
  return mk(__dsub_rn(__dmul_rn(a.r, s), __dmul_rn(a.i, 0.0)), __dadd_rn(__dmul_rn(a.r, 0.0), __dmul_rn(a.i, s)));
}
// complex / real: each part divided (numba's lowering of the reference's "/ SQRT[k]"); y = RN(1/d)
// makes each correctly rounded quotient three FP64 operations (div_by_recip)
__device__ __forceinline__ cx cdivr(cx a, double d, double y) {
  return mk(mm::div_by_recip(__dadd_rn(a.r, __dmul_rn(a.i, 0.0)), d, y),
            mm::div_by_recip(__dsub_rn(a.i, __dmul_rn(a.r, 0.0)), d, y));
}
// complex / complex: Smith's algorithm (numpy's complex division loop)
__device__ __forceinline__ cx cdiv(cx a, cx b) {
  if (fabs(b.r) >= fabs(b.i)) {
    const double rat = __ddiv_rn(b.i, b.r), scl = __ddiv_rn(1.0, __dadd_rn(b.r, __dmul_rn(b.i, rat)));
    return mk(__dmul_rn(__dadd_rn(a.r, __dmul_rn(a.i, rat)), scl), __dmul_rn(__dsub_rn(a.i, __dmul_rn(a.r, rat)), scl));
  }
  const double rat = __ddiv_rn(b.r, b.i), scl = __ddiv_rn(1.0, __dadd_rn(b.i, __dmul_rn(b.r, rat)));
  return mk(__dmul_rn(__dadd_rn(__dmul_rn(a.r, rat), a.i), scl), __dmul_rn(__dsub_rn(__dmul_rn(a.i, rat), a.r), scl));
}
// principal square root: t = sqrt((|x| + |z|) / 2), the other part y / (2t)
__device__ __forceinline__ cx csqrt_p(cx z) {
  if (z.r == 0.0 && z.i == 0.0) return mk(0.0, z.i);
  const double t = sqrt(__dmul_rn(__dadd_rn(fabs(z.r), hypot(z.r, z.i)), 0.5));
  if (z.r >= 0.0) return mk(t, __ddiv_rn(z.i, __dmul_rn(2.0, t)));
  return mk(__ddiv_rn(fabs(z.i), __dmul_rn(2.0, t)), copysign(t, z.i));
}
__device__ __forceinline__ cx cexp_p(cx z) {
  double s, c;
  sincos(z.i, &s, &c);
  const double e = exp(z.r);
  return mk(__dmul_rn(e, c), __dmul_rn(e, s));
}

// In-place LU with partial pivoting on |re| + |im|, the inverse (identity
// columns solved one by one) and the determinant; false for a singular matrix.
__device__ bool lu_inv_det(int n, cx* a, cx* inv, cx& det) {
  int piv[AS_MAXN];
  cx d = mk(1.0, 0.0);
  for (int k = 0; k < n; ++k) {
    int p = k;
    double best = -1.0;
    for (int r = k; r < n; ++r) {
      const double v = __dadd_rn(fabs(a[r * n + k].r), fabs(a[r * n + k].i));
      if (v > best) {
        best = v;
        p = r;
      }
    }
    piv[k] = p;
    if (best == 0.0) return false;
    if (p != k) {
      for (int c = 0; c < n; ++c) {
        const cx t = a[k * n + c];
        a[k * n + c] = a[p * n + c];
        a[p * n + c] = t;
      }
      d = mk(-d.r, -d.i);
    }
    d = cmul(d, a[k * n + k]);
    for (int r = k + 1; r < n; ++r) {
      const cx f = cdiv(a[r * n + k], a[k * n + k]);
      a[r * n + k] = f;
      for (int c = k + 1; c < n; ++c) a[r * n + c] = csub(a[r * n + c], cmul(f, a[k * n + c]));
    }
  }
  det = d;
  for (int col = 0; col < n; ++col) {
    cx x[AS_MAXN];
    for (int r = 0; r < n; ++r) x[r] = mk(r == col ? 1.0 : 0.0, 0.0);
    for (int k = 0; k < n; ++k)
      if (piv[k] != k) {
        const cx t = x[k];
        x[k] = x[piv[k]];
        x[piv[k]] = t;
      }
    for (int r = 1; r < n; ++r)
      for (int c = 0; c < r; ++c) x[r] = csub(x[r], cmul(a[r * n + c], x[c]));
    for (int r = n - 1; r >= 0; --r) {
      for (int c = r + 1; c < n; ++c) x[r] = csub(x[r], cmul(a[r * n + c], x[c]));
      x[r] = cdiv(x[r], a[r * n + r]);
    }
    for (int r = 0; r < n; ++r) inv[r * n + col] = x[r];
  }
  return true;
}

template <int M>
__global__ void __launch_bounds__(128) autoshape_kernel(int64_t B, const double2* __restrict__ Ag,
                                                        const double2* __restrict__ bg, const double2* __restrict__ cg,
                                                        double max_prob, int64_t max_shape, int64_t min_shape,
                                                        int64_t* __restrict__ shapes) {
  const int64_t gid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (gid >= B * M) return;
  const int64_t s = gid / M;
  const int m = (int)(gid - s * M);
  constexpr int n = M - 1, N = 2 * (M - 1), W = 2 * M;
  const double2* A = Ag + s * (int64_t)W * W;
  const double2* b = bg + s * (int64_t)W;
  auto ld = [](const double2* p) {
    const double2 v = __ldg(p);
    return mk(v.x, v.y);
  };
  int idx[AS_MAXM];
  for (int j = 0, t = 0; j < M; ++j)
    if (j != m) idx[t++] = j;
  // reduction to mode m
  cx A1[4], b1[2];
  cx Ann[N > 0 ? N * N : 1], Z[N > 0 ? N * N : 1], Amn[N > 0 ? 2 * N : 1], bn[N > 0 ? N : 1];
  for (int a = 0; a < 2; ++a)
    for (int a2 = 0; a2 < 2; ++a2) {
      A1[a * 2 + a2] = ld(A + (a * M + m) * W + a2 * M + m);
      for (int j = 0; j < n; ++j) Amn[a * N + a2 * n + j] = ld(A + (a * M + m) * W + a2 * M + idx[j]);
    }
  for (int a = 0; a < 2; ++a)
    for (int i = 0; i < n; ++i)
      for (int a2 = 0; a2 < 2; ++a2)
        for (int j = 0; j < n; ++j) {
          const int r = a * n + i, c = a2 * n + j;
          const cx v = ld(A + (a * M + idx[i]) * W + a2 * M + idx[j]);
          const bool x = (r < n) ? (c == r + n) : (c == r - n);
          Ann[r * N + c] = x ? csub(v, mk(1.0, 0.0)) : v;
        }
  for (int a2 = 0; a2 < 2; ++a2)
    for (int j = 0; j < n; ++j) bn[a2 * n + j] = ld(b + a2 * M + idx[j]);
  b1[0] = ld(b + m);
  b1[1] = ld(b + M + m);
  cx det = mk(1.0, 0.0);
  if (N > 0 && !lu_inv_det(N, Ann, Z, det)) {
    shapes[gid] = -1;
    return;
  }
  for (int a = 0; a < 2; ++a) {
    cx T[N > 0 ? N : 1];
    for (int c = 0; c < N; ++c) {
      cx acc = mk(0.0, 0.0);
      for (int t = 0; t < N; ++t) acc = cadd(acc, cmul(Amn[a * N + t], Z[t * N + c]));
      T[c] = acc;
    }
    for (int a2 = 0; a2 < 2; ++a2) {
      cx acc = mk(0.0, 0.0);
      for (int c = 0; c < N; ++c) acc = cadd(acc, cmul(T[c], Amn[a2 * N + c]));
      A1[a * 2 + a2] = csub(A1[a * 2 + a2], acc);
    }
    cx acc = mk(0.0, 0.0);
    for (int c = 0; c < N; ++c) acc = cadd(acc, cmul(T[c], bn[c]));
    b1[a] = csub(b1[a], acc);
  }
  cx q = mk(0.0, 0.0);
  for (int c = 0; c < N; ++c) {
    cx w = mk(0.0, 0.0);
    for (int t = 0; t < N; ++t) w = cadd(w, cmul(cmulr(bn[t], -0.5), Z[t * N + c]));
    q = cadd(q, cmul(w, bn[c]));
  }
  const double2 cv = __ldg(cg + s);
  const cx c1 = cdiv(cmul(mk(cv.x, cv.y), cexp_p(q)), csqrt_p(det));
  // buffered single-mode recurrence (o: buffers of step k, n1: of step k + 1)
  cx buf2[2][2], buf3[2][3];
  for (int u = 0; u < 2; ++u) {
    buf2[u][0] = buf2[u][1] = mk(0.0, 0.0);
    buf3[u][0] = buf3[u][1] = buf3[u][2] = mk(0.0, 0.0);
  }
  buf3[0][1] = c1;
  double norm = hypot(c1.r, c1.i);
  int64_t k = 0;
  double s0 = 0.0, s1 = 1.0, s2 = sqrt(2.0);  // sqrt(k), sqrt(k + 1), sqrt(k + 2), carried over steps
  double y1 = 1.0, y2 = __drcp_rn(s2);          // RN(1 / s1), RN(1 / s2)
  while (norm < max_prob && k < max_shape) {
    const int o = (int)(k & 1), n1 = o ^ 1;
    for (int i = 0; i < 2; ++i) {
      const cx Av = cadd(cmul(A1[i * 2 + 0], buf2[o][0]), cmul(A1[i * 2 + 1], buf2[o][1]));
      buf2[n1][i] = cdivr(cadd(cmul(b1[i], buf3[o][1]), cmulr(Av, s0)), s1, y1);
    }
    buf3[n1][0] = cdivr(
        cadd(cadd(cmul(b1[0], buf2[n1][0]), cmulr(cmul(A1[0], buf3[o][1]), s1)), cmulr(cmul(A1[1], buf3[o][0]), s0)),
        s2, y2);
    buf3[n1][1] = cdivr(
        cadd(cadd(cmul(b1[1], buf2[n1][0]), cmulr(cmul(A1[2], buf3[o][1]), s1)), cmulr(cmul(A1[3], buf3[o][0]), s0)),
        s1, y1);
    buf3[n1][2] = cdivr(
        cadd(cadd(cmul(b1[1], buf2[n1][1]), cmulr(cmul(A1[2], buf3[o][2]), s0)), cmulr(cmul(A1[3], buf3[o][1]), s1)),
        s2, y2);
    norm = __dadd_rn(norm, hypot(buf3[n1][1].r, buf3[n1][1].i));
    ++k;
    s0 = s1;
    s1 = s2;
    y1 = y2;
    s2 = sqrt((double)(k + 2));
    y2 = __drcp_rn(s2);
  }
  if (k < min_shape) k = min_shape;
  if (k > max_shape) k = max_shape;
  shapes[gid] = k;
}

}  // namespace

extern "C" {

// See include/mm_gb300.h.
MM_API int mm_autoshape_batched(int64_t B, int M, const mm_c128* A, const mm_c128* b, const mm_c128* c,
                                double max_prob, int64_t max_shape, int64_t min_shape, int64_t* shapes,
                                mm_stream_t stream) {
  if (B < 0 || M < 1) return MM_ERR_INVALID_ARG;
  if (M > AS_MAXM) return MM_ERR_UNSUPPORTED;
  // the reference's table SQRT = sqrt(arange(100000)) is read at k + 2 <= max_shape + 1
  if (max_shape > 99998) return MM_ERR_TOO_LARGE;
  if (B == 0) return MM_OK;
  if (!A || !b || !c || !shapes) return MM_ERR_INVALID_ARG;
  const int64_t threads = B * M;
  if ((threads + 127) / 128 > INT32_MAX) return MM_ERR_TOO_LARGE;
  const dim3 grid((unsigned)((threads + 127) / 128));
  cudaStream_t st = (cudaStream_t)stream;
  const double2 *Ad = (const double2*)A, *bd = (const double2*)b, *cd = (const double2*)c;
  switch (M) {
#define MM_AS_CASE(MM)                                                                                        \
  case MM:                                                                                                    \
    autoshape_kernel<MM><<<grid, 128, 0, st>>>(B, Ad, bd, cd, max_prob, max_shape, min_shape, shapes); \
    break;
    MM_AS_CASE(1)
    MM_AS_CASE(2)
    MM_AS_CASE(3)
    MM_AS_CASE(4)
    MM_AS_CASE(5)
    MM_AS_CASE(6)
    MM_AS_CASE(7)
    MM_AS_CASE(8)
#undef MM_AS_CASE
  }
  mm::note_launches(1);
  return cudaGetLastError() == cudaSuccess ? MM_OK : MM_ERR_CUDA;
}

}  // extern "C"
