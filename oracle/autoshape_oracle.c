/*
 * CPU oracle for autoshape.  TEST INFRASTRUCTURE ONLY: the tests' checker and
 * the timed CPU baseline of bench.py; never linked into the product library.
 *
 * Restates autoshape_numba (mrmustard/math/lattice/autoshape.py:23-154), called
 * by State.auto_shape (mrmustard/lab/states/base.py:383-430) on the density-
 * matrix triple of a state (2M x 2M A, 2M-vector b, scalar c; the first M
 * variables belong to the bra copy, the last M to the ket copy):
 *   for every mode m (autoshape.py:110-128):
 *     n = the other M-1 modes; X = [[0, I], [I, 0]] of size 2(M-1);
 *     Z = inv(A_nn - X); A_ = A_mm - (A_mn Z) A_mn^T; b_ = b_m - (A_mn Z) b_n;
 *     c_ = c exp(-1/2 (b_n Z) b_n) / sqrt(det(A_nn - X))
 *     (A_nm is taken as A_mn^T, as the reference does);
 *   then the buffered single-mode recurrence of autoshape.py:130-152 (two
 *   2-element and two 3-element buffers, indices mod 2) adds |rho_kk| until
 *   the sum reaches max_prob or k reaches max_shape; shape[m] = k;
 *   finally np.clip(shape, min_shape, max_shape) (autoshape.py:154).
 * Blocks are picked with the reference's index order (A reshaped (2, M, 2, M),
 * rows and columns ordered copy-major).  inv and det use an LU factorisation
 * with partial pivoting on |re| + |im| (LAPACK's choice), the determinant as
 * the product of U's diagonal (numba's det; numpy's goes through slogdet, one
 * ulp apart); sqrt and exp of a complex number are C99's csqrt and cexp
 * (numpy's npy_csqrt / npy_cexp).
 * Complex arithmetic, the complex/real division (both lowerings, selected by
 * oracle_set_numpy_division, defined in hermite_oracle.c) and matrix-vector
 * orders follow the reference's expressions term by term.  Parity is pinned
 * against the reference source's own outputs (tests/golden/autoshape_golden.npz,
 * tests/golden/make_autoshape_golden.py).
 */
#include <complex.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

typedef double _Complex cplx;

#define AS_MAXM 16
#define AS_MAXN (2 * (AS_MAXM - 1))

extern int oracle_numpy_division(void);

static inline cplx mul(cplx a, cplx b) {
  double ar = creal(a), ai = cimag(a), br = creal(b), bi = cimag(b);
  return CMPLX(ar * br - ai * bi, ar * bi + ai * br);
}
static inline cplx add(cplx a, cplx b) { return CMPLX(creal(a) + creal(b), cimag(a) + cimag(b)); }
static inline cplx sub(cplx a, cplx b) { return CMPLX(creal(a) - creal(b), cimag(a) - cimag(b)); }
/* complex * real, the real promoted to (s, 0) */
static inline cplx mulr(cplx a, double s) {
  double ar = creal(a), ai = cimag(a);
  return CMPLX(ar * s - ai * 0.0, ar * 0.0 + ai * s);
}
/* complex / real: numba's lowering, or numpy's reciprocal multiply */
static inline cplx divr(cplx a, double d) {
  double ar = creal(a), ai = cimag(a);
  if (oracle_numpy_division()) {
    double scl = 1.0 / (d + 0.0 * 0.0);
    return CMPLX((ar + ai * 0.0) * scl, (ai - ar * 0.0) * scl);
  }
  return CMPLX((ar + ai * 0.0) / d, (ai - ar * 0.0) / d);
}
/* full complex division (LU solves), Smith's algorithm as numpy's loops */
static inline cplx cdiv(cplx a, cplx b) {
  double ar = creal(a), ai = cimag(a), br = creal(b), bi = cimag(b);
  if (fabs(br) >= fabs(bi)) {
    double rat = bi / br, scl = 1.0 / (br + bi * rat);
    return CMPLX((ar + ai * rat) * scl, (ai - ar * rat) * scl);
  }
  double rat = br / bi, scl = 1.0 / (bi + br * rat);
  return CMPLX((ar * rat + ai) * scl, (ai * rat - ar) * scl);
}

/* In-place LU with partial pivoting (pivot: largest |re| + |im|), then the
 * inverse (columns of the identity solved one by one) and the determinant.
 * Returns 0, or 1 for a singular matrix. */
static int lu_inv_det(int n, cplx* a, cplx* inv, cplx* det) {
  int piv[AS_MAXN];
  cplx d = CMPLX(1.0, 0.0);
  for (int k = 0; k < n; ++k) {
    int p = k;
    double best = -1.0;
    for (int r = k; r < n; ++r) {
      double v = fabs(creal(a[r * n + k])) + fabs(cimag(a[r * n + k]));
      if (v > best) {
        best = v;
        p = r;
      }
    }
    piv[k] = p;
    if (best == 0.0) return 1;
    if (p != k) {
      for (int c = 0; c < n; ++c) {
        cplx t = a[k * n + c];
        a[k * n + c] = a[p * n + c];
        a[p * n + c] = t;
      }
      d = CMPLX(-creal(d), -cimag(d));
    }
    d = mul(d, a[k * n + k]);
    for (int r = k + 1; r < n; ++r) {
      cplx f = cdiv(a[r * n + k], a[k * n + k]);
      a[r * n + k] = f;
      for (int c = k + 1; c < n; ++c) a[r * n + c] = sub(a[r * n + c], mul(f, a[k * n + c]));
    }
  }
  *det = d;
  for (int col = 0; col < n; ++col) {
    cplx x[AS_MAXN];
    for (int r = 0; r < n; ++r) x[r] = CMPLX(r == col ? 1.0 : 0.0, 0.0);
    /* apply the row swaps, forward (unit lower), backward (upper) */
    for (int k = 0; k < n; ++k)
      if (piv[k] != k) {
        cplx t = x[k];
        x[k] = x[piv[k]];
        x[piv[k]] = t;
      }
    for (int r = 1; r < n; ++r)
      for (int c = 0; c < r; ++c) x[r] = sub(x[r], mul(a[r * n + c], x[c]));
    for (int r = n - 1; r >= 0; --r) {
      for (int c = r + 1; c < n; ++c) x[r] = sub(x[r], mul(a[r * n + c], x[c]));
      x[r] = cdiv(x[r], a[r * n + r]);
    }
    for (int r = 0; r < n; ++r) inv[r * n + col] = x[r];
  }
  return 0;
}

/* Single-mode (A_, b_, c_) of mode m (autoshape.py:110-128). */
static int reduce_mode(int M, const cplx* A, const cplx* b, cplx c, int m, cplx A1[4], cplx b1[2], cplx* c1) {
  const int n = M - 1, N = 2 * n;
  int idx[AS_MAXM];
  for (int j = 0, t = 0; j < M; ++j)
    if (j != m) idx[t++] = j;
  cplx Ann[AS_MAXN * AS_MAXN], Z[AS_MAXN * AS_MAXN], Amn[2 * AS_MAXN], bn[AS_MAXN];
  for (int a = 0; a < 2; ++a)
    for (int i = 0; i < n; ++i) {
      const int r = a * n + i;
      for (int a2 = 0; a2 < 2; ++a2)
        for (int j = 0; j < n; ++j) {
          const int s = a2 * n + j;
          cplx v = A[(a * M + idx[i]) * 2 * M + a2 * M + idx[j]];
          const int x = (r < n) ? (s == r + n) : (s == r - n);
          Ann[r * N + s] = x ? sub(v, CMPLX(1.0, 0.0)) : v;
        }
    }
  for (int a = 0; a < 2; ++a)
    for (int a2 = 0; a2 < 2; ++a2) {
      A1[a * 2 + a2] = A[(a * M + m) * 2 * M + a2 * M + m];
      for (int j = 0; j < n; ++j) Amn[a * N + a2 * n + j] = A[(a * M + m) * 2 * M + a2 * M + idx[j]];
    }
  for (int a2 = 0; a2 < 2; ++a2)
    for (int j = 0; j < n; ++j) bn[a2 * n + j] = b[a2 * M + idx[j]];
  b1[0] = b[m];
  b1[1] = b[M + m];
  cplx det = CMPLX(1.0, 0.0);
  if (N > 0 && lu_inv_det(N, Ann, Z, &det)) return 1;
  /* T = A_mn Z; A_ -= T A_mn^T; b_ -= T b_n */
  cplx T[2 * AS_MAXN];
  for (int a = 0; a < 2; ++a)
    for (int s = 0; s < N; ++s) {
      cplx acc = CMPLX(0.0, 0.0);
      for (int t = 0; t < N; ++t) acc = add(acc, mul(Amn[a * N + t], Z[t * N + s]));
      T[a * N + s] = acc;
    }
  for (int a = 0; a < 2; ++a) {
    for (int a2 = 0; a2 < 2; ++a2) {
      cplx acc = CMPLX(0.0, 0.0);
      for (int s = 0; s < N; ++s) acc = add(acc, mul(T[a * N + s], Amn[a2 * N + s]));
      A1[a * 2 + a2] = sub(A1[a * 2 + a2], acc);
    }
    cplx acc = CMPLX(0.0, 0.0);
    for (int s = 0; s < N; ++s) acc = add(acc, mul(T[a * N + s], bn[s]));
    b1[a] = sub(b1[a], acc);
  }
  /* q = ((-1/2 b_n) Z) b_n, the reference's left-to-right evaluation */
  cplx q = CMPLX(0.0, 0.0);
  for (int s = 0; s < N; ++s) {
    cplx w = CMPLX(0.0, 0.0);
    for (int t = 0; t < N; ++t) w = add(w, mul(mulr(bn[t], -0.5), Z[t * N + s]));
    q = add(q, mul(w, bn[s]));
  }
  *c1 = cdiv(mul(c, cexp(q)), csqrt(det));
  return 0;
}

/* The buffered recurrence of autoshape.py:130-152; returns k. */
static int64_t mode_cutoff(const cplx A[4], const cplx b[2], cplx c, double max_prob, int64_t max_shape) {
  cplx buf2[2][2] = {{0}}, buf3[2][3] = {{0}};
  buf3[0][1] = c;
  double norm = cabs(c);
  int64_t k = 0;
  while (norm < max_prob && k < max_shape) {
    const int o = (int)(k % 2), n = (int)((k + 1) % 2);
    const double s0 = sqrt((double)k), s1 = sqrt((double)(k + 1)), s2 = sqrt((double)(k + 2));
    for (int i = 0; i < 2; ++i) {
      cplx Av = add(mul(A[i * 2 + 0], buf2[o][0]), mul(A[i * 2 + 1], buf2[o][1]));
      buf2[n][i] = divr(add(mul(b[i], buf3[o][1]), mulr(Av, s0)), s1);
    }
    buf3[n][0] = divr(add(add(mul(b[0], buf2[n][0]), mulr(mul(A[0], buf3[o][1]), s1)), mulr(mul(A[1], buf3[o][0]), s0)),
                      s2);
    buf3[n][1] = divr(add(add(mul(b[1], buf2[n][0]), mulr(mul(A[2], buf3[o][1]), s1)), mulr(mul(A[3], buf3[o][0]), s0)),
                      s1);
    buf3[n][2] = divr(add(add(mul(b[1], buf2[n][1]), mulr(mul(A[2], buf3[o][2]), s0)), mulr(mul(A[3], buf3[o][1]), s1)),
                      s2);
    norm += cabs(buf3[n][1]);
    ++k;
  }
  return k;
}

/* One state: shape[M]; returns 0, 1 for bad arguments, 2 for a singular reduction. */
int oracle_autoshape(int M, const cplx* A, const cplx* b, const cplx* c, double max_prob, int64_t max_shape,
                     int64_t min_shape, int64_t* shape) {
  if (M < 1 || M > AS_MAXM) return 1;
  for (int m = 0; m < M; ++m) {
    cplx A1[4], b1[2], c1;
    if (reduce_mode(M, A, b, *c, m, A1, b1, &c1)) return 2;
    int64_t k = mode_cutoff(A1, b1, c1, max_prob, max_shape);
    if (k < min_shape) k = min_shape;
    if (k > max_shape) k = max_shape;
    shape[m] = k;
  }
  return 0;
}

/* Ragged set of states, OpenMP over states: state s has M[s] modes, its A at
 * A + a_off[s] ((2M)^2 entries), b at b + b_off[s] (2M), c[s], shape at shape + s_off[s]. */
int oracle_autoshape_ragged(int64_t B, const int32_t* M, const int64_t* a_off, const int64_t* b_off,
                            const int64_t* s_off, const cplx* A, const cplx* b, const cplx* c, double max_prob,
                            int64_t max_shape, int64_t min_shape, int64_t* shape) {
  int bad = 0;
#pragma omp parallel for schedule(dynamic, 8) reduction(| : bad)
  for (int64_t s = 0; s < B; ++s)
    bad |= oracle_autoshape(M[s], A + a_off[s], b + b_off[s], c + s, max_prob, max_shape, min_shape, shape + s_off[s]);
  return bad;
}
