/*
 * CPU oracle for the Gaussian->Fock hot path.  TEST INFRASTRUCTURE ONLY.
 *
 * This file is a plain-C restatement of MrMustard's numba strategies, used by
 * the tests as the checker and by bench.py as the timed CPU baseline.  It is
 * never linked into, or called by, the product library.
 *
 * Each function follows the reference's loop order and operation order:
 *   oracle_vanilla      mrmustard/math/lattice/strategies/vanilla/core.py:25-124
 *   oracle_stable       mrmustard/math/lattice/strategies/vanilla/core.py:127-213
 *   oracle_vjp          mrmustard/math/lattice/strategies/vanilla/gradients.py:25-82
 *   oracle_*_batch      vanilla/batch.py:27-61 and gradients.py:85-116 (prange -> OpenMP)
 *   oracle_*_ragged     a per-instance loop of the above (the reference has no
 *                       ragged entry point; its batch API needs one shape)
 *
 * Arithmetic follows numba's lowering of the reference source: complex
 * products are (ar*br - ai*bi, ar*bi + ai*br) with no fused multiply-add
 * (build with -ffp-contract=off), complex/real is component-wise division,
 * numpy's negative-index wraparound is reproduced, and the final
 * sum(G*dLdG) is a sequential loop as numba compiles np.sum.
 * Parity of this restatement is pinned against outputs of the reference source
 * itself (tests/golden/hermite_golden.npz, generated by
 * tests/golden/make_golden.py).
 */
#include <complex.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

typedef double _Complex cplx;

#define ORACLE_MAXD 32

/* SQRT[n] = sqrt(n): correctly rounded, as np.sqrt(np.arange(100000)) (core.py:22). */
static inline double sq(int64_t n) { return sqrt((double)n); }

static inline cplx cmul(cplx a, cplx b) {
  double ar = creal(a), ai = cimag(a), br = creal(b), bi = cimag(b);
  return CMPLX(ar * br - ai * bi, ar * bi + ai * br);
}
/* complex * real as numba lowers it: the real operand is promoted to (s, 0). */
static inline cplx cmulr(cplx a, double s) {
  double ar = creal(a), ai = cimag(a);
  return CMPLX(ar * s - ai * 0.0, ar * 0.0 + ai * s);
}
static inline cplx cadd(cplx a, cplx b) { return CMPLX(creal(a) + creal(b), cimag(a) + cimag(b)); }
/*
 * complex / real.  numba lowers it as CPython's _Py_c_quot with b = (d, 0):
 * ((ar + ai*0)/d, (ai - ar*0)/d).  numpy's scalar loop (what the reference source
 * runs as plain CPython) multiplies by scl = 1/(d + 0*0) instead.  The default is
 * numba's lowering; oracle_set_numpy_division(1) selects numpy's, with which this
 * restatement reproduces the reference source run under CPython bit for bit.
 */
static int g_numpy_div = 0;
void oracle_set_numpy_division(int on) { g_numpy_div = on; }
int oracle_numpy_division(void) { return g_numpy_div; }
static inline cplx cdivr(cplx a, double d) {
  double ar = creal(a), ai = cimag(a);
  if (g_numpy_div) {
    double scl = 1.0 / (d + 0.0 * 0.0);
    return CMPLX((ar + ai * 0.0) * scl, (ai - ar * 0.0) * scl);
  }
  return CMPLX((ar + ai * 0.0) / d, (ai - ar * 0.0) / d);
}
/* numpy's complex division (Smith's method), used for dLdc = sum / c. */
static inline cplx cdiv(cplx a, cplx b) {
  double ar = creal(a), ai = cimag(a), br = creal(b), bi = cimag(b);
  if (fabs(br) >= fabs(bi)) {
    double rat = bi / br, den = br + bi * rat;
    return CMPLX((ar + ai * rat) / den, (ai - ar * rat) / den);
  }
  double rat = br / bi, den = bi + br * rat;
  return CMPLX((ar * rat + ai) / den, (ai * rat - ar) / den);
}

/* numpy flat indexing with one wraparound for negative indices. */
static inline cplx rd(const cplx *G, int64_t n, int64_t idx) {
  if (idx < 0) idx += n;
  if (idx < 0 || idx >= n) return 0.0; /* numba reads out of bounds here; the product is x*0 */
  return G[idx];
}

static int64_t strides_of(int D, const int64_t *shape, int64_t *strides) {
  strides[D - 1] = 1;
  for (int i = D - 1; i > 0; --i) strides[i - 1] = strides[i] * shape[i];
  return strides[0] * shape[0];
}

static inline void next_index(int D, const int64_t *shape, int64_t *idx) {
  for (int d = D - 1; d >= 0; --d) {
    if (++idx[d] < shape[d]) return;
    idx[d] = 0;
  }
}

/* vanilla_numba (core.py:25-124).  G must hold prod(shape) elements; it is fully written. */
int oracle_vanilla(int D, const int64_t *shape, const cplx *A, const cplx *b, const cplx *cp, cplx *G) {
  cplx c = *cp;
  if (D < 1 || D > ORACLE_MAXD) return 1;
  int64_t strides[ORACLE_MAXD], idx[ORACLE_MAXD];
  int64_t n = strides_of(D, shape, strides);
  if (n <= 0) return 0;
  memset(G, 0, (size_t)n * sizeof(cplx)); /* np.zeros when out is None (core.py:73) */
  memset(idx, 0, sizeof(idx));
  G[0] = c;
  /* face loop with pivot search (core.py:85-104) */
  for (int64_t f = 1; f < strides[0] && f < n; ++f) {
    next_index(D, shape, idx);
    int i = 0;
    int64_t pivot = 0;
    for (int s = 0; s < D; ++s) {
      pivot = f - strides[s];
      if (pivot >= 0) break;
      ++i;
    }
    cplx v = cmul(b[i], rd(G, n, pivot));
    v = cadd(v, cmul(cmulr(A[i * D + i], sq(idx[i] - 1)), rd(G, n, pivot - strides[i])));
    for (int j = i + 1; j < D; ++j)
      v = cadd(v, cmul(cmulr(A[i * D + j], sq(idx[j])), rd(G, n, pivot - strides[j])));
    G[f] = cdivr(v, sq(idx[i]));
  }
  /* bulk loop, pivot on axis 0 (core.py:108-122) */
  for (int64_t f = strides[0]; f < n; ++f) {
    next_index(D, shape, idx);
    int64_t pivot = f - strides[0];
    cplx v = cmul(b[0], G[pivot]);
    v = cadd(v, cmul(cmulr(A[0], sq(idx[0] - 1)), rd(G, n, pivot - strides[0])));
    for (int j = 1; j < D; ++j) v = cadd(v, cmul(cmulr(A[j], sq(idx[j])), rd(G, n, pivot - strides[j])));
    G[f] = cdivr(v, sq(idx[0]));
  }
  return 0;
}

/* stable_numba (core.py:127-213). */
int oracle_stable(int D, const int64_t *shape, const cplx *A, const cplx *b, const cplx *cp, cplx *G) {
  cplx c = *cp;
  if (D < 1 || D > ORACLE_MAXD) return 1;
  int64_t strides[ORACLE_MAXD], idx[ORACLE_MAXD];
  int64_t n = strides_of(D, shape, strides);
  if (n <= 0) return 0;
  memset(G, 0, (size_t)n * sizeof(cplx));
  memset(idx, 0, sizeof(idx));
  G[0] = c;
  for (int64_t f = 1; f < n; ++f) {
    next_index(D, shape, idx);
    int npiv = 0;
    cplx vals = 0.0;
    for (int i = 0; i < D; ++i) {
      if (idx[i] == 0) continue;
      ++npiv;
      int64_t pivot = f - strides[i];
      cplx v = cmul(b[i], G[pivot]);
      for (int j = 0; j < i; ++j)
        v = cadd(v, cmul(cmulr(A[i * D + j], sq(idx[j])), rd(G, n, pivot - strides[j])));
      v = cadd(v, cmul(cmulr(A[i * D + i], sq(idx[i] - 1)), rd(G, n, pivot - strides[i])));
      for (int j = i + 1; j < D; ++j)
        v = cadd(v, cmul(cmulr(A[i * D + j], sq(idx[j])), rd(G, n, pivot - strides[j])));
      vals = cadd(vals, cdivr(v, sq(idx[i])));
    }
    G[f] = cdivr(vals, (double)npiv);
  }
  return 0;
}

/* vanilla_vjp_numba (gradients.py:25-82).  dA is D x D row-major, db has D entries. */
int oracle_vjp(int D, const int64_t *shape, const cplx *G, const cplx *cp, const cplx *dLdG, cplx *dA_out,
               cplx *db_out, cplx *dc_out) {
  cplx c = *cp;
  if (D < 1 || D > ORACLE_MAXD) return 1;
  int64_t strides[ORACLE_MAXD], idx[ORACLE_MAXD];
  int64_t n = strides_of(D, shape, strides);
  cplx *dLdA = (cplx *)calloc((size_t)D * D, sizeof(cplx));
  cplx *dA = (cplx *)calloc((size_t)D * D, sizeof(cplx));
  cplx db[ORACLE_MAXD], dLdb[ORACLE_MAXD];
  if (!dLdA || !dA) {
    free(dLdA);
    free(dA);
    return 3;
  }
  for (int i = 0; i < D; ++i) db[i] = dLdb[i] = 0.0;
  memset(idx, 0, sizeof(idx));
  for (int64_t f = 1; f < n; ++f) {
    next_index(D, shape, idx);
    for (int i = 0; i < D; ++i) {
      int64_t pivot = f - strides[i];
      db[i] = cmulr(rd(G, n, pivot), sq(idx[i]));
      dA[i * D + i] = idx[i] > 1 ? cmulr(rd(G, n, pivot - strides[i]), 0.5 * sq(idx[i]) * sq(idx[i] - 1)) : 0.0;
      for (int j = i + 1; j < D; ++j) dA[i * D + j] = cmulr(rd(G, n, pivot - strides[j]), sq(idx[i]) * sq(idx[j]));
    }
    cplx g = dLdG[f];
    for (int k = 0; k < D * D; ++k) dLdA[k] = cadd(dLdA[k], cmul(dA[k], g));
    for (int i = 0; i < D; ++i) dLdb[i] = cadd(dLdb[i], cmul(db[i], g));
  }
  cplx s = 0.0;
  for (int64_t f = 0; f < n; ++f) s = cadd(s, cmul(G[f], dLdG[f]));
  *dc_out = cdiv(s, c);
  for (int i = 0; i < D; ++i) {
    db_out[i] = dLdb[i];
    for (int j = 0; j < D; ++j) {
      cplx t = cadd(dLdA[i * D + j], dLdA[j * D + i]);
      dA_out[i * D + j] = CMPLX(creal(t) / 2.0, cimag(t) / 2.0);
    }
  }
  free(dLdA);
  free(dA);
  return 0;
}

/* ------------------------------------------------------------------ batches */

static int64_t prod64(int D, const int64_t *shape) {
  int64_t n = 1;
  for (int i = 0; i < D; ++i) n *= shape[i];
  return n;
}

/* vanilla_batch_numba (batch.py:27-61): one shape, instances in parallel. */
int oracle_fwd_batch(int64_t B, int D, const int64_t *shape, const cplx *A, const cplx *b, const cplx *c, int stable,
                     cplx *G) {
  int64_t n = prod64(D, shape);
  int err = 0;
#pragma omp parallel for schedule(dynamic, 1) reduction(| : err)
  for (int64_t k = 0; k < B; ++k) {
    err |= stable ? oracle_stable(D, shape, A + k * D * D, b + k * D, c + k, G + k * n)
                  : oracle_vanilla(D, shape, A + k * D * D, b + k * D, c + k, G + k * n);
  }
  return err;
}

/* vanilla_batch_vjp_numba (gradients.py:85-116). */
int oracle_vjp_batch(int64_t B, int D, const int64_t *shape, const cplx *G, const cplx *c, const cplx *dLdG, cplx *dA,
                     cplx *db, cplx *dc) {
  int64_t n = prod64(D, shape);
  int err = 0;
#pragma omp parallel for schedule(dynamic, 1) reduction(| : err)
  for (int64_t k = 0; k < B; ++k)
    err |= oracle_vjp(D, shape, G + k * n, c + k, dLdG + k * n, dA + k * D * D, db + k * D, dc + k);
  return err;
}

/*
 * Ragged batch: instance k has D[k] modes and shape shapes[shape_off[k] .. +D[k]).
 * A/b/G/dLdG are packed back to back; a_off/b_off/g_off give each instance's
 * element offset.  Instances run in parallel, largest first.
 */
int oracle_fwd_ragged(int64_t B, const int32_t *D, const int64_t *shapes, const int64_t *shape_off, const cplx *A,
                      const int64_t *a_off, const cplx *b, const int64_t *b_off, const cplx *c, int stable, cplx *G,
                      const int64_t *g_off, const int64_t *order) {
  int err = 0;
#pragma omp parallel for schedule(dynamic, 1) reduction(| : err)
  for (int64_t t = 0; t < B; ++t) {
    int64_t k = order ? order[t] : t;
    const int64_t *sh = shapes + shape_off[k];
    err |= stable ? oracle_stable(D[k], sh, A + a_off[k], b + b_off[k], c + k, G + g_off[k])
                  : oracle_vanilla(D[k], sh, A + a_off[k], b + b_off[k], c + k, G + g_off[k]);
  }
  return err;
}

int oracle_vjp_ragged(int64_t B, const int32_t *D, const int64_t *shapes, const int64_t *shape_off, const cplx *G,
                      const int64_t *g_off, const cplx *c, const cplx *dLdG, cplx *dA, const int64_t *a_off, cplx *db,
                      const int64_t *b_off, cplx *dc, const int64_t *order) {
  int err = 0;
#pragma omp parallel for schedule(dynamic, 1) reduction(| : err)
  for (int64_t t = 0; t < B; ++t) {
    int64_t k = order ? order[t] : t;
    err |= oracle_vjp(D[k], shapes + shape_off[k], G + g_off[k], c + k, dLdG + g_off[k], dA + a_off[k], db + b_off[k],
                      dc + k);
  }
  return err;
}

int oracle_num_threads(void) {
#ifdef _OPENMP
  extern int omp_get_max_threads(void);
  return omp_get_max_threads();
#else
  return 1;
#endif
}
