/*
 * CPU oracle for the binomial strategy.  TEST INFRASTRUCTURE ONLY: the tests'
 * checker and the timed CPU baseline of bench.py; never linked into the
 * product library.
 *
 * Restates binomial(local_cutoffs, A, b, c, max_l2, global_cutoff)
 * (mrmustard/math/lattice/strategies/binomial.py:30-70), reached through
 * math.hermite_renormalized_binomial (mrmustard/math/backend_manager.py:790-814,
 * backend_numpy.py:405-421):
 *   G[0] = c, norm = |c|^2; for photons = 1 .. global_cutoff-1: every index of
 *   that total photon number inside the local cutoffs, in the order of
 *   paths.binomial_subspace_basis (paths.py:20-72: mode 0 outermost, ascending),
 *   is computed by steps.vanilla_step (steps.py:15-42):
 *     i = first non-zero axis (pivots.first_available_pivot), p = index - 1_i,
 *     value = b_i G[p] + sum_{j=0}^{D-1} A_ij sqrt(p_j) G[p - 1_j]   (all j; a
 *     -1 coordinate wraps around as numpy/numba index it, times sqrt(0) = 0),
 *     G[index] = value / sqrt(index_i);
 *   the subspace adds sum |value|^2 to norm; the fill stops after the first
 *   subspace with norm > max_l2.  Returns norm.
 * Complex arithmetic follows the reference's expressions term by term (no fused
 * multiply-add: build with -ffp-contract=off); the complex/real division has
 * both lowerings (oracle_set_numpy_division, hermite_oracle.c).  Parity is
 * pinned against the reference source's own outputs
 * (tests/golden/binomial_golden.npz, tests/golden/make_binomial_golden.py).
 */
#include <complex.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

typedef double _Complex cplx;

#define BN_MAXD 32

extern int oracle_numpy_division(void);

static inline cplx bmul(cplx a, cplx b) {
  double ar = creal(a), ai = cimag(a), br = creal(b), bi = cimag(b);
  return CMPLX(ar * br - ai * bi, ar * bi + ai * br);
}
static inline cplx badd(cplx a, cplx b) { return CMPLX(creal(a) + creal(b), cimag(a) + cimag(b)); }
static inline cplx bmulr(cplx a, double s) {
  double ar = creal(a), ai = cimag(a);
  return CMPLX(ar * s - ai * 0.0, ar * 0.0 + ai * s);
}
static inline cplx bdivr(cplx a, double d) {
  double ar = creal(a), ai = cimag(a);
  if (oracle_numpy_division()) {
    double scl = 1.0 / (d + 0.0 * 0.0);
    return CMPLX((ar + ai * 0.0) * scl, (ai - ar * 0.0) * scl);
  }
  return CMPLX((ar + ai * 0.0) / d, (ai - ar * 0.0) / d);
}

/* Fills G (C-order, shape[D], zero-initialised by the caller except nothing);
 * returns the norm; *stop receives the last photon number filled. */
double oracle_binomial(int D, const int64_t* shape, const cplx* A, const cplx* b, const cplx* c, double max_l2,
                       int64_t global_cutoff, cplx* G, int64_t* stop) {
  int64_t strides[BN_MAXD], n = 1;
  for (int j = D - 1; j >= 0; --j) {
    strides[j] = n;
    n *= shape[j];
  }
  memset(G, 0, (size_t)n * sizeof(cplx));
  G[0] = *c;
  double h = cabs(*c);
  double norm = h * h;
  *stop = 0;
  for (int64_t photons = 1; photons < global_cutoff; ++photons) {
    double sub = 0.0;
    /* lexicographic walk over indices of weight `photons` inside the cutoffs */
    int64_t k[BN_MAXD];
    int64_t rest = photons;
    int ok = 1;
    for (int j = 0; j < D; ++j) k[j] = 0;
    /* first element: greedy from the last axis backwards is not lexicographic; build the
       smallest lexicographic index instead: fill the last axes first */
    for (int j = D - 1; j >= 0; --j) {
      int64_t t = rest < shape[j] - 1 ? rest : shape[j] - 1;
      k[j] = t;
      rest -= t;
    }
    if (rest != 0) ok = 0; /* the subspace is empty */
    while (ok) {
      int i = 0;
      while (k[i] == 0) ++i;
      int64_t p[BN_MAXD];
      for (int j = 0; j < D; ++j) p[j] = k[j];
      p[i] -= 1;
      int64_t fp = 0;
      for (int j = 0; j < D; ++j) fp += p[j] * strides[j];
      cplx value = bmul(b[i], G[fp]);
      for (int j = 0; j < D; ++j) {
        int64_t q = p[j] - 1;
        if (q < 0) q += shape[j]; /* numpy / numba wraparound */
        const int64_t fn = fp + (q - p[j]) * strides[j];
        value = badd(value, bmul(bmulr(A[i * D + j], sqrt((double)p[j])), G[fn]));
      }
      value = bdivr(value, sqrt((double)k[i]));
      int64_t f = 0;
      for (int j = 0; j < D; ++j) f += k[j] * strides[j];
      G[f] = value;
      const double a = cabs(value);
      sub = sub + a * a;
      /* next index of the same weight in lexicographic order: find the rightmost axis j < D-1
         that can grow while the axes after it can still hold the remainder */
      int advanced = 0;
      int64_t tail = k[D - 1];
      for (int j = D - 2; j >= 0 && !advanced; --j) {
        /* tail = sum of k over axes > j */
        if (k[j] + 1 < shape[j] && tail >= 1) {
          k[j] += 1;
          int64_t r = tail - 1;
          for (int m = D - 1; m > j; --m) {
            int64_t t = r < shape[m] - 1 ? r : shape[m] - 1;
            k[m] = t;
            r -= t;
          }
          /* r == 0 always: the axes after j could hold `tail`, so they hold tail - 1 */
          advanced = 1;
        } else {
          tail += k[j];
        }
      }
      if (!advanced) break;
    }
    norm += sub;
    *stop = photons;
    if (norm > max_l2) break;
  }
  return norm;
}
