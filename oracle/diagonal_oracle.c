/*
 * CPU oracle for the diagonal strategies.  TEST INFRASTRUCTURE ONLY: the tests'
 * checker and the timed CPU baseline of bench.py; never linked into the product
 * library.
 *
 * 1. compactFock diagonal amplitudes: fock_representation_diagonal_amps
 *    (mrmustard/math/lattice/strategies/compactFock/diagonal_amps.py:17-187), reached
 *    through hermite_multidimensional_diagonal (compactFock/inputValidation.py:61-79) and
 *    math.hermite_renormalized_diagonal (backend_manager.py:729-757,
 *    backend_numpy.py:423-432).  M modes with cutoffs c_0..c_{M-1}; the five arrays of
 *    the reference (arr0, arr2, arr1010, arr1001, arr1, each over the params lattice
 *    and an optional batch axis of B) are stored back to back in one buffer W of
 *    "slots": slot 0 = arr0, 1+d = arr2[d], 1+M+d(M-1)+e = arr1010[d][e],
 *    1+M+M(M-1)+d(M-1)+e = arr1001[d][e], 1+M+2M(M-1)+i = arr1[i]; each slot holds
 *    P*nb values (P = prod c_k, params in C order, batch index last), which is the
 *    reference's own layout of each array.
 * 2. their Jacobians: fock_representation_diagonal_grad
 *    (compactFock/diagonal_grad.py:17-378): every slot value carries d/dA (2M x 2M) and
 *    d/dB (2M), stored as J[slot][P][4M^2 + 2M] (dA row-major, then dB).
 * 3. fast_diagonal (mrmustard/math/lattice/strategies/fast_diagonal.py:32-200), which
 *    backend_numpy.hermite_renormalized_1leftoverMode calls (backend_numpy.py:434-446).
 *
 * Arithmetic follows the reference's expressions term by term (no fused multiply-add:
 * build with -ffp-contract=off).  The reference's `A[i] @ G_in` is a BLAS dot whose
 * summation order is the BLAS library's; here it is the plain left-to-right sum, so
 * parity with the reference is to rounding (pinned against fixtures made from the
 * reference source, tests/golden/make_diagonal_golden.py).
 */
#include <complex.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

typedef double _Complex cplx;

#define DG_MAXM 16

extern int oracle_numpy_division(void);
extern int oracle_vanilla(int D, const int64_t *shape, const cplx *A, const cplx *b, const cplx *cp, cplx *G);
extern int oracle_stable(int D, const int64_t *shape, const cplx *A, const cplx *b, const cplx *cp, cplx *G);

static inline cplx dmul(cplx a, cplx b) {
  double ar = creal(a), ai = cimag(a), br = creal(b), bi = cimag(b);
  return CMPLX(ar * br - ai * bi, ar * bi + ai * br);
}
static inline cplx dadd(cplx a, cplx b) { return CMPLX(creal(a) + creal(b), cimag(a) + cimag(b)); }
/* complex * real with the real promoted to (s, 0), as numpy and numba do */
static inline cplx dmulr(cplx a, double s) {
  double ar = creal(a), ai = cimag(a);
  return CMPLX(ar * s - ai * 0.0, ar * 0.0 + ai * s);
}
static inline cplx ddivr_np(cplx a, double d) { /* numpy: scl = 1/(d + 0*0) */
  double ar = creal(a), ai = cimag(a);
  double scl = 1.0 / (d + 0.0 * 0.0);
  return CMPLX((ar + ai * 0.0) * scl, (ai - ar * 0.0) * scl);
}
static inline cplx ddivr(cplx a, double d) {
  if (oracle_numpy_division()) return ddivr_np(a, d);
  double ar = creal(a), ai = cimag(a);
  return CMPLX((ar + ai * 0.0) / d, (ai - ar * 0.0) / d);
}
static inline double SQ(int64_t n) { return sqrt((double)n); }

/* ------------------------------------------------------------ the params lattice */

typedef struct {
  int M;
  int64_t c[DG_MAXM], st[DG_MAXM], P, nb;
} Lat;

static int lat_init(Lat *L, int M, const int64_t *cutoffs, int64_t nb) {
  if (M < 1 || M > DG_MAXM) return 1;
  L->M = M;
  L->nb = nb;
  L->P = 1;
  for (int k = M - 1; k >= 0; --k) {
    if (cutoffs[k] < 1) return 1;
    L->c[k] = cutoffs[k];
    L->st[k] = L->P;
    L->P *= cutoffs[k];
  }
  return 0;
}
static inline int64_t slot_arr2(const Lat *L, int d) { return 1 + d; }
static inline int64_t slot_1010(const Lat *L, int d, int e) { return 1 + L->M + (int64_t)d * (L->M - 1) + e; }
static inline int64_t slot_1001(const Lat *L, int d, int e) {
  return 1 + L->M + (int64_t)L->M * (L->M - 1) + (int64_t)d * (L->M - 1) + e;
}
static inline int64_t slot_arr1(const Lat *L, int i) { return 1 + L->M + 2 * (int64_t)L->M * (L->M - 1) + i; }
int64_t oracle_diagonal_slots(int M) { return 1 + M + 2 * (int64_t)M * (M - 1) + 2 * M; }

/* params lattice points in the order of construct_dict_params (helperFunctions.py:29-45):
 * grouped by sum, np.ndindex (C) order inside a group. */
static int64_t *params_by_weight(const Lat *L, int64_t *nweights) {
  int64_t W = 1;
  for (int k = 0; k < L->M; ++k) W += L->c[k] - 1;
  int64_t *order = (int64_t *)malloc((size_t)L->P * sizeof(int64_t));
  int64_t pos = 0;
  for (int64_t s = 0; s < W; ++s)
    for (int64_t f = 0; f < L->P; ++f) {
      int64_t w = 0, r = f;
      for (int k = 0; k < L->M; ++k) {
        w += r / L->st[k];
        r %= L->st[k];
      }
      if (w == s) order[pos++] = f;
    }
  *nweights = W;
  return order;
}

/* ---------------------------------------------------- 1. diagonal amplitudes */

#define AT(slot, f, col) W[((slot) * L->P + (f)) * L->nb + (col)]

/* A[i] @ G_in + GB[i], then / K_i (diagonal_amps.py:83-88, :131-136) */
static cplx row_dot(const Lat *L, const cplx *A, int i, const cplx *Gin) {
  const int n = 2 * L->M;
  cplx acc = 0.0;
  for (int l = 0; l < n; ++l) acc = dadd(acc, dmul(A[i * n + l], Gin[l]));
  return acc;
}

/* use_diag_pivot (diagonal_amps.py:92-137) for one batch column */
static void diag_pivot(const Lat *L, const cplx *A, const cplx *B, const int64_t *p, int64_t f, int64_t col,
                       cplx *W) {
  const int M = L->M, n = 2 * M;
  cplx Gin[2 * DG_MAXM];
  const cplx g = AT(0, f, col);
  for (int i = 0; i < n; ++i) {
    Gin[i] = 0.0;
    if (p[i / 2] > 0) Gin[i] = AT(slot_arr1(L, i + 1 - 2 * (i % 2)), f - L->st[i / 2], col);
  }
  for (int i = 0; i < n; ++i) Gin[i] = dmulr(Gin[i], SQ(p[i / 2]));
  for (int i = 0; i < n; ++i) {
    if (p[i / 2] + 1 < L->c[i / 2] && (i != 1 || p[0] + 2 < L->c[0])) {
      const cplx GB = dmul(g, B[i * L->nb + col]);
      AT(slot_arr1(L, i), f, col) = ddivr(dadd(GB, row_dot(L, A, i, Gin)), SQ(p[i / 2] + 1));
    }
  }
}

/* use_offDiag_pivot (diagonal_amps.py:17-89) for one batch column */
static void offdiag_pivot(const Lat *L, const cplx *A, const cplx *B, const int64_t *p, int64_t f, int d, int64_t col,
                          cplx *W) {
  const int M = L->M, n = 2 * M;
  cplx Gin[2 * DG_MAXM];
  double Kl[2 * DG_MAXM], Ki[2 * DG_MAXM];
  for (int k = 0; k < M; ++k) {
    Kl[2 * k] = SQ(p[k] + (k == d));
    Kl[2 * k + 1] = SQ(p[k]);
    Ki[2 * k] = SQ(p[k] + (k == d) + 1);
    Ki[2 * k + 1] = SQ(p[k] + 1);
  }
  const cplx g = AT(slot_arr1(L, 2 * d), f, col);
  for (int i = 0; i < n; ++i) Gin[i] = 0.0;
  Gin[2 * d] = AT(0, f, col);
  if (p[d] > 0) Gin[2 * d + 1] = AT(slot_arr2(L, d), f - L->st[d], col);
  for (int i = d + 1; i < M; ++i)
    if (p[i] > 0) {
      Gin[2 * i] = AT(slot_1001(L, d, i - d - 1), f - L->st[i], col);
      Gin[2 * i + 1] = AT(slot_1010(L, d, i - d - 1), f - L->st[i], col);
    }
  for (int i = 0; i < n; ++i) Gin[i] = dmulr(Gin[i], Kl[i]);
#define OUT(row) ddivr(dadd(dmul(g, B[(row) * L->nb + col]), row_dot(L, A, (row), Gin)), Ki[row])
  AT(0, f + L->st[d], col) = OUT(2 * d + 1);
  if (p[d] + 2 < L->c[d]) AT(slot_arr2(L, d), f, col) = OUT(2 * d);
  for (int i = d + 1; i < M; ++i)
    if (p[i] + 1 < L->c[i]) {
      AT(slot_1010(L, d, i - d - 1), f, col) = OUT(2 * i);
      AT(slot_1001(L, d, i - d - 1), f, col) = OUT(2 * i + 1);
    }
#undef OUT
}

/*
 * W: oracle_diagonal_slots(M) * P * nb values, zeroed here; B is (2M, nb) row-major;
 * G0 has nb values (the reference broadcasts one G0 over the batch).
 */
int oracle_diagonal_amps(int M, const int64_t *cutoffs, int64_t nb, const cplx *A, const cplx *B, const cplx *G0,
                         cplx *W) {
  Lat Ls, *L = &Ls;
  if (lat_init(L, M, cutoffs, nb) || nb < 1) return 1;
  memset(W, 0, (size_t)(oracle_diagonal_slots(M) * L->P * nb) * sizeof(cplx));
  for (int64_t col = 0; col < nb; ++col) AT(0, 0, col) = G0[col];
  int64_t nw;
  int64_t *order = params_by_weight(L, &nw);
  int64_t p[DG_MAXM];
  for (int64_t t = 0; t < L->P; ++t) {
    const int64_t f = order[t];
    int64_t r = f;
    for (int k = 0; k < M; ++k) {
      p[k] = r / L->st[k];
      r %= L->st[k];
    }
    for (int64_t col = 0; col < nb; ++col) {
      if (L->c[0] == 1 || p[0] < L->c[0] - 1) diag_pivot(L, A, B, p, f, col, W);
      for (int d = 0; d < M; ++d) {
        int lower_zero = 1;
        for (int k = 0; k < d; ++k) lower_zero &= (p[k] == 0);
        if (lower_zero && p[d] < L->c[d] - 1) offdiag_pivot(L, A, B, p, f, d, col, W);
      }
    }
  }
  free(order);
  return 0;
}
#undef AT

/* ------------------------------------------------------ 2. Jacobians d/dA, d/dB */

/*
 * calc_dA_dB (diagonal_grad.py:17-41) for output row i: the Jacobian of
 * (B_i g + sum_l A_il K_l Gin_l) / K_i, with g the pivot value.
 *   dA = dg_A B_i + sum_l (K_l A_il) dGin_l ; dA[i][l] += K_l Gin_l (after term l)
 *   dB = dg_B B_i ; dB[i] += g ; dB += sum_l (K_l A_il) dGin_l
 * Jrow, Jpiv and Jin[l] point at 4M^2 + 2M values (dA then dB).
 */
static void calc_dA_dB(int M, int i, const cplx *A, const cplx *B, const double *Kl, double Ki, cplx g, const cplx *Jpiv,
                       const cplx *Gin_scaled, const cplx *const *Jin, cplx *Jrow) {
  const int n = 2 * M, nA = n * n;
  for (int q = 0; q < nA; ++q) {
    cplx acc = dmul(Jpiv[q], B[i]);
    for (int l = 0; l < n; ++l) {
      acc = dadd(acc, dmul(dmulr(A[i * n + l], Kl[l]), Jin[l] ? Jin[l][q] : 0.0));
      if (q == i * n + l) acc = dadd(acc, Gin_scaled[l]);
    }
    Jrow[q] = ddivr(acc, Ki);
  }
  for (int r = 0; r < n; ++r) {
    cplx acc = dmul(Jpiv[nA + r], B[i]);
    if (r == i) acc = dadd(acc, g);
    for (int l = 0; l < n; ++l) acc = dadd(acc, dmul(dmulr(A[i * n + l], Kl[l]), Jin[l] ? Jin[l][nA + r] : 0.0));
    Jrow[nA + r] = ddivr(acc, Ki);
  }
}

/*
 * Wv: the forward slots of oracle_diagonal_amps (nb = 1); J: slots * P * (4M^2 + 2M),
 * zeroed here.  Returns the Jacobians of every slot; arr0's are J[0 .. P*(4M^2+2M)).
 */
int oracle_diagonal_grad(int M, const int64_t *cutoffs, const cplx *A, const cplx *B, const cplx *Wv, cplx *J) {
  Lat Ls, *L = &Ls;
  if (lat_init(L, M, cutoffs, 1)) return 1;
  const int n = 2 * M;
  const int64_t nc = (int64_t)n * n + n;
  memset(J, 0, (size_t)(oracle_diagonal_slots(M) * L->P * nc) * sizeof(cplx));
#define V(slot, f) Wv[(slot) * L->P + (f)]
#define JJ(slot, f) (J + ((slot) * L->P + (f)) * nc)
  int64_t nw;
  int64_t *order = params_by_weight(L, &nw);
  int64_t p[DG_MAXM];
  cplx Gin[2 * DG_MAXM];
  const cplx *Jin[2 * DG_MAXM];
  double Kl[2 * DG_MAXM];
  for (int64_t t = 0; t < L->P; ++t) {
    const int64_t f = order[t];
    int64_t r = f;
    for (int k = 0; k < M; ++k) {
      p[k] = r / L->st[k];
      r %= L->st[k];
    }
    /* use_diag_pivot_grad (diagonal_grad.py:201-258) */
    if (L->c[0] == 1 || p[0] < L->c[0] - 1) {
      for (int i = 0; i < n; ++i) {
        Gin[i] = 0.0;
        Jin[i] = NULL;
        Kl[i] = SQ(p[i / 2]);
        if (p[i / 2] > 0) {
          const int64_t s = slot_arr1(L, i + 1 - 2 * (i % 2));
          Gin[i] = V(s, f - L->st[i / 2]);
          Jin[i] = JJ(s, f - L->st[i / 2]);
        }
      }
      for (int i = 0; i < n; ++i) Gin[i] = dmulr(Gin[i], Kl[i]);
      for (int i = 0; i < n; ++i)
        if (p[i / 2] + 1 < L->c[i / 2] && (i != 1 || p[0] + 2 < L->c[0]))
          calc_dA_dB(M, i, A, B, Kl, SQ(p[i / 2] + 1), V(0, f), JJ(0, f), Gin, Jin, JJ(slot_arr1(L, i), f));
    }
    /* use_offDiag_pivot_grad (diagonal_grad.py:44-198) */
    for (int d = 0; d < M; ++d) {
      int lower_zero = 1;
      for (int k = 0; k < d; ++k) lower_zero &= (p[k] == 0);
      if (!(lower_zero && p[d] < L->c[d] - 1)) continue;
      double Ki[2 * DG_MAXM];
      for (int k = 0; k < M; ++k) {
        Kl[2 * k] = SQ(p[k] + (k == d));
        Kl[2 * k + 1] = SQ(p[k]);
        Ki[2 * k] = SQ(p[k] + (k == d) + 1);
        Ki[2 * k + 1] = SQ(p[k] + 1);
      }
      for (int i = 0; i < n; ++i) {
        Gin[i] = 0.0;
        Jin[i] = NULL;
      }
      Gin[2 * d] = V(0, f);
      Jin[2 * d] = JJ(0, f);
      if (p[d] > 0) {
        Gin[2 * d + 1] = V(slot_arr2(L, d), f - L->st[d]);
        Jin[2 * d + 1] = JJ(slot_arr2(L, d), f - L->st[d]);
      }
      for (int i = d + 1; i < M; ++i)
        if (p[i] > 0) {
          Gin[2 * i] = V(slot_1001(L, d, i - d - 1), f - L->st[i]);
          Jin[2 * i] = JJ(slot_1001(L, d, i - d - 1), f - L->st[i]);
          Gin[2 * i + 1] = V(slot_1010(L, d, i - d - 1), f - L->st[i]);
          Jin[2 * i + 1] = JJ(slot_1010(L, d, i - d - 1), f - L->st[i]);
        }
      for (int i = 0; i < n; ++i) Gin[i] = dmulr(Gin[i], Kl[i]);
      const int64_t ps = slot_arr1(L, 2 * d);
      const cplx g = V(ps, f);
      const cplx *Jp = JJ(ps, f);
      calc_dA_dB(M, 2 * d + 1, A, B, Kl, Ki[2 * d + 1], g, Jp, Gin, Jin, JJ(0, f + L->st[d]));
      if (p[d] + 2 < L->c[d]) calc_dA_dB(M, 2 * d, A, B, Kl, Ki[2 * d], g, Jp, Gin, Jin, JJ(slot_arr2(L, d), f));
      for (int i = d + 1; i < M; ++i)
        if (p[i] + 1 < L->c[i]) {
          calc_dA_dB(M, 2 * i, A, B, Kl, Ki[2 * i], g, Jp, Gin, Jin, JJ(slot_1010(L, d, i - d - 1), f));
          calc_dA_dB(M, 2 * i + 1, A, B, Kl, Ki[2 * i + 1], g, Jp, Gin, Jin, JJ(slot_1001(L, d, i - d - 1), f));
        }
    }
  }
#undef V
#undef JJ
  free(order);
  return 0;
}

/* ------------------------------------------------------------ 3. fast_diagonal */

/*
 * The near-diagonal lattice of fast_diagonal: 2(L-1) coordinates in pairs (a_j, b_j),
 * 0 <= a_j, b_j <= pnr_j, |a_j - b_j| <= 2, at most one pair with |a_j - b_j| = 2
 * (enumerate_diagonal_coords, fast_diagonal.py:160-200).  Point storage is dense over
 * per-pair states a*5 + (a - b + 2) (mixed radix over pairs, pair 0 slowest), each point
 * an (oc+1) x (oc+1) block.
 */
typedef struct {
  int K;                 /* L - 1 pairs */
  int64_t pnr[DG_MAXM];  /* pnr cutoffs (inclusive maxima) */
  int64_t rad[DG_MAXM];  /* 5 * (pnr + 1) */
  int64_t pst[DG_MAXM];  /* mixed-radix strides */
  int64_t npts;
} FdLat;

static void fd_init(FdLat *F, int K, const int64_t *pnr) {
  F->K = K;
  F->npts = 1;
  for (int j = K - 1; j >= 0; --j) {
    F->pnr[j] = pnr[j];
    F->rad[j] = 5 * (pnr[j] + 1);
    F->pst[j] = F->npts;
    F->npts *= F->rad[j];
  }
}
/* coords k[0..2K) of a dense id; returns 0 when the id is not a lattice point */
static int fd_decode(const FdLat *F, int64_t id, int64_t *k) {
  int n2 = 0;
  for (int j = 0; j < F->K; ++j) {
    const int64_t s = (id / F->pst[j]) % F->rad[j];
    const int64_t a = s / 5, dl = s % 5 - 2, b = a - dl;
    if (b < 0 || b > F->pnr[j]) return 0;
    n2 += (dl == 2 || dl == -2);
    k[2 * j] = a;
    k[2 * j + 1] = b;
  }
  return n2 <= 1;
}
static int64_t fd_encode(const FdLat *F, const int64_t *k) {
  int64_t id = 0;
  for (int j = 0; j < F->K; ++j) id += (k[2 * j] * 5 + (k[2 * j] - k[2 * j + 1] + 2)) * F->pst[j];
  return id;
}

/*
 * A (2L x 2L), b (2L) in the caller's order (all first copies, then all second copies);
 * out: (pnr_1+1, ..., pnr_{L-1}+1, oc+1, oc+1), the layout fast_diagonal returns.
 * stable selects stable_numba for the first block (fast_diagonal.py:62-65).
 */
int oracle_fast_diagonal(int Lm, const int64_t *pnr, int64_t oc, const cplx *A_in, const cplx *b_in, const cplx *cp,
                         int stable, cplx *out) {
  if (Lm < 1 || Lm > DG_MAXM || oc < 0) return 1;
  const int K = Lm - 1, n = 2 * Lm;
  const int64_t q = oc + 1, blk = q * q;
  /* perm = [m, m + L for m in range(L)] */
  int perm[2 * DG_MAXM];
  for (int m = 0; m < Lm; ++m) {
    perm[2 * m] = m;
    perm[2 * m + 1] = m + Lm;
  }
  cplx A[4 * DG_MAXM * DG_MAXM], b[2 * DG_MAXM];
  for (int r = 0; r < n; ++r) {
    b[r] = b_in[perm[r]];
    for (int s = 0; s < n; ++s) A[r * n + s] = A_in[perm[r] * n + perm[s]];
  }
  int64_t nout = blk;
  for (int j = 0; j < K; ++j) nout *= pnr[j] + 1;
  memset(out, 0, (size_t)nout * sizeof(cplx));
  /* first block: the 2-mode recurrence of mode 0 */
  cplx A2[4] = {A[0], A[1], A[n], A[n + 1]};
  const int64_t sh2[2] = {q, q};
  cplx *first = (cplx *)malloc((size_t)blk * sizeof(cplx));
  if (stable)
    oracle_stable(2, sh2, A2, b, cp, first);
  else
    oracle_vanilla(2, sh2, A2, b, cp, first);
  memcpy(out, first, (size_t)blk * sizeof(cplx));
  if (K == 0) {
    free(first);
    return 0;
  }
  FdLat F;
  fd_init(&F, K, pnr);
  cplx *G = (cplx *)calloc((size_t)(F.npts * blk), sizeof(cplx));
  int64_t k[2 * DG_MAXM], pv[2 * DG_MAXM];
  for (int64_t j = 0; j < 2 * K; ++j) k[j] = 0;
  memcpy(G + fd_encode(&F, k) * blk, first, (size_t)blk * sizeof(cplx));
  free(first);
  int64_t sum_pnr = 0;
  for (int j = 0; j < K; ++j) sum_pnr += pnr[j];
  const int64_t wend = 2 * oc + 2 * sum_pnr - Lm; /* range(1, wend) (fast_diagonal.py:70) */
  cplx *val = (cplx *)malloc((size_t)blk * sizeof(cplx));
  for (int64_t weight = 1; weight < wend; ++weight) {
    for (int64_t id = 0; id < F.npts; ++id) {
      if (!fd_decode(&F, id, k)) continue;
      int64_t w = 0;
      for (int j = 0; j < 2 * K; ++j) w += k[j];
      if (w != weight) continue;
      /* get_pivot (fast_diagonal.py:80-99) */
      int mbest = 0;
      int64_t dbest = -1;
      for (int m = 0; m < K; ++m) {
        const int64_t dl = llabs(k[2 * m] - k[2 * m + 1]);
        if (dl > dbest) {
          dbest = dl;
          mbest = m;
        }
      }
      int i;
      if (dbest == 0) {
        i = 0;
        for (int j = 1; j < 2 * K; ++j)
          if (k[j] > k[i]) i = j;
      } else {
        i = k[2 * mbest] > k[2 * mbest + 1] ? 2 * mbest : 2 * mbest + 1;
      }
      for (int j = 0; j < 2 * K; ++j) pv[j] = k[j];
      pv[i] -= 1;
      const cplx *mat = G + fd_encode(&F, pv) * blk;
      /* single_step (fast_diagonal.py:102-124) */
      const cplx bi = b[i + 2], a0 = A[(i + 2) * n + 0], a1 = A[(i + 2) * n + 1];
      for (int64_t e = 0; e < blk; ++e) val[e] = dmul(bi, mat[e]);
      for (int64_t r = 1; r < q; ++r)
        for (int64_t c = 0; c < q; ++c) val[r * q + c] = dadd(val[r * q + c], dmul(dmulr(a0, SQ(r)), mat[(r - 1) * q + c]));
      for (int64_t r = 0; r < q; ++r)
        for (int64_t c = 1; c < q; ++c) val[r * q + c] = dadd(val[r * q + c], dmul(dmulr(a1, SQ(c)), mat[r * q + c - 1]));
      for (int j = 0; j < 2 * K; ++j) {
        if (pv[j] <= 0) continue;
        const cplx coef = dmulr(A[(i + 2) * n + j + 2], SQ(pv[j]));
        pv[j] -= 1;
        const cplx *low = G + fd_encode(&F, pv) * blk;
        pv[j] += 1;
        for (int64_t e = 0; e < blk; ++e) val[e] = dadd(val[e], dmul(coef, low[e]));
      }
      cplx *dst = G + id * blk;
      const double dv = SQ(pv[i] + 1);
      for (int64_t e = 0; e < blk; ++e) dst[e] = ddivr_np(val[e], dv); /* numpy array / float */
      /* diagonal points of even weight are outputs (fast_diagonal.py:75-77) */
      int diag = 1;
      for (int j = 0; j < K; ++j) diag &= (k[2 * j] == k[2 * j + 1]);
      if (diag) {
        int64_t o = 0;
        for (int j = 0; j < K; ++j) o = o * (pnr[j] + 1) + k[2 * j];
        memcpy(out + o * blk, dst, (size_t)blk * sizeof(cplx));
      }
    }
  }
  free(val);
  free(G);
  return 0;
}

/* --------------------------------------------- 4. leftover mode (compactFock) */

/*
 * fock_representation_1leftoverMode_amps (compactFock/singleLeftoverMode_amps.py:18-421) and
 * its Jacobians (singleLeftoverMode_grad.py:18-724), reached through
 * hermite_multidimensional_1leftoverMode / grad_hermite_multidimensional_1leftoverMode
 * (compactFock/inputValidation.py:103-142).  M modes: mode 0 is left over (block q x q,
 * q = cutoffs[0]), modes 1..M-1 (M' = M - 1 of them) are detected, with the params lattice of
 * the diagonal strategy over cutoffs[1..].  A (2M x 2M) and B (2M) in the interleaved order.
 * Storage: W[slot][m][n][P'] with the diagonal strategy's slot numbering over the M' detected
 * modes; J[slot][m][n][P'][4M^2 + 2M].
 */
typedef struct {
  Lat t;     /* the detected modes' lattice (M' modes) */
  int M;     /* all modes */
  int64_t q; /* leftover cutoff */
} LoLat;

#define LW(slot, m, n, f) W[(((slot) * L->q + (m)) * L->q + (n)) * L->t.P + (f)]
#define LJ(slot, m, n, f) (J + ((((slot) * L->q + (m)) * L->q + (n)) * L->t.P + (f)) * nc)

/* one block entry of write_block (singleLeftoverMode_amps.py:20-75): row `row` of A (full
 * index), the pivot block `ps` at params f, the scaled inputs Gin[l] (2M' of them) */
static cplx lo_entry(const LoLat *L, const cplx *A, const cplx *B, int row, int64_t ps, int64_t f, int64_t m,
                     int64_t n, const cplx *Gin, double Ki, const cplx *W) {
  const int N = 2 * L->M;
  cplx dot = 0.0;
  if (m > 0) dot = dadd(dot, dmul(A[row * N + 0], dmulr(LW(ps, m - 1, n, f), SQ(m))));
  if (n > 0) dot = dadd(dot, dmul(A[row * N + 1], dmulr(LW(ps, m, n - 1, f), SQ(n))));
  for (int l = 0; l < N - 2; ++l) dot = dadd(dot, dmul(A[row * N + 2 + l], Gin[l]));
  const cplx GB = dmul(LW(ps, m, n, f), B[row]);
  return ddivr(dadd(GB, dot), Ki);
}

static void lo_first_fill(const LoLat *L, const cplx *A, const cplx *B, cplx *W) {
  /* singleLeftoverMode_amps.py:339-352: the leftover mode with every detected mode at 0 */
  const int N = 2 * L->M;
  const int64_t q = L->q;
  for (int64_t m = 0; m + 1 < q; ++m) {
    const cplx prev = m >= 1 ? LW(0, m - 1, 0, 0) : LW(0, q - 1, 0, 0); /* index -1 wraps (times sqrt(0)) */
    LW(0, m + 1, 0, 0) = ddivr(dadd(dmul(LW(0, m, 0, 0), B[0]), dmul(dmulr(A[0], SQ(m)), prev)), SQ(m + 1));
  }
  for (int64_t m = 0; m < q; ++m)
    for (int64_t n = 0; n + 1 < q; ++n) {
      const cplx up = m >= 1 ? LW(0, m - 1, n, 0) : LW(0, q - 1, n, 0);
      const cplx left = n >= 1 ? LW(0, m, n - 1, 0) : LW(0, m, q - 1, 0);
      cplx v = dmul(LW(0, m, n, 0), B[1]);
      v = dadd(v, dmul(dmulr(A[N + 0], SQ(m)), up));
      v = dadd(v, dmul(dmulr(A[N + 1], SQ(n)), left));
      LW(0, m, n + 1, 0) = ddivr(v, SQ(n + 1));
    }
}

int64_t oracle_leftover_slots(int M) { return oracle_diagonal_slots(M - 1); }

int oracle_leftover_amps(int M, const int64_t *cutoffs, const cplx *A, const cplx *B, const cplx *G0, cplx *W) {
  if (M < 2) return 1;
  LoLat Ls, *L = &Ls;
  if (lat_init(&L->t, M - 1, cutoffs + 1, 1)) return 1;
  L->M = M;
  L->q = cutoffs[0];
  if (L->q < 1) return 1;
  const int Mt = M - 1, nt = 2 * Mt;
  const int64_t S = oracle_diagonal_slots(Mt);
  memset(W, 0, (size_t)(S * L->q * L->q * L->t.P) * sizeof(cplx));
  LW(0, 0, 0, 0) = *G0;
  lo_first_fill(L, A, B, W);
  int64_t nw;
  int64_t *order = params_by_weight(&L->t, &nw);
  int64_t p[DG_MAXM];
  cplx Gin[2 * DG_MAXM];
  for (int64_t t = 0; t < L->t.P; ++t) {
    const int64_t f = order[t];
    int64_t r = f;
    for (int k = 0; k < Mt; ++k) {
      p[k] = r / L->t.st[k];
      r %= L->t.st[k];
    }
    /* use_diag_pivot (singleLeftoverMode_amps.py:213-284) */
    if (L->t.c[0] == 1 || p[0] < L->t.c[0] - 1) {
      for (int64_t m = 0; m < L->q; ++m)
        for (int64_t n = 0; n < L->q; ++n) {
          for (int i = 0; i < nt; ++i) {
            Gin[i] = 0.0;
            if (p[i / 2] > 0) Gin[i] = LW(slot_arr1(&L->t, i + 1 - 2 * (i % 2)), m, n, f - L->t.st[i / 2]);
            Gin[i] = dmulr(Gin[i], SQ(p[i / 2]));
          }
          for (int i = 0; i < nt; ++i)
            if (p[i / 2] + 1 < L->t.c[i / 2] && (i != 1 || p[0] + 2 < L->t.c[0]))
              LW(slot_arr1(&L->t, i), m, n, f) = lo_entry(L, A, B, i + 2, 0, f, m, n, Gin, SQ(p[i / 2] + 1), W);
        }
    }
    /* use_offDiag_pivot (singleLeftoverMode_amps.py:101-210) */
    for (int d = 0; d < Mt; ++d) {
      int lower_zero = 1;
      for (int k = 0; k < d; ++k) lower_zero &= (p[k] == 0);
      if (!(lower_zero && p[d] < L->t.c[d] - 1)) continue;
      double Kl[2 * DG_MAXM], Ki[2 * DG_MAXM];
      for (int k = 0; k < Mt; ++k) {
        Kl[2 * k] = SQ(p[k] + (k == d));
        Kl[2 * k + 1] = SQ(p[k]);
        Ki[2 * k] = SQ(p[k] + (k == d) + 1);
        Ki[2 * k + 1] = SQ(p[k] + 1);
      }
      const int64_t ps = slot_arr1(&L->t, 2 * d);
      for (int64_t m = 0; m < L->q; ++m)
        for (int64_t n = 0; n < L->q; ++n) {
          for (int i = 0; i < nt; ++i) Gin[i] = 0.0;
          Gin[2 * d] = LW(0, m, n, f);
          if (p[d] > 0) Gin[2 * d + 1] = LW(slot_arr2(&L->t, d), m, n, f - L->t.st[d]);
          for (int i = d + 1; i < Mt; ++i)
            if (p[i] > 0) {
              Gin[2 * i] = LW(slot_1001(&L->t, d, i - d - 1), m, n, f - L->t.st[i]);
              Gin[2 * i + 1] = LW(slot_1010(&L->t, d, i - d - 1), m, n, f - L->t.st[i]);
            }
          for (int i = 0; i < nt; ++i) Gin[i] = dmulr(Gin[i], Kl[i]);
          LW(0, m, n, f + L->t.st[d]) = lo_entry(L, A, B, 2 * d + 3, ps, f, m, n, Gin, Ki[2 * d + 1], W);
          if (p[d] + 2 < L->t.c[d])
            LW(slot_arr2(&L->t, d), m, n, f) = lo_entry(L, A, B, 2 * d + 2, ps, f, m, n, Gin, Ki[2 * d], W);
          for (int i = d + 1; i < Mt; ++i)
            if (p[i] + 1 < L->t.c[i]) {
              LW(slot_1010(&L->t, d, i - d - 1), m, n, f) = lo_entry(L, A, B, 2 * i + 2, ps, f, m, n, Gin, Ki[2 * i], W);
              LW(slot_1001(&L->t, d, i - d - 1), m, n, f) =
                  lo_entry(L, A, B, 2 * i + 3, ps, f, m, n, Gin, Ki[2 * i + 1], W);
            }
        }
    }
  }
  free(order);
  return 0;
}

/* calc_dA_dB of the leftover strategy (singleLeftoverMode_grad.py:18-46) for block entry (m, n):
 * terms l = 0 (m > 0: pivot (m-1, n), K = sqrt(m)), l = 1 (n > 0: pivot (m, n-1), K = sqrt(n)),
 * l = 2 .. 2M-1 (input l - 2, K = Kl[l - 2]); Jacobian rows of nc entries. */
static void lo_jac_entry(const LoLat *L, const cplx *A, const cplx *B, int row, int64_t ps, int64_t f, int64_t m,
                         int64_t n, const cplx *Gin_scaled, const cplx *const *Jin, const double *Kl, double Ki,
                         const cplx *W, cplx *J, cplx *out) {
  const int N = 2 * L->M, nA = N * N;
  const int64_t nc = (int64_t)nA + N;
  int nterm = 0;
  int ls[2 * DG_MAXM + 2];
  double Ks[2 * DG_MAXM + 2];
  cplx Gs[2 * DG_MAXM + 2];
  const cplx *Js[2 * DG_MAXM + 2];
  if (m > 0) {
    ls[nterm] = 0;
    Ks[nterm] = SQ(m);
    Gs[nterm] = dmulr(LW(ps, m - 1, n, f), SQ(m));
    Js[nterm++] = LJ(ps, m - 1, n, f);
  }
  if (n > 0) {
    ls[nterm] = 1;
    Ks[nterm] = SQ(n);
    Gs[nterm] = dmulr(LW(ps, m, n - 1, f), SQ(n));
    Js[nterm++] = LJ(ps, m, n - 1, f);
  }
  for (int l = 0; l < N - 2; ++l) {
    ls[nterm] = l + 2;
    Ks[nterm] = Kl[l];
    Gs[nterm] = Gin_scaled[l];
    Js[nterm++] = Jin[l];
  }
  const cplx *Jp = LJ(ps, m, n, f);
  for (int64_t qd = 0; qd < nA; ++qd) {
    cplx acc = dmul(Jp[qd], B[row]);
    for (int t = 0; t < nterm; ++t) {
      acc = dadd(acc, dmul(dmulr(A[row * N + ls[t]], Ks[t]), Js[t] ? Js[t][qd] : 0.0));
      if (qd == (int64_t)row * N + ls[t]) acc = dadd(acc, Gs[t]);
    }
    out[qd] = ddivr(acc, Ki);
  }
  for (int r = 0; r < N; ++r) {
    cplx acc = dmul(Jp[nA + r], B[row]);
    if (r == row) acc = dadd(acc, LW(ps, m, n, f));
    for (int t = 0; t < nterm; ++t) acc = dadd(acc, dmul(dmulr(A[row * N + ls[t]], Ks[t]), Js[t] ? Js[t][nA + r] : 0.0));
    out[nA + r] = ddivr(acc, Ki);
  }
}

int oracle_leftover_grad(int M, const int64_t *cutoffs, const cplx *A, const cplx *B, const cplx *W, cplx *J) {
  if (M < 2) return 1;
  LoLat Ls, *L = &Ls;
  if (lat_init(&L->t, M - 1, cutoffs + 1, 1)) return 1;
  L->M = M;
  L->q = cutoffs[0];
  const int Mt = M - 1, nt = 2 * Mt, N = 2 * M, nA = N * N;
  const int64_t nc = (int64_t)nA + N, q = L->q;
  const int64_t S = oracle_diagonal_slots(Mt);
  memset(J, 0, (size_t)(S * q * q * L->t.P * nc) * sizeof(cplx));
  /* first fill (singleLeftoverMode_grad.py:606-650) */
  for (int64_t m = 0; m + 1 < q; ++m) {
    cplx *dst = LJ(0, m + 1, 0, 0);
    const cplx *cur = LJ(0, m, 0, 0), *prev = m >= 1 ? LJ(0, m - 1, 0, 0) : LJ(0, q - 1, 0, 0);
    const cplx vprev = m >= 1 ? LW(0, m - 1, 0, 0) : LW(0, q - 1, 0, 0);
    for (int64_t c = 0; c < nc; ++c)
      dst[c] = ddivr_np(dadd(dmul(cur[c], B[0]), dmul(dmulr(A[0], SQ(m)), prev[c])), SQ(m + 1));
    dst[0] = dadd(dst[0], ddivr_np(dmulr(vprev, SQ(m)), SQ(m + 1)));
    dst[nA + 0] = dadd(dst[nA + 0], ddivr_np(LW(0, m, 0, 0), SQ(m + 1)));
  }
  for (int64_t m = 0; m < q; ++m)
    for (int64_t n = 0; n + 1 < q; ++n) {
      cplx *dst = LJ(0, m, n + 1, 0);
      const cplx *cur = LJ(0, m, n, 0);
      const cplx *up = m >= 1 ? LJ(0, m - 1, n, 0) : LJ(0, q - 1, n, 0);
      const cplx *left = n >= 1 ? LJ(0, m, n - 1, 0) : LJ(0, m, q - 1, 0);
      const cplx vup = m >= 1 ? LW(0, m - 1, n, 0) : LW(0, q - 1, n, 0);
      const cplx vleft = n >= 1 ? LW(0, m, n - 1, 0) : LW(0, m, q - 1, 0);
      for (int64_t c = 0; c < nc; ++c) {
        cplx v = dmul(cur[c], B[1]);
        v = dadd(v, dmul(dmulr(A[N + 0], SQ(m)), up[c]));
        v = dadd(v, dmul(dmulr(A[N + 1], SQ(n)), left[c]));
        dst[c] = ddivr_np(v, SQ(n + 1));
      }
      dst[N + 0] = dadd(dst[N + 0], ddivr_np(dmulr(vup, SQ(m)), SQ(n + 1)));
      dst[N + 1] = dadd(dst[N + 1], ddivr_np(dmulr(vleft, SQ(n)), SQ(n + 1)));
      dst[nA + 1] = dadd(dst[nA + 1], ddivr_np(LW(0, m, n, 0), SQ(n + 1)));
    }
  int64_t nw;
  int64_t *order = params_by_weight(&L->t, &nw);
  int64_t p[DG_MAXM];
  cplx Gin[2 * DG_MAXM];
  const cplx *Jin[2 * DG_MAXM];
  double Kl[2 * DG_MAXM], Ki[2 * DG_MAXM];
  for (int64_t t = 0; t < L->t.P; ++t) {
    const int64_t f = order[t];
    int64_t r = f;
    for (int k = 0; k < Mt; ++k) {
      p[k] = r / L->t.st[k];
      r %= L->t.st[k];
    }
    if (L->t.c[0] == 1 || p[0] < L->t.c[0] - 1) {
      for (int i = 0; i < nt; ++i) Kl[i] = SQ(p[i / 2]);
      for (int64_t m = 0; m < q; ++m)
        for (int64_t n = 0; n < q; ++n) {
          for (int i = 0; i < nt; ++i) {
            Gin[i] = 0.0;
            Jin[i] = NULL;
            if (p[i / 2] > 0) {
              const int64_t s = slot_arr1(&L->t, i + 1 - 2 * (i % 2));
              Gin[i] = LW(s, m, n, f - L->t.st[i / 2]);
              Jin[i] = LJ(s, m, n, f - L->t.st[i / 2]);
            }
            Gin[i] = dmulr(Gin[i], Kl[i]);
          }
          for (int i = 0; i < nt; ++i)
            if (p[i / 2] + 1 < L->t.c[i / 2] && (i != 1 || p[0] + 2 < L->t.c[0]))
              lo_jac_entry(L, A, B, i + 2, 0, f, m, n, Gin, Jin, Kl, SQ(p[i / 2] + 1), W, J,
                           LJ(slot_arr1(&L->t, i), m, n, f));
        }
    }
    for (int d = 0; d < Mt; ++d) {
      int lower_zero = 1;
      for (int k = 0; k < d; ++k) lower_zero &= (p[k] == 0);
      if (!(lower_zero && p[d] < L->t.c[d] - 1)) continue;
      for (int k = 0; k < Mt; ++k) {
        Kl[2 * k] = SQ(p[k] + (k == d));
        Kl[2 * k + 1] = SQ(p[k]);
        Ki[2 * k] = SQ(p[k] + (k == d) + 1);
        Ki[2 * k + 1] = SQ(p[k] + 1);
      }
      const int64_t ps = slot_arr1(&L->t, 2 * d);
      for (int64_t m = 0; m < q; ++m)
        for (int64_t n = 0; n < q; ++n) {
          for (int i = 0; i < nt; ++i) {
            Gin[i] = 0.0;
            Jin[i] = NULL;
          }
          Gin[2 * d] = LW(0, m, n, f);
          Jin[2 * d] = LJ(0, m, n, f);
          if (p[d] > 0) {
            Gin[2 * d + 1] = LW(slot_arr2(&L->t, d), m, n, f - L->t.st[d]);
            Jin[2 * d + 1] = LJ(slot_arr2(&L->t, d), m, n, f - L->t.st[d]);
          }
          for (int i = d + 1; i < Mt; ++i)
            if (p[i] > 0) {
              Gin[2 * i] = LW(slot_1001(&L->t, d, i - d - 1), m, n, f - L->t.st[i]);
              Jin[2 * i] = LJ(slot_1001(&L->t, d, i - d - 1), m, n, f - L->t.st[i]);
              Gin[2 * i + 1] = LW(slot_1010(&L->t, d, i - d - 1), m, n, f - L->t.st[i]);
              Jin[2 * i + 1] = LJ(slot_1010(&L->t, d, i - d - 1), m, n, f - L->t.st[i]);
            }
          for (int i = 0; i < nt; ++i) Gin[i] = dmulr(Gin[i], Kl[i]);
          lo_jac_entry(L, A, B, 2 * d + 3, ps, f, m, n, Gin, Jin, Kl, Ki[2 * d + 1], W, J, LJ(0, m, n, f + L->t.st[d]));
          if (p[d] + 2 < L->t.c[d])
            lo_jac_entry(L, A, B, 2 * d + 2, ps, f, m, n, Gin, Jin, Kl, Ki[2 * d], W, J, LJ(slot_arr2(&L->t, d), m, n, f));
          for (int i = d + 1; i < Mt; ++i)
            if (p[i] + 1 < L->t.c[i]) {
              lo_jac_entry(L, A, B, 2 * i + 2, ps, f, m, n, Gin, Jin, Kl, Ki[2 * i], W, J,
                           LJ(slot_1010(&L->t, d, i - d - 1), m, n, f));
              lo_jac_entry(L, A, B, 2 * i + 3, ps, f, m, n, Gin, Jin, Kl, Ki[2 * i + 1], W, J,
                           LJ(slot_1001(&L->t, d, i - d - 1), m, n, f));
            }
        }
    }
  }
  free(order);
  return 0;
}
#undef LW
#undef LJ
