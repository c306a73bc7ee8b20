/*
 * sg4_oracle.c -- CPU oracle for ElVibRot's SG4 H.psi (TEST INFRASTRUCTURE).
 *
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline/reference
 * arm load this file's library.  It restates, in plain C + OpenMP, the
 * reference routines cited at each function (paths relative to the ElVibRot
 * source tree).  Parity is pinned against the reference's known answers
 * (HermQuadra nodes/weights, Henon-Heiles SG4 Davidson levels) by the tests.
 *
 * The structure deliberately follows the reference, not a GPU design:
 * OpenMP static loop over Smolyak terms, per-term gather, mode-by-mode 1-D
 * matrix products with the Fortran loop order, operator on the grid, and an
 * atomic weighted scatter (sub_OpPsi_SG4.f90:833-865).
 */
#include "sg4_oracle.h"

#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define ORC_MAXD 64

typedef long double ldbl;

typedef struct {
  int nb, nq;
  double *x, *w;                 /* nodes (scaled), wrho (scaled) */
  double *d0, *d1, *d2;          /* dnRGB: nq x nb column-major */
  double *bgw;                   /* dnRBGwrho%d0: nb x nq column-major */
  double *d1gg, *d2gg;           /* dnRGG%d1, %d2: nq x nq column-major */
} orc_basis1;

struct orc_sg4 {
  int D, L, LB, Lmin;
  int* nb_of_l;                  /* [D][L+1] */
  int* nq_of_l;
  orc_basis1* b;                 /* [D][L+1] */
  int* i_to_l;                   /* [D][nbmax]: L_i(n) for n = 1..nb(L) */
  int nbmax_mode;                /* max over modes of nb(L) */
  /* packed basis (type 5p) */
  long long N;
  int* packed;                   /* [N][D], 1-based */
  /* Smolyak terms (type -5) */
  long long nb_SG;
  int* tab_l;                    /* [nb_SG][D] */
  double* weight;
  long long *off_nb, *off_nq;    /* exclusive prefix sums */
  long long sum_nb, sum_nq;
  int max_nb, max_nq;
  int* map;                      /* [sum_nb] */
};

/* ------------------------------------------------------------------------ */
/* 1-D Gauss-Hermite quadrature.                                             */
/* Restates the node/weight definition used by sub_quadra_hermite            */
/* (sub_quadra_herm.f90:48-244): nodes = zeros of H_nq, the weight read from */
/* herm{nq}.txt column 4 is w_i exp(x_i^2).  Computed here in long double:   */
/* Sturm bisection on the Jacobi matrix, Newton polish, Christoffel weights. */
/* ------------------------------------------------------------------------ */
static int sturm_count(int n, ldbl lam) {
  /* number of eigenvalues of the symmetric tridiagonal Jacobi matrix
   * (diag 0, offdiag sqrt(k/2)) strictly below lam */
  int cnt = 0;
  ldbl q = -lam;
  if (q < 0) cnt++;
  for (int k = 1; k < n; ++k) {
    ldbl b2 = (ldbl)k / 2.0L;
    if (q == 0) q = 1e-4000L;
    q = -lam - b2 / q;
    if (q < 0) cnt++;
  }
  return cnt;
}

static void herm_orthonormal(int n, ldbl x, ldbl* pn, ldbl* pnm1, ldbl* sumsq_psi) {
  /* orthonormal Hermite functions psi_k = p_k exp(-x^2/2), k = 0..n */
  ldbl e = expl(-x * x / 2.0L);
  ldbl pm = 0, p = powl(acosl(-1.0L), -0.25L) * e, s = 0;
  for (int k = 0; k < n; ++k) {
    s += p * p;
    ldbl pp = sqrtl(2.0L / (k + 1)) * x * p - sqrtl((ldbl)k / (k + 1)) * pm;
    pm = p;
    p = pp;
  }
  *pn = p;
  *pnm1 = pm;
  *sumsq_psi = s;
}

void orc_gauss_hermite(int nq, double* x, double* w, double* wrho) {
  ldbl* xr = (ldbl*)malloc(sizeof(ldbl) * nq);
  ldbl R = sqrtl(2.0L * nq + 1.0L) + 1.0L;
  for (int i = 0; i < nq; ++i) {
    ldbl lo = -R, hi = R;
    for (int it = 0; it < 200; ++it) {
      ldbl mid = 0.5L * (lo + hi);
      if (mid == lo || mid == hi) break;
      if (sturm_count(nq, mid) > i) hi = mid; else lo = mid;
    }
    ldbl r = 0.5L * (lo + hi);
    for (int it = 0; it < 4; ++it) {
      ldbl pn, pnm1, s;
      herm_orthonormal(nq, r, &pn, &pnm1, &s);
      ldbl dp = sqrtl(2.0L * nq) * pnm1;
      if (dp != 0) r -= pn / dp;
    }
    xr[i] = r;
  }
  for (int i = 0; i < nq / 2; ++i) {
    ldbl a = 0.5L * (xr[nq - 1 - i] - xr[i]);
    xr[i] = -a;
    xr[nq - 1 - i] = a;
  }
  if (nq % 2 == 1) xr[nq / 2] = 0.0L;
  for (int i = 0; i < nq; ++i) {
    ldbl pn, pnm1, s;
    herm_orthonormal(nq, xr[i], &pn, &pnm1, &s);
    ldbl wr = 1.0L / s;               /* w exp(x^2) */
    x[i] = (double)xr[i];
    if (wrho) wrho[i] = (double)wr;
    if (w) w[i] = (double)(wr * expl(-xr[i] * xr[i]));
  }
  free(xr);
}

/* ------------------------------------------------------------------------ */
/* Hermite functions and derivatives at a point, in double, with the         */
/* reference recurrence: poly_Hermite + d0d1d2poly_Hermite_exp               */
/* (Ext_Lib/FOR_EVRT_loc/.../sub_polyortho.f90:838-900, 1090-1162).          */
/* ------------------------------------------------------------------------ */
static double poly_hermite(double x, int l) {
  const double pi = 3.14159265358979323846264338327950288;
  double norme = sqrt(pi);
  if (l == 0) return 1.0 / sqrt(norme);
  if (l == 1) { norme *= 2.0; return 2.0 * x / sqrt(norme); }
  double pl2 = 1.0, pl1 = 2.0 * x, pl0 = 0.0;
  norme *= 2.0;
  for (int i = 2; i <= l; ++i) {
    norme = norme * 2.0 * (double)i;
    pl0 = 2.0 * (x * pl1 - (double)(i - 1) * pl2);
    pl2 = pl1;
    pl1 = pl0;
  }
  return pl0 / sqrt(norme);
}

static void d0d1d2_hermite_exp(double x, int l, double* d0, double* d1, double* d2) {
  double v0 = poly_hermite(x, l), v1, v2;
  if (l == 0) { v1 = 0.0; v2 = 0.0; }
  else if (l == 1) { v1 = sqrt(2.0) * poly_hermite(x, 0); v2 = 0.0; }
  else {
    v1 = sqrt(2.0 * (double)l) * poly_hermite(x, l - 1);
    v2 = 2.0 * (x * v1 - v0 * (double)l);
  }
  double pexp = exp(-0.5 * x * x);
  *d2 = (v2 - 2.0 * x * v1 + (x * x - 1.0) * v0) * pexp;
  *d1 = (v1 - x * v0) * pexp;
  *d0 = v0 * pexp;
}

/* Moore-Penrose pseudo-inverse of the full-column-rank nq x nb matrix A
 * (column-major), returned nb x nq column-major, computed in long double as
 * (A^T A)^{-1} A^T.  This is the matrix sub_dnGB_TO_dnGG builds as
 * d0b_pseudoInv = d0b^T (d0b d0b^T)^+ (sub_module_basis.f90:2048-2180). */
static void pinv_ld(int nq, int nb, const double* A, ldbl* P) {
  ldbl* M = (ldbl*)calloc((size_t)nb * 2 * nb, sizeof(ldbl));  /* [M | I] row-major nb x 2nb */
  for (int i = 0; i < nb; ++i) {
    for (int j = 0; j < nb; ++j) {
      ldbl s = 0;
      for (int q = 0; q < nq; ++q) s += (ldbl)A[q + (size_t)nq * i] * (ldbl)A[q + (size_t)nq * j];
      M[i * 2 * nb + j] = s;
    }
    M[i * 2 * nb + nb + i] = 1.0L;
  }
  for (int c = 0; c < nb; ++c) {            /* Gauss-Jordan, partial pivoting */
    int piv = c;
    for (int r = c + 1; r < nb; ++r)
      if (fabsl(M[r * 2 * nb + c]) > fabsl(M[piv * 2 * nb + c])) piv = r;
    if (piv != c)
      for (int k = 0; k < 2 * nb; ++k) {
        ldbl t = M[c * 2 * nb + k]; M[c * 2 * nb + k] = M[piv * 2 * nb + k]; M[piv * 2 * nb + k] = t;
      }
    ldbl d = M[c * 2 * nb + c];
    for (int k = 0; k < 2 * nb; ++k) M[c * 2 * nb + k] /= d;
    for (int r = 0; r < nb; ++r) {
      if (r == c) continue;
      ldbl f = M[r * 2 * nb + c];
      if (f == 0) continue;
      for (int k = 0; k < 2 * nb; ++k) M[r * 2 * nb + k] -= f * M[c * 2 * nb + k];
    }
  }
  for (int i = 0; i < nb; ++i)              /* P = inv(A^T A) A^T */
    for (int q = 0; q < nq; ++q) {
      ldbl s = 0;
      for (int k = 0; k < nb; ++k) s += M[i * 2 * nb + nb + k] * (ldbl)A[q + (size_t)nq * k];
      P[i + (size_t)nb * q] = s;
    }
  free(M);
}

/* One 1-D HO basis: quadrature, Hermite functions, scaling, dnRBGwrho, dnRGG.
 * Order of steps as construct_primitive_basis (sub_module_basis.f90:396-796):
 * sub_quadra_hermite -> sub_scale_basis (:1499-1585) -> sub_dnGB_TO_dnGG
 * (:2048-2329) -> sub_dnGB_TO_dnBG (:1949-2013). */
static void build_basis1(orc_basis1* b, int nb, int nq, double Q0, double scaleQ) {
  b->nb = nb;
  b->nq = nq;
  b->x = (double*)malloc(sizeof(double) * nq);
  b->w = (double*)malloc(sizeof(double) * nq);
  b->d0 = (double*)malloc(sizeof(double) * nq * nb);
  b->d1 = (double*)malloc(sizeof(double) * nq * nb);
  b->d2 = (double*)malloc(sizeof(double) * nq * nb);
  b->bgw = (double*)malloc(sizeof(double) * nq * nb);
  b->d1gg = (double*)malloc(sizeof(double) * nq * nq);
  b->d2gg = (double*)malloc(sizeof(double) * nq * nq);
  orc_gauss_hermite(nq, b->x, NULL, b->w);   /* base%w = wrho = file column 4 */
  for (int k = 0; k < nq; ++k)
    for (int i = 0; i < nb; ++i)
      d0d1d2_hermite_exp(b->x[k], i, &b->d0[k + nq * i], &b->d1[k + nq * i], &b->d2[k + nq * i]);
  if (!(Q0 == 0.0 && scaleQ == 1.0)) {        /* sub_scale_basis, ndim = 1 */
    double s_inv = 1.0 / scaleQ, sd0 = sqrt(scaleQ), sd1 = sqrt(scaleQ) * scaleQ,
           sd2 = sqrt(scaleQ) * scaleQ * scaleQ;
    for (int k = 0; k < nq; ++k) {
      b->x[k] = Q0 + b->x[k] / scaleQ;
      b->w[k] = b->w[k] * s_inv;
    }
    for (int k = 0; k < nq * nb; ++k) {
      b->d0[k] *= sd0;
      b->d1[k] *= sd1;
      b->d2[k] *= sd2;
    }
  }
  ldbl* P = (ldbl*)malloc(sizeof(ldbl) * nq * nb);
  pinv_ld(nq, nb, b->d0, P);
  for (int r = 0; r < nq; ++r)
    for (int c = 0; c < nq; ++c) {
      ldbl s1 = 0, s2 = 0;
      for (int k = 0; k < nb; ++k) {
        s1 += (ldbl)b->d1[r + nq * k] * P[k + (size_t)nb * c];
        s2 += (ldbl)b->d2[r + nq * k] * P[k + (size_t)nb * c];
      }
      b->d1gg[r + nq * c] = (double)s1;
      b->d2gg[r + nq * c] = (double)s2;
    }
  free(P);
  for (int i = 0; i < nb; ++i)
    for (int k = 0; k < nq; ++k) b->bgw[i + nb * k] = b->d0[k + nq * i] * b->w[k];
}

/* ------------------------------------------------------------------------ */
/* Index sets.                                                               */
/* ------------------------------------------------------------------------ */
static int lin_n(int A, int B, int l) { return A + B * l; }

/* L of the n-th (1-based) 1-D function: smallest l with nb(l) >= n, i.e. the
 * Tab_L of the Lmax primitive basis (sub_module_basis.f90:710-722, used as
 * tab_i_TO_l in RecSparseGrid_ForDP_type4). */
static int l_of_n(int A, int B, int n, int Lmax) {
  for (int l = 0; l <= Lmax; ++l)
    if (lin_n(A, B, l) >= n) return l;
  return Lmax + 1;
}

static int cmp_tuple_D;
static int cmp_tuple(const void* a, const void* b) {
  const int* x = (const int*)a;
  const int* y = (const int*)b;
  for (int i = 0; i < cmp_tuple_D; ++i)
    if (x[i] != y[i]) return x[i] < y[i] ? -1 : 1;
  return 0;
}

/* Enumerates nDindex type 5p: nDval in [1..nDsize_i], sum_i L_i(nDval_i) <= LB,
 * lexicographic with the LAST index fastest (ADD_ONE_TO_nDindex_type5p,
 * Ext_Lib/nDindex_loc/.../sub_module_nDindex.f90:2670-2736).  Because L_i is
 * non-decreasing in nDval_i the reference's carry logic visits exactly these
 * tuples in this order. */
static long long enum_type5p(int D, const int* nDsize, const int* i_to_l, int ldil, int LB, int** out) {
  long long cap = 1024, n = 0;
  int* buf = (int*)malloc(sizeof(int) * D * cap);
  int v[ORC_MAXD];
  for (int i = 0; i < D; ++i) v[i] = 1;
  for (;;) {
    int Ls = 0, over = -1;
    for (int i = 0; i < D; ++i) {
      Ls += i_to_l[i * ldil + v[i] - 1];
      if (Ls > LB) { over = i; break; }
    }
    if (over < 0) {
      if (n == cap) { cap *= 2; buf = (int*)realloc(buf, sizeof(int) * D * cap); }
      memcpy(buf + n * D, v, sizeof(int) * D);
      n++;
      v[D - 1]++;
    } else {
      /* the prefix v[0..over] alone exceeds LB and L_i is non-decreasing:
       * no tuple with this prefix (or a larger v[over]) is in the set */
      for (int j = over + 1; j < D; ++j) v[j] = 1;
      v[over] = nDsize[over] + 1;
    }
    int i = over < 0 ? D - 1 : over;
    while (i >= 0 && v[i] > nDsize[i]) {
      if (i == 0) { *out = buf; return n; }
      v[i] = 1;
      v[i - 1]++;
      i--;
    }
  }
}

/* ------------------------------------------------------------------------ */
orc_sg4* orc_create(int D, int L, int LB, int A_nb, int B_nb, int A_nq, int B_nq,
                    const double* Q0, const double* scaleQ) {
  if (D < 1 || D > ORC_MAXD) return NULL;
  int a[ORC_MAXD], b[ORC_MAXD], c[ORC_MAXD], d[ORC_MAXD];
  for (int i = 0; i < D; ++i) {
    a[i] = A_nb;
    b[i] = B_nb;
    c[i] = A_nq;
    d[i] = B_nq;
  }
  return orc_create_modes(D, L, LB, a, b, c, d, Q0, scaleQ);
}

orc_sg4* orc_create_modes(int D, int L, int LB, const int* A_nb, const int* B_nb, const int* A_nq,
                          const int* B_nq, const double* Q0, const double* scaleQ) {
  if (D < 1 || D > ORC_MAXD || L < 0 || LB < 0) return NULL;
  orc_sg4* s = (orc_sg4*)calloc(1, sizeof(orc_sg4));
  s->D = D;
  s->L = L;
  s->LB = LB;
  s->Lmin = L - D + 1 > 0 ? L - D + 1 : 0;   /* sub_quadra_SparseBasis.f90:989-990 */
  s->nb_of_l = (int*)malloc(sizeof(int) * D * (L + 1));
  s->nq_of_l = (int*)malloc(sizeof(int) * D * (L + 1));
  s->b = (orc_basis1*)calloc((size_t)D * (L + 1), sizeof(orc_basis1));
  for (int m = 0; m < D; ++m)
    for (int l = 0; l <= L; ++l) {
      int nb = lin_n(A_nb[m], B_nb[m], l), nq = lin_n(A_nq[m], B_nq[m], l);
      s->nb_of_l[m * (L + 1) + l] = nb;
      s->nq_of_l[m * (L + 1) + l] = nq;
      build_basis1(&s->b[m * (L + 1) + l], nb, nq, Q0 ? Q0[m] : 0.0, scaleQ ? scaleQ[m] : 1.0);
    }
  /* tab_i_TO_l and nDsize from the Lmax basis */
  int nDsize[ORC_MAXD];
  s->nbmax_mode = 0;
  for (int m = 0; m < D; ++m) {
    nDsize[m] = s->nb_of_l[m * (L + 1) + L];
    if (nDsize[m] > s->nbmax_mode) s->nbmax_mode = nDsize[m];
  }
  s->i_to_l = (int*)malloc(sizeof(int) * D * s->nbmax_mode);
  for (int m = 0; m < D; ++m)
    for (int n = 1; n <= s->nbmax_mode; ++n)
      s->i_to_l[m * s->nbmax_mode + n - 1] = l_of_n(A_nb[m], B_nb[m], n, L);
  s->N = enum_type5p(D, nDsize, s->i_to_l, s->nbmax_mode, LB, &s->packed);

  /* Smolyak terms, nDindex type -5: l_i in [0..L], Lmin <= sum l <= L, first
   * index fastest (ADD_ONE_TO_nDindex_type5m, sub_module_nDindex.f90:2737-2791). */
  {
    long long cap = 256, n = 0;
    int* buf = (int*)malloc(sizeof(int) * D * cap);
    int v[ORC_MAXD];
    for (int i = 0; i < D; ++i) v[i] = 0;
    for (;;) {
      int Ls = 0;
      for (int i = 0; i < D; ++i) Ls += v[i];
      if (Ls >= s->Lmin && Ls <= L) {
        if (n == cap) { cap *= 2; buf = (int*)realloc(buf, sizeof(int) * D * cap); }
        memcpy(buf + n * D, v, sizeof(int) * D);
        n++;
      }
      int i = 0;
      v[0]++;
      for (;;) {
        int Lp = 0;
        for (int k = 0; k < D; ++k) Lp += v[k];
        if (Lp <= L) break;
        if (i == D - 1) goto done_terms;
        v[i] = 0;
        v[i + 1]++;
        i++;
      }
    }
  done_terms:
    s->nb_SG = n;
    s->tab_l = buf;
  }
  /* weights: calc_Weight_OF_SRep (sub_module_param_SGType2.f90:770-866) */
  s->weight = (double*)malloc(sizeof(double) * s->nb_SG);
  for (long long t = 0; t < s->nb_SG; ++t) {
    int Ls = 0;
    for (int i = 0; i < D; ++i) Ls += s->tab_l[t * D + i];
    int dL = L - Ls;
    if (dL < 0 || dL > D - 1) { s->weight[t] = 0.0; continue; }
    double c = 1.0;                             /* binomial(D-1, dL) */
    for (int k = 1; k <= dL; ++k) c = c * (double)(D - 1 - dL + k) / (double)k;
    c = (double)llround(c);
    s->weight[t] = (dL % 2 == 0) ? c : -c;
  }
  /* sizes and offsets (sub_quadra_SparseBasis.f90:1268-1318) */
  s->off_nb = (long long*)malloc(sizeof(long long) * (s->nb_SG + 1));
  s->off_nq = (long long*)malloc(sizeof(long long) * (s->nb_SG + 1));
  s->off_nb[0] = s->off_nq[0] = 0;
  s->max_nb = s->max_nq = 0;
  for (long long t = 0; t < s->nb_SG; ++t) {
    long long nb = 1, nq = 1;
    for (int i = 0; i < D; ++i) {
      int l = s->tab_l[t * D + i];
      nb *= s->nb_of_l[i * (L + 1) + l];
      nq *= s->nq_of_l[i * (L + 1) + l];
    }
    s->off_nb[t + 1] = s->off_nb[t] + nb;
    s->off_nq[t + 1] = s->off_nq[t] + nq;
    if (nb > s->max_nb) s->max_nb = (int)nb;
    if (nq > s->max_nq) s->max_nq = (int)nq;
  }
  s->sum_nb = s->off_nb[s->nb_SG];
  s->sum_nq = s->off_nq[s->nb_SG];
  /* gather map: Set_tables_FOR_SmolyakRepBasis_TO_tabPackedBasis
   * (sub_module_basis_BtoG_GtoB_SG4.f90:630-954): DP index with mode 1
   * fastest (ADD_ONE_TO_nDval_m1), 0 when sum L_i(n_i) > LB, else the
   * 1-based position of the tuple in the packed enumeration. */
  s->map = (int*)malloc(sizeof(int) * (s->sum_nb > 0 ? s->sum_nb : 1));
  cmp_tuple_D = D;
  for (long long t = 0; t < s->nb_SG; ++t) {
    int nbm[ORC_MAXD], v[ORC_MAXD];
    for (int i = 0; i < D; ++i) {
      nbm[i] = s->nb_of_l[i * (L + 1) + s->tab_l[t * D + i]];
      v[i] = 1;
    }
    long long nb_t = s->off_nb[t + 1] - s->off_nb[t];
    for (long long k = 0; k < nb_t; ++k) {
      int Ls = 0;
      for (int i = 0; i < D; ++i) Ls += s->i_to_l[i * s->nbmax_mode + v[i] - 1];
      int idx = 0;
      if (Ls <= LB) {
        const int* hit = (const int*)bsearch(v, s->packed, (size_t)s->N, sizeof(int) * D, cmp_tuple);
        idx = hit ? (int)((hit - s->packed) / D) + 1 : 0;
      }
      s->map[s->off_nb[t] + k] = idx;
      for (int i = 0; i < D; ++i) {           /* ADD_ONE_TO_nDval_m1 */
        v[i]++;
        if (v[i] <= nbm[i]) break;
        v[i] = 1;
      }
    }
  }
  return s;
}

void orc_destroy(orc_sg4* s) {
  if (!s) return;
  for (int k = 0; k < s->D * (s->L + 1); ++k) {
    orc_basis1* b = &s->b[k];
    free(b->x); free(b->w); free(b->d0); free(b->d1); free(b->d2);
    free(b->bgw); free(b->d1gg); free(b->d2gg);
  }
  free(s->b); free(s->nb_of_l); free(s->nq_of_l); free(s->i_to_l);
  free(s->packed); free(s->tab_l); free(s->weight); free(s->off_nb); free(s->off_nq);
  free(s->map);
  free(s);
}

void orc_sizes(const orc_sg4* s, long long* z) {
  z[0] = s->N; z[1] = s->nb_SG; z[2] = s->sum_nb; z[3] = s->sum_nq;
  z[4] = s->max_nb; z[5] = s->max_nq; z[6] = s->D; z[7] = s->L;
}

void orc_tables(const orc_sg4* s, int* tab_l, double* weight, int* map, int* packed) {
  if (tab_l) memcpy(tab_l, s->tab_l, sizeof(int) * s->nb_SG * s->D);
  if (weight) memcpy(weight, s->weight, sizeof(double) * s->nb_SG);
  if (map) memcpy(map, s->map, sizeof(int) * s->sum_nb);
  if (packed) memcpy(packed, s->packed, sizeof(int) * s->N * s->D);
}

void orc_basis1d(const orc_sg4* s, int mode, int l, double* x, double* w, double* d0,
                 double* d1, double* d2, double* RBGwrho, double* d1GG, double* d2GG) {
  const orc_basis1* b = &s->b[mode * (s->L + 1) + l];
  int nq = b->nq, nb = b->nb;
  if (x) memcpy(x, b->x, sizeof(double) * nq);
  if (w) memcpy(w, b->w, sizeof(double) * nq);
  if (d0) memcpy(d0, b->d0, sizeof(double) * nq * nb);
  if (d1) memcpy(d1, b->d1, sizeof(double) * nq * nb);
  if (d2) memcpy(d2, b->d2, sizeof(double) * nq * nb);
  if (RBGwrho) memcpy(RBGwrho, b->bgw, sizeof(double) * nq * nb);
  if (d1GG) memcpy(d1GG, b->d1gg, sizeof(double) * nq * nq);
  if (d2GG) memcpy(d2GG, b->d2gg, sizeof(double) * nq * nq);
}

/* Rec_Qact_SG4_with_Tab_iq (sub_module_basis.f90:3979-4049) over every term. */
void orc_grid_points(const orc_sg4* s, double* Q) {
  int D = s->D;
  for (long long t = 0; t < s->nb_SG; ++t) {
    const orc_basis1* bs[ORC_MAXD];
    int iq[ORC_MAXD];
    for (int i = 0; i < D; ++i) {
      bs[i] = &s->b[i * (s->L + 1) + s->tab_l[t * D + i]];
      iq[i] = 0;
    }
    long long nq_t = s->off_nq[t + 1] - s->off_nq[t];
    for (long long p = 0; p < nq_t; ++p) {
      for (int i = 0; i < D; ++i) Q[(s->off_nq[t] + p) * D + i] = bs[i]->x[iq[i]];
      for (int i = 0; i < D; ++i) {
        if (++iq[i] < bs[i]->nq) break;
        iq[i] = 0;
      }
    }
  }
}

/* ------------------------------------------------------------------------ */
/* Per-term kernels, instantiated in double and in long double.              */
/* ------------------------------------------------------------------------ */
#define REAL double
#define ORC_FN(name) name##_d
#define ORC_HPSI_NAME orc_hpsi
#include "sg4_oracle_hpsi.inc"
#undef REAL
#undef ORC_FN
#undef ORC_HPSI_NAME
#define REAL long double
#define ORC_FN(name) name##_ld
#define ORC_HPSI_NAME orc_hpsi_ld
#include "sg4_oracle_hpsi.inc"
#undef REAL
#undef ORC_FN
#undef ORC_HPSI_NAME
