// sg4_setup.cpp -- host-side SG4 tables for harmonic-oscillator bases.
//
// Builds what ElVibRot's RecSparseGrid_ForDP_type4
// (SRC/sub_Basis/sub_quadra_SparseBasis.f90:922-1434) leaves in
// para_Op%BasisnD for "HO"/"Hm" primitive bases, so that a caller without a
// Fortran front-end can fill an evr_sg4_desc:
//   * 1-D Gauss-Hermite grids and normalised Hermite functions with first and
//     second derivatives (sub_quadra_herm.f90:48-244,
//     sub_polyortho.f90:1090-1190), scaled by Q0/scaleQ
//     (sub_module_basis.f90:1499-1585);
//   * dnRBGwrho = dnRGB^T diag(wrho) (sub_module_basis.f90:1949-2013) and the
//     grid-grid derivative matrices dnRGG = dnRGB%d1,d2 . pinv(dnRGB%d0)
//     (sub_module_basis.f90:2048-2329);
//   * the packed basis (nDindex type 5p, last index fastest, sum L_i <= LB),
//     the Smolyak terms (type -5, first index fastest, Lmin <= |l| <= L),
//     WeightSG (sub_module_param_SGType2.f90:770-866) and the gather map
//     tab_iB_OF_SRep_TO_iB (sub_module_basis_BtoG_GtoB_SG4.f90:630-954).
// Numerics are done in long double: Golub-Welsch (implicit QL) nodes with a
// Newton polish, Christoffel weights, Hermite functions by the normalised
// three-term recurrence, the pseudo-inverse by Householder QR.  The packed
// index of a tuple is computed by combinatorial ranking instead of a search.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "evr_sg4.h"
#include "sg4_internal.h"

namespace evr {

typedef long double ld;

// ---------------------------------------------------------------- quadrature
// Nodes: eigenvalues of the symmetric tridiagonal Jacobi matrix of the
// Hermite weight exp(-x^2) (zero diagonal, off-diagonal sqrt(k/2)) -- the
// Golub-Welsch construction (G. H. Golub and J. H. Welsch, "Calculation of
// Gauss quadrature rules", Math. Comp. 23 (1969) 221-230) -- by the implicit
// QL method with Wilkinson shifts (eigenvalues only; the EISPACK tql1 scheme
// of Bowdler, Martin, Reinsch and Wilkinson, Numer. Math. 11 (1968) 293-306),
// then Newton steps on the orthonormal recurrence.
static void jacobi_ql(int n, std::vector<ld>& d, std::vector<ld>& e) {
  for (int l = 0; l < n; ++l) {
    int iter = 0, m;
    do {
      for (m = l; m < n - 1; ++m) {
        ld dd = std::fabs(d[m]) + std::fabs(d[m + 1]);
        if (std::fabs(e[m]) <= 1e-30L * dd) break;
      }
      if (m != l) {
        if (++iter > 200) break;
        ld g = (d[l + 1] - d[l]) / (2.0L * e[l]);
        ld r = std::hypot(g, (ld)1.0L);
        g = d[m] - d[l] + e[l] / (g + (g >= 0 ? std::fabs(r) : -std::fabs(r)));
        ld s = 1.0L, c = 1.0L, p = 0.0L;
        int i;
        for (i = m - 1; i >= l; --i) {
          ld f = s * e[i], b = c * e[i];
          r = std::hypot(f, g);
          e[i + 1] = r;
          if (r == 0.0L) {
            d[i + 1] -= p;
            e[m] = 0.0L;
            break;
          }
          s = f / r;
          c = g / r;
          g = d[i + 1] - p;
          r = (d[i] - g) * s + 2.0L * c * b;
          p = s * r;
          d[i + 1] = g + p;
          g = c * r - b;
        }
        if (r == 0.0L && i >= l) continue;
        d[l] -= p;
        e[l] = g;
        e[m] = 0.0L;
      }
    } while (m != l);
  }
}

// orthonormal Hermite functions psi_k(x) = p_k(x) exp(-x^2/2), k = 0..n
static void hermite_functions(int n, ld x, ld* psi) {
  psi[0] = std::pow(std::acos(-1.0L), -0.25L) * std::exp(-0.5L * x * x);
  if (n >= 1) psi[1] = std::sqrt(2.0L) * x * psi[0];
  for (int k = 1; k < n; ++k)
    psi[k + 1] = std::sqrt(2.0L / (k + 1)) * x * psi[k] - std::sqrt((ld)k / (k + 1)) * psi[k - 1];
}

void gauss_hermite(int nq, std::vector<double>& x, std::vector<double>& wrho) {
  std::vector<ld> d(nq, 0.0L), e(nq, 0.0L);
  for (int k = 0; k + 1 < nq; ++k) e[k] = std::sqrt((ld)(k + 1) / 2.0L);
  jacobi_ql(nq, d, e);
  std::vector<ld> r(d.begin(), d.end());
  for (int i = 0; i < nq; ++i)
    for (int j = i + 1; j < nq; ++j)
      if (r[j] < r[i]) std::swap(r[i], r[j]);
  std::vector<ld> psi(nq + 1);
  for (int i = 0; i < nq; ++i) {
    for (int it = 0; it < 3; ++it) {   // Newton: p_n / p_n', p_n' = sqrt(2n) p_{n-1}
      hermite_functions(nq, r[i], psi.data());
      ld den = std::sqrt(2.0L * nq) * psi[nq - 1];
      if (den != 0.0L) r[i] -= psi[nq] / den;
    }
  }
  for (int i = 0; i < nq / 2; ++i) {   // exact symmetry of the rule
    ld a = 0.5L * (r[nq - 1 - i] - r[i]);
    r[i] = -a;
    r[nq - 1 - i] = a;
  }
  if (nq % 2) r[nq / 2] = 0.0L;
  x.resize(nq);
  wrho.resize(nq);
  for (int i = 0; i < nq; ++i) {
    hermite_functions(nq - 1, r[i], psi.data());
    ld s = 0.0L;
    for (int k = 0; k < nq; ++k) s += psi[k] * psi[k];
    x[i] = (double)r[i];
    wrho[i] = (double)(1.0L / s);  // Christoffel weight times exp(x^2)
  }
}

// --------------------------------------------------------------- 1-D basis
// Householder QR of the nq x nb (column-major) matrix A; returns the
// pseudo-inverse P = R^{-1} Q^T (nb x nq, column-major) in long double.
static void pseudo_inverse(int nq, int nb, const std::vector<ld>& A, std::vector<ld>& P) {
  std::vector<ld> R(A);
  std::vector<ld> Qt((size_t)nq * nq, 0.0L);  // Q^T accumulated, column-major
  for (int i = 0; i < nq; ++i) Qt[i + (size_t)nq * i] = 1.0L;
  std::vector<ld> v(nq);
  for (int k = 0; k < nb; ++k) {
    ld nrm = 0.0L;
    for (int i = k; i < nq; ++i) nrm += R[i + (size_t)nq * k] * R[i + (size_t)nq * k];
    nrm = std::sqrt(nrm);
    if (nrm == 0.0L) continue;
    ld alpha = R[k + (size_t)nq * k] > 0 ? -nrm : nrm;
    for (int i = 0; i < nq; ++i) v[i] = 0.0L;
    v[k] = R[k + (size_t)nq * k] - alpha;
    for (int i = k + 1; i < nq; ++i) v[i] = R[i + (size_t)nq * k];
    ld vv = 0.0L;
    for (int i = k; i < nq; ++i) vv += v[i] * v[i];
    if (vv == 0.0L) continue;
    for (int j = 0; j < nb; ++j) {
      ld s = 0.0L;
      for (int i = k; i < nq; ++i) s += v[i] * R[i + (size_t)nq * j];
      s = 2.0L * s / vv;
      for (int i = k; i < nq; ++i) R[i + (size_t)nq * j] -= s * v[i];
    }
    for (int j = 0; j < nq; ++j) {
      ld s = 0.0L;
      for (int i = k; i < nq; ++i) s += v[i] * Qt[i + (size_t)nq * j];
      s = 2.0L * s / vv;
      for (int i = k; i < nq; ++i) Qt[i + (size_t)nq * j] -= s * v[i];
    }
  }
  // P = R(0:nb,0:nb)^{-1} (Q^T)(0:nb, :)
  P.assign((size_t)nb * nq, 0.0L);
  for (int c = 0; c < nq; ++c)
    for (int i = nb - 1; i >= 0; --i) {
      ld s = Qt[i + (size_t)nq * c];
      for (int j = i + 1; j < nb; ++j) s -= R[i + (size_t)nq * j] * P[j + (size_t)nb * c];
      P[i + (size_t)nb * c] = s / R[i + (size_t)nq * i];
    }
}

static void build_mode_level(Basis1D& b, int nb, int nq, double Q0, double scaleQ) {
  b.nb = nb;
  b.nq = nq;
  std::vector<double> xr, wr;
  gauss_hermite(nq, xr, wr);
  std::vector<ld> f0((size_t)nq * nb), f1((size_t)nq * nb), f2((size_t)nq * nb);
  std::vector<ld> psi(nb + 2);
  for (int k = 0; k < nq; ++k) {
    ld x = xr[k];
    hermite_functions(nb, x, psi.data());
    for (int i = 0; i < nb; ++i) {
      ld pm = i > 0 ? psi[i - 1] : 0.0L;
      f0[k + (size_t)nq * i] = psi[i];
      f1[k + (size_t)nq * i] = std::sqrt((ld)i / 2.0L) * pm - std::sqrt((ld)(i + 1) / 2.0L) * psi[i + 1];
      f2[k + (size_t)nq * i] = (x * x - (ld)(2 * i + 1)) * psi[i];
    }
  }
  const bool scaled = !(Q0 == 0.0 && scaleQ == 1.0);
  ld s = scaleQ;
  ld sd0 = scaled ? std::sqrt(s) : 1.0L, sd1 = scaled ? std::sqrt(s) * s : 1.0L,
     sd2 = scaled ? std::sqrt(s) * s * s : 1.0L;
  b.x.resize(nq);
  b.w.resize(nq);
  for (int k = 0; k < nq; ++k) {
    b.x[k] = scaled ? Q0 + xr[k] / scaleQ : xr[k];
    b.w[k] = scaled ? wr[k] * (1.0 / scaleQ) : wr[k];
  }
  std::vector<ld> A((size_t)nq * nb);
  b.RGB.resize((size_t)nq * nb);
  for (size_t k = 0; k < A.size(); ++k) {
    b.RGB[k] = (double)(f0[k] * sd0);
    A[k] = b.RGB[k];
  }
  std::vector<ld> P;
  pseudo_inverse(nq, nb, A, P);
  b.d1GG.assign((size_t)nq * nq, 0.0);
  b.d2GG.assign((size_t)nq * nq, 0.0);
  for (int r = 0; r < nq; ++r)
    for (int c = 0; c < nq; ++c) {
      ld a1 = 0.0L, a2 = 0.0L;
      for (int k = 0; k < nb; ++k) {
        // derivative matrices rounded to double first, as the reference stores them
        ld g1 = (double)(f1[r + (size_t)nq * k] * sd1), g2 = (double)(f2[r + (size_t)nq * k] * sd2);
        a1 += g1 * P[k + (size_t)nb * c];
        a2 += g2 * P[k + (size_t)nb * c];
      }
      b.d1GG[r + (size_t)nq * c] = (double)a1;
      b.d2GG[r + (size_t)nq * c] = (double)a2;
    }
  b.RBGw.resize((size_t)nb * nq);
  for (int i = 0; i < nb; ++i)
    for (int k = 0; k < nq; ++k) b.RBGw[i + (size_t)nb * k] = b.RGB[k + (size_t)nq * i] * b.w[k];
}

// --------------------------------------------------------------- index sets
// Packed basis ranking.  cnt[i][b] = number of suffix tuples (n_i..n_D) whose
// level sum is <= b; levels of the n-th function: lev(n) = min{l: nb(l) >= n}.
struct PackedRanker {
  int D, LB;
  std::vector<std::vector<int>> lev;                 // [D][nDsize]
  std::vector<std::vector<long long>> cnt;           // [D+1][LB+1]
  void init(int D_, int LB_, const std::vector<std::vector<int>>& lev_) {
    D = D_;
    LB = LB_;
    lev = lev_;
    cnt.assign(D + 1, std::vector<long long>(LB + 1, 0));
    for (int b = 0; b <= LB; ++b) cnt[D][b] = 1;
    for (int i = D - 1; i >= 0; --i)
      for (int b = 0; b <= LB; ++b) {
        long long s = 0;
        for (int lv : lev[i])
          if (lv <= b) s += cnt[i + 1][b - lv];
        cnt[i][b] = s;
      }
  }
  long long size() const { return cnt[0][LB]; }
  // 0-based rank of n (1-based entries), or -1 if outside the set
  long long rank(const int* n) const {
    long long r = 0;
    int budget = LB;
    for (int i = 0; i < D; ++i) {
      for (int m = 1; m < n[i]; ++m) {
        int lv = lev[i][m - 1];
        if (lv <= budget) r += cnt[i + 1][budget - lv];
      }
      budget -= lev[i][n[i] - 1];
      if (budget < 0) return -1;
    }
    return r;
  }
};

}  // namespace evr

using namespace evr;

extern "C" int evr_sg4_basis_build_ho(int D, int L, int LB, int A_nb, int B_nb, int A_nq, int B_nq,
                                      const double* Q0, const double* scaleQ, evr_sg4_basis** out) {
  if (!out) return set_error(EVR_ERR_ARG, "evr_sg4_basis_build_ho: out is NULL");
  *out = nullptr;
  if (D < 1 || D > EVR_MAXD) return set_error(EVR_ERR_ARG, "evr_sg4_basis_build_ho: need 1 <= D <= %d", EVR_MAXD);
  std::vector<int> a(D, A_nb), b(D, B_nb), c(D, A_nq), d(D, B_nq);
  return evr_sg4_basis_build_ho_modes(D, L, LB, a.data(), b.data(), c.data(), d.data(), Q0, scaleQ, out);
}

extern "C" int evr_sg4_basis_build_ho_modes(int D, int L, int LB, const int* A_nb_m, const int* B_nb_m,
                                            const int* A_nq_m, const int* B_nq_m, const double* Q0,
                                            const double* scaleQ, evr_sg4_basis** out) {
  if (!out) return set_error(EVR_ERR_ARG, "evr_sg4_basis_build_ho: out is NULL");
  *out = nullptr;
  if (D < 1 || D > EVR_MAXD || L < 0 || LB < 0)
    return set_error(EVR_ERR_ARG, "evr_sg4_basis_build_ho: need 1 <= D <= %d, L >= 0, LB >= 0", EVR_MAXD);
  if (!A_nb_m || !B_nb_m || !A_nq_m || !B_nq_m) return set_error(EVR_ERR_ARG, "evr_sg4_basis_build_ho: NULL rule");
  for (int i = 0; i < D; ++i) {
    const int A_nb = A_nb_m[i], B_nb = B_nb_m[i], A_nq = A_nq_m[i], B_nq = B_nq_m[i];
    if (A_nb < 1 || B_nb < 0 || A_nq < 1 || B_nq < 0)
      return set_error(EVR_ERR_ARG, "evr_sg4_basis_build_ho: nb(0), nq(0) must be >= 1 (mode %d)", i);
    if (A_nb > A_nq || B_nb > B_nq)  // sub_read_data.f90:804 rejects nb > nq growth
      return set_error(EVR_ERR_ARG, "evr_sg4_basis_build_ho: L_TO_nb must not exceed L_TO_nq (mode %d)", i);
    if (A_nq + B_nq * L > EVR_MAXN)
      return set_error(EVR_ERR_ARG, "evr_sg4_basis_build_ho: nq(L)=%d exceeds %d (mode %d)", A_nq + B_nq * L,
                       EVR_MAXN, i);
  }
  if (scaleQ)
    for (int i = 0; i < D; ++i)
      if (!(scaleQ[i] > 0.0)) return set_error(EVR_ERR_ARG, "evr_sg4_basis_build_ho: scaleQ must be > 0");
  evr_sg4_basis* b = new evr_sg4_basis();
  b->D = D;
  b->L = L;
  b->LB = LB;
  b->nb_of_l.resize((size_t)D * (L + 1));
  b->nq_of_l.resize((size_t)D * (L + 1));
  b->mats.resize((size_t)D * (L + 1));
  for (int i = 0; i < D; ++i)
    for (int l = 0; l <= L; ++l) {
      int nb = A_nb_m[i] + B_nb_m[i] * l, nq = A_nq_m[i] + B_nq_m[i] * l;
      b->nb_of_l[i * (L + 1) + l] = nb;
      b->nq_of_l[i * (L + 1) + l] = nq;
      build_mode_level(b->mats[i * (L + 1) + l], nb, nq, Q0 ? Q0[i] : 0.0, scaleQ ? scaleQ[i] : 1.0);
    }
  // concatenated arrays in descriptor order
  for (auto& m : b->mats) {
    b->cat_x.insert(b->cat_x.end(), m.x.begin(), m.x.end());
    b->cat_RGB.insert(b->cat_RGB.end(), m.RGB.begin(), m.RGB.end());
    b->cat_RBGw.insert(b->cat_RBGw.end(), m.RBGw.begin(), m.RBGw.end());
    b->cat_d1.insert(b->cat_d1.end(), m.d1GG.begin(), m.d1GG.end());
    b->cat_d2.insert(b->cat_d2.end(), m.d2GG.begin(), m.d2GG.end());
  }
  // packed basis
  std::vector<std::vector<int>> lev(D);
  for (int i = 0; i < D; ++i) {
    int nsz = b->nb_of_l[i * (L + 1) + L];
    lev[i].resize(nsz);
    for (int n = 1; n <= nsz; ++n) {
      int lv = 0;
      while (lv <= L && b->nb_of_l[i * (L + 1) + lv] < n) ++lv;
      lev[i][n - 1] = lv;
    }
  }
  PackedRanker pr;
  pr.init(D, LB, lev);
  b->N = pr.size();
  if (b->N > 2147483647LL) {
    delete b;
    return set_error(EVR_ERR_ARG, "evr_sg4_basis_build_ho: packed basis too large for int32 map");
  }
  // Smolyak terms: Lmin <= |l| <= L, first index fastest
  const int Lmin = std::max(0, L - D + 1);
  std::vector<int> l(D, 0);
  for (;;) {
    int s = 0;
    for (int v : l) s += v;
    if (s >= Lmin && s <= L) b->tab_l.insert(b->tab_l.end(), l.begin(), l.end());
    int i = 0;
    for (;;) {
      l[i]++;
      s = 0;
      for (int v : l) s += v;
      if (s <= L) break;
      l[i] = 0;
      if (++i == D) goto terms_done;
    }
  }
terms_done:
  b->nb_SG = (long long)b->tab_l.size() / D;
  b->weight.resize(b->nb_SG);
  for (long long t = 0; t < b->nb_SG; ++t) {
    int s = 0;
    for (int i = 0; i < D; ++i) s += b->tab_l[t * D + i];
    int dl = L - s;
    double c = 0.0;
    if (dl >= 0 && dl <= D - 1) {
      long double bin = 1.0L;
      for (int k = 1; k <= dl; ++k) bin = bin * (D - dl - 1 + k) / k;
      c = (double)std::llround(bin);
      if (dl % 2) c = -c;
    }
    b->weight[t] = c;
  }
  // gather map
  for (long long t = 0; t < b->nb_SG; ++t) {
    int nbm[EVR_MAXD], n[EVR_MAXD];
    long long nbt = 1;
    for (int i = 0; i < D; ++i) {
      nbm[i] = b->nb_of_l[i * (L + 1) + b->tab_l[t * D + i]];
      n[i] = 1;
      nbt *= nbm[i];
    }
    for (long long k = 0; k < nbt; ++k) {
      long long r = pr.rank(n);
      b->map.push_back(r < 0 ? 0 : (int)(r + 1));
      for (int i = 0; i < D; ++i) {
        if (++n[i] <= nbm[i]) break;
        n[i] = 1;
      }
    }
  }
  *out = b;
  return EVR_OK;
}

extern "C" int evr_sg4_basis_desc(const evr_sg4_basis* b, evr_sg4_desc* d) {
  if (!b || !d) return set_error(EVR_ERR_ARG, "evr_sg4_basis_desc: NULL argument");
  d->D = b->D;
  d->L = b->L;
  d->LB = b->LB;
  d->nb0 = 1;
  d->nb_of_l = b->nb_of_l.data();
  d->nq_of_l = b->nq_of_l.data();
  d->x = b->cat_x.data();
  d->RGB = b->cat_RGB.data();
  d->RBGwrho = b->cat_RBGw.data();
  d->d1GG = b->cat_d1.data();
  d->d2GG = b->cat_d2.data();
  d->nb_SG = b->nb_SG;
  d->tab_l = b->tab_l.data();
  d->weight = b->weight.data();
  d->map = b->map.data();
  d->N = b->N;
  return EVR_OK;
}

extern "C" int evr_sg4_basis_grid_points(const evr_sg4_basis* b, double* Q) {
  if (!b || !Q) return set_error(EVR_ERR_ARG, "evr_sg4_basis_grid_points: NULL argument");
  const int D = b->D, L = b->L;
  long long p0 = 0;
  for (long long t = 0; t < b->nb_SG; ++t) {
    const Basis1D* m[EVR_MAXD];
    int iq[EVR_MAXD];
    long long nqt = 1;
    for (int i = 0; i < D; ++i) {
      m[i] = &b->mats[i * (L + 1) + b->tab_l[t * D + i]];
      iq[i] = 0;
      nqt *= m[i]->nq;
    }
    for (long long p = 0; p < nqt; ++p) {
      for (int i = 0; i < D; ++i) Q[(p0 + p) * D + i] = m[i]->x[iq[i]];
      for (int i = 0; i < D; ++i) {
        if (++iq[i] < m[i]->nq) break;
        iq[i] = 0;
      }
    }
    p0 += nqt;
  }
  return EVR_OK;
}

extern "C" void evr_sg4_basis_free(evr_sg4_basis* b) { delete b; }

extern "C" int evr_sg4_desc_sizes(const evr_sg4_desc* d, long long* out) {
  if (!d || !out) return set_error(EVR_ERR_ARG, "evr_sg4_desc_sizes: NULL argument");
  DescSizes z;
  int rc = desc_sizes(d, &z);
  if (rc) return rc;
  out[0] = d->N;
  out[1] = d->nb_SG;
  out[2] = z.sum_nb;
  out[3] = z.sum_nq;
  out[4] = z.max_nb;
  out[5] = z.max_nq;
  out[6] = d->D;
  out[7] = d->L;
  return EVR_OK;
}
