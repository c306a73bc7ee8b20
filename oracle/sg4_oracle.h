/*
 * sg4_oracle.h -- CPU oracle for ElVibRot's Smolyak type-4 (SG4) H.psi.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of the reference
 * algorithm, used by tests/ as the parity checker and by bench.py as the
 * timed CPU baseline ("reference" arm).  The product (elvibrot_gb300/) never
 * links, imports or calls it.
 *
 * Parity pin: the restatement is checked against the reference's own known
 * answers -- Internal_data/HermQuadra/herm{1..40}.txt (1-D Gauss-Hermite nodes
 * and weights) and the Henon-Heiles SG4 Davidson levels in
 * Working_tests/MPI_tests/{6D,21D}_Davidson_S0/benchmark -- through fixtures
 * committed under tests/golden/.
 *
 * Every function cites the reference routine it restates (paths relative to
 * the ElVibRot source tree).
 */
#ifndef SG4_ORACLE_H
#define SG4_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_sg4 orc_sg4;

/* Builds the HO (Hermite) SG4 basis: 1-D bases for every (mode, level),
 * packed basis (nDindex type 5p), Smolyak terms (type -5), weights and the
 * packed<->term gather map.
 * nb(l) = A_nb + B_nb*l, nq(l) = A_nq + B_nq*l (L_TO_n_type 0, expo 1).
 * Restates RecSparseGrid_ForDP_type4 (SRC/sub_Basis/sub_quadra_SparseBasis.f90:922-1434). */
orc_sg4* orc_create(int D, int L, int LB, int A_nb, int B_nb, int A_nq, int B_nq,
                    const double* Q0, const double* scaleQ);
/* The same with one nb/nq rule per mode (arrays of D), as the reference reads
 * L_TO_nq_A/B per primitive basis (&basis_nD). */
orc_sg4* orc_create_modes(int D, int L, int LB, const int* A_nb, const int* B_nb, const int* A_nq,
                          const int* B_nq, const double* Q0, const double* scaleQ);
void orc_destroy(orc_sg4* s);

/* sizes[0..7] = N (packed size), nb_SG, sum_nb, sum_nq, max_nb_term, max_nq_term, D, L */
void orc_sizes(const orc_sg4* s, long long* sizes);

/* Term tables: tab_l[nb_SG*D] (term-major), weight[nb_SG], map[sum_nb] (1-based
 * packed index, 0 = not in the packed basis), packed[N*D] (1-based n_i). */
void orc_tables(const orc_sg4* s, int* tab_l, double* weight, int* map, int* packed);

/* 1-D basis of (mode, level): x[nq], w[nq] (wrho), d0,d1,d2 [nq*nb] (column-major
 * nq x nb), RBGwrho [nb*nq] (column-major nb x nq), d1GG,d2GG [nq*nq]. */
void orc_basis1d(const orc_sg4* s, int mode, int l, double* x, double* w, double* d0,
                 double* d1, double* d2, double* RBGwrho, double* d1GG, double* d2GG);

/* Coordinates of every term grid point, Q[sum_nq*D] (point-major), terms in
 * Smolyak order, points mode-1-fastest (Rec_Qact_SG4_with_Tab_iq). */
void orc_grid_points(const orc_sg4* s, double* Q);

/* Operator description for orc_hpsi.
 *  type 0 : y = V.x
 *  type 1 : y = sum_terms F_t Der_t x, terms (0,0),(i<=j),(i,0) in the
 *           reference order; F2[D*D] (i,j)-> constant coefficient of d_i d_j
 *           (row-major, i<=j used), F1[D] constant coefficient of d_i;
 *           F2_grid[D*D*sum_nq] (term (i,j) at [(i*D+j)*sum_nq + point]) and
 *           F1_grid[D*sum_nq], when given, replace them with Q-dependent
 *           coefficients (OpGrid(iterm)%Grid), a grid zero everywhere being
 *           a grid_zero term.
 *  type 10: y = -1/2 sum_i d_i (Jac sum_j G_ji d_j (s x)) / (Jac s) + V x,
 *           s = sqRhoOVERJac.  G[sum_nq*D*D] per term laid out (iq, j, i) with
 *           iq fastest (GGiq), NULL = identity; Jac, sqRho NULL = 1.
 *  V[sum_nq] concatenated per term (OpGrid%Grid layout), NULL = 0.
 *  Fields given in analytic form instead of grids are evaluated term by
 *  term, once per call, at the term's grid points, as the reference's type-10
 *  path evaluates its fields per term inside the term loop
 *  (get_OpGrid_type10_OF_ONEDP_FOR_SG4, sub_OpPsi_SG4.f90:2536, called at
 *  :1553; V per point through get_d0MatOp_AT_Qact):
 *    V (when V is NULL and V_nterms > 0) = sum_t V_coef[t] prod_i Q_i^V_expo[t*D+i];
 *    G (type 10, when G is NULL and G0 or G1 is given)
 *      G_ij(Q) = G0[i*D+j] (identity if NULL) + sum_k G1[(i*D+j)*D+k] Q_k. */
typedef struct {
  int type;
  const double* V;
  const double* G;
  const double* Jac;
  const double* sqRho;
  const double* F2;
  const double* F1;
  int V_nterms;
  const double* V_coef;
  const int* V_expo;
  const double* G0;
  const double* G1;
  const double* F2_grid; /* type 1: Q-dependent coefficients, replace F2 / F1 when given */
  const double* F1_grid;
} orc_op;

/* hpsi[N*nrhs] = H psi[N*nrhs] (column-major, ld = N).  nthreads <= 0 = all. */
int orc_hpsi(const orc_sg4* s, const orc_op* op, int nrhs, const double* psi,
             double* hpsi, int nthreads);

/* Same as orc_hpsi with every intermediate in long double (x87 80-bit on
 * x86-64, IEEE binary128 on aarch64): the accuracy yardstick for the tests. */
int orc_hpsi_ld(const orc_sg4* s, const orc_op* op, int nrhs, const double* psi,
                double* hpsi, int nthreads);

/* Gauss-Hermite quadrature of nq points: x[nq], w[nq] (weight for exp(-x^2) f),
 * wrho[nq] = w exp(x^2).  Restates hercom/herm*.txt (sub_quadra_herm.f90:48-244). */
void orc_gauss_hermite(int nq, double* x, double* w, double* wrho);

#ifdef __cplusplus
}
#endif
#endif
