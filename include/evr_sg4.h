/*
 * evr_sg4.h -- C ABI of the GB300 (sm_103a) Smolyak type-4 (SG4) H.psi.
 *
 * Drop-in boundary for ElVibRot's operator action on an SG4 basis:
 *
 *   SUBROUTINE sub_TabOpPsi(TabPsi, TabOpPsi, para_Op, ...)
 *       SRC/sub_Operator/sub_OpPsi.f90:705, SG4 branch :864-884
 *   -> SUBROUTINE sub_TabOpPsi_FOR_SGtype4(Psi, OpPsi, para_Op)
 *       SRC/sub_Operator/sub_OpPsi_SG4.f90:681-977
 *
 * Every entry point returns an int status (EVR_OK = 0) and never exits,
 * aborts or traps; evr_sg4_last_error() gives the message of the last
 * failure on the calling thread.  No CUDA or torch types appear in the
 * signatures: streams are passed as void* (a cudaStream_t, NULL = legacy
 * default stream).  Vectors are column-major N x nrhs (Fortran order) with a
 * leading dimension, exactly the packed layout of param_psi%RvecB
 * (SRC/sub_WP/sub_module_psi_set_alloc.f90:56-169): index (ib0-1)*N + nDI,
 * nDI enumerating nDindB type 5p.  The library never frees caller memory.
 * A context is single-stream and not thread-safe; distinct contexts are
 * independent.
 */
#ifndef EVR_SG4_H
#define EVR_SG4_H

#ifdef __cplusplus
extern "C" {
#endif

#define EVR_OK 0
#define EVR_ERR_ARG 1      /* invalid argument / size (the reference STOPs) */
#define EVR_ERR_CUDA 2     /* a CUDA runtime call failed */
#define EVR_ERR_ALLOC 3    /* device or host allocation failed */
#define EVR_ERR_STATE 4    /* call order (e.g. hpsi before set_operator) */
#define EVR_ERR_TIMEOUT 5  /* a bounded device wait gave up */
#define EVR_ERR_NUMERIC 6  /* non-finite input or diverging iteration */

typedef struct evr_sg4_basis evr_sg4_basis; /* host-side tables */
typedef struct evr_sg4_ctx evr_sg4_ctx;     /* device-side operator */

/* ------------------------------------------------------------------------
 * Basis descriptor: the SG4 tables as ElVibRot holds them after
 * RecSparseGrid_ForDP_type4 (SRC/sub_Basis/sub_quadra_SparseBasis.f90:922).
 * A Fortran caller fills it from para_Op%BasisnD:
 *   nb_of_l/nq_of_l  <- tab_basisPrimSG(l,i)%nb / nq
 *   x                <- tab_basisPrimSG(l,i)%x(1,:)
 *   RGB              <- tab_basisPrimSG(l,i)%dnRGB%d0      (nq x nb)
 *   RBGwrho          <- tab_basisPrimSG(l,i)%dnRBGwrho%d0  (nb x nq)
 *   d1GG, d2GG       <- tab_basisPrimSG(l,i)%dnRGG%d1, %d2 (nq x nq)
 *   tab_l            <- para_SGType2%nDind_SmolyakRep%Tab_nDval (transposed)
 *   weight           <- BasisnD%WeightSG
 *   map              <- para_SGType2%tab_iB_OF_SRep_TO_iB
 *   N                <- BasisnD%nDindB%Max_nDI
 * Per-(mode,level) arrays are concatenated mode-major, level-minor
 * (i*(L+1)+l); matrices column-major.  Terms are in nDind_SmolyakRep order;
 * inside a term the DP index runs mode 1 fastest.
 * ---------------------------------------------------------------------- */
typedef struct {
  int D;                    /* number of modes */
  int L;                    /* Smolyak grid level (L_SparseGrid) */
  int LB;                   /* basis level (L_SparseBasis) */
  int nb0;                  /* channels (electronic states, nb_be), 1..8: a vector is nb0
                               blocks of N (RvecB((ie-1)*Max_nDI + iB)); nb0 > 1 takes
                               operator types 0, 1 and 10 with V as a grid */
  const int* nb_of_l;       /* [D*(L+1)] */
  const int* nq_of_l;       /* [D*(L+1)] */
  const double* x;          /* sum over (i,l) of nq */
  const double* RGB;        /* sum of nq*nb */
  const double* RBGwrho;    /* sum of nb*nq */
  const double* d1GG;       /* sum of nq*nq */
  const double* d2GG;       /* sum of nq*nq */
  long long nb_SG;          /* number of Smolyak terms */
  const int* tab_l;         /* [nb_SG*D] term-major */
  const double* weight;     /* [nb_SG] */
  const int* map;           /* [sum_nb], 1-based packed index, 0 = skipped */
  long long N;              /* packed basis size */
} evr_sg4_desc;

/* Sizes derived from a descriptor: out[0..7] = N, nb_SG, sum_nb, sum_nq,
 * max_nb_term, max_nq_term, D, L. */
int evr_sg4_desc_sizes(const evr_sg4_desc* d, long long* out);

/* ------------------------------------------------------------------------
 * Host builder for harmonic-oscillator (Hermite) primitive bases.
 * Restates RecSparseGrid_ForDP_type4 (sub_quadra_SparseBasis.f90:922-1434)
 * with basis "HO"/"Hm" per mode: nb(l) = A_nb + B_nb*l, nq(l) = A_nq + B_nq*l
 * (L_TO_n_type 0, expo 1), Gauss-Hermite grids (sub_quadra_herm.f90:48),
 * scaling x -> Q0 + x/scaleQ (sub_module_basis.f90:1499), dnRGG through the
 * pseudo-inverse of dnRGB%d0 (sub_module_basis.f90:2048), nDindB type 5p
 * and nDind_SmolyakRep type -5 (Ext_Lib/nDindex_loc), WeightSG
 * (sub_module_param_SGType2.f90:770) and tab_iB_OF_SRep_TO_iB
 * (sub_module_basis_BtoG_GtoB_SG4.f90:630).  Q0/scaleQ may be NULL (0, 1).
 * ---------------------------------------------------------------------- */
int evr_sg4_basis_build_ho(int D, int L, int LB, int A_nb, int B_nb, int A_nq, int B_nq,
                           const double* Q0, const double* scaleQ, evr_sg4_basis** out);
/* The same with one rule per mode (arrays of D): the reference reads
 * L_TO_nq_A/B (and L_TO_nb) per primitive basis (&basis_nD). */
int evr_sg4_basis_build_ho_modes(int D, int L, int LB, const int* A_nb, const int* B_nb, const int* A_nq,
                                 const int* B_nq, const double* Q0, const double* scaleQ, evr_sg4_basis** out);
/* Fills *d with pointers into the basis' own storage (valid until free). */
int evr_sg4_basis_desc(const evr_sg4_basis* b, evr_sg4_desc* d);
/* Coordinates of every term grid point: Q[sum_nq*D], point-major
 * (Rec_Qact_SG4_with_Tab_iq, sub_module_basis.f90:3979). */
int evr_sg4_basis_grid_points(const evr_sg4_basis* b, double* Q);
void evr_sg4_basis_free(evr_sg4_basis* b);

/* ------------------------------------------------------------------------
 * Device context.  Copies the descriptor's tables to the device.
 * ---------------------------------------------------------------------- */
int evr_sg4_create(const evr_sg4_desc* d, evr_sg4_ctx** out);
int evr_sg4_destroy(evr_sg4_ctx* c);

/* ------------------------------------------------------------------------
 * Operator.  Replaces param_Op%type_Op with its cached grids (OpGrid,
 * get_OpGrid_type0/1/10_OF_ONEDP_FOR_SG4, sub_OpPsi_SG4.f90:2536-3319):
 *   type 0  : y = V.x                                           (CASE 0 :1446)
 *   type 1  : y = V.x + sum_{i<=j} F2_ij d_i d_j x + sum_i F1_i d_i x
 *             (d_i d_i through dnRGG%d2, others through %d1)     (CASE 1 :1488)
 *   type 10 : y = -1/2 sum_i d_i(Jac sum_j G_ji d_j(s x)) / (Jac s) + V.x,
 *             s = sqRhoOVERJac                                  (CASE 10 :1546)
 * V is a grid (sum_nq values, OpGrid%Grid layout, terms concatenated) or a
 * polynomial sum_t coef_t prod_i Q_i^expo_ti evaluated on the device.  With
 * nb0 > 1 channels V is the electronic matrix on the grid:
 * V_grid[(a*nb0 + b)*sum_nq + point] couples channel b into channel a
 * (OpGrid(iterm)%Grid(:,a,b)), and the derivative terms act on every channel;
 * as a polynomial, V_coef holds nb0*nb0 blocks of V_nterms coefficients over
 * the same monomials (element (a, b) at V_coef[(a*nb0 + b)*V_nterms + t]),
 * the matrix the reference's get_d0MatOp_AT_Qact gives at each point
 * (SRC/sub_Operator/sub_PrimOp.f90:257); such fields stay resident.
 * G (type 10) is a grid GGiq(iq,j,i) per term, concatenated (sum_nq*D*D),
 * or the affine form G_ij(Q) = G0_ij + sum_k G1_ijk Q_k ([D*D], [D*D*D],
 * row-major ijk); neither = identity.  Jac / sqRho grids: NULL = 1.
 * F2 [D*D] row-major (entries i<=j used) and F1 [D]: constant coefficients.
 * F2_grid [D*D*nb0*nb0*sum_nq] (term (i, j), i <= j, channel pair (a, b) at
 * [((i*D + j)*nb0*nb0 + a*nb0 + b)*sum_nq + point]) and F1_grid
 * [D*nb0*nb0*sum_nq] (term i at [(i*nb0*nb0 + a*nb0 + b)*sum_nq + point]):
 * Q-dependent coefficients of the type-1 derivative terms (OpGrid(iterm)%Grid
 * when it is not grid_cte; element (a, b) couples channel b into channel a,
 * OpPsi(:,a) += GridOp(:,a,b,iterm) * Psi_ch(:,b)); when given they replace
 * F2 / F1.  Then every derivative term is applied on its own, its
 * derivatives first and its coefficient grids after, in Init_TypeOp order
 * ((i, j >= i), then (i, 0)), and a grid that is zero everywhere is skipped
 * (grid_zero).  Such grids stay resident.  Constant F2 / F1 act on every
 * channel alike.
 * All pointers are host pointers; the fields are built once on the device
 * (the equivalent of Save_MemGrid).
 * ---------------------------------------------------------------------- */
typedef struct {
  int type;
  const double* V_grid;
  int V_nterms;
  const double* V_coef;     /* [V_nterms] */
  const int* V_expo;        /* [V_nterms*D] */
  const double* G_grid;
  const double* G0;
  const double* G1;
  const double* Jac_grid;
  const double* sqRho_grid;
  const double* F2;
  const double* F1;
  const double* F2_grid;
  const double* F1_grid;
} evr_sg4_op_desc;

int evr_sg4_set_operator(evr_sg4_ctx* c, const evr_sg4_op_desc* op);

/* ------------------------------------------------------------------------
 * H.psi on device pointers (batched persistent kernel, the fast path):
 *   hpsi(:,r) = (H psi(:,r) - E0 psi(:,r)) / Esc,  r = 1..nrhs
 * A column holds the nb0 channel blocks of N (ld >= nb0*N).
 * E0 = 0, Esc = 1 is sub_TabOpPsi; other values are sub_scaledOpPsi
 * (sub_OpPsi.f90:2821-2864).  psi and hpsi must not overlap.
 * ---------------------------------------------------------------------- */
int evr_sg4_hpsi(evr_sg4_ctx* c, int nrhs, const double* psi, long long ldpsi, double* hpsi,
                 long long ldh, double E0, double Esc, void* stream);

/* Same result through one kernel launch per Smolyak term (the "plain"
 * per-term GPU path, kept as the baseline the one-launch path is measured
 * against; it mirrors the reference's per-term loop). */
int evr_sg4_hpsi_plain(evr_sg4_ctx* c, int nrhs, const double* psi, long long ldpsi,
                       double* hpsi, long long ldh, void* stream);

/* Complex psi, interleaved complex128 (CvecB): the real operator applied to
 * the real and imaginary parts, as sub_PrimOpPsi's SG4 branch does with
 * CplxPsi_TO_RCpsi (sub_OpPsi.f90:395-412). ld in complex elements. */
int evr_sg4_hpsi_cplx(evr_sg4_ctx* c, int nrhs, const double* psi, long long ldpsi, double* hpsi,
                      long long ldh, double E0, double Esc, void* stream);

/* General form of the three calls above plus the transposed operator:
 *   flags & EVR_APPLY_TRANSPOSE : apply H^T instead of H.  The SG4 H is not
 *       symmetric in general (grid-grid derivatives on nq > nb grids make the
 *       type-10 KEO non-Hermitian); H^T gives its symmetric part
 *       (H + H^T)/2, which is what Davidson diagonalises after
 *       sub_hermitic_H (SRC/sub_inactive/sub_ana_HS.f90:56), and the adjoint
 *       a costate propagation needs.  Same kernels, transposed 1-D matrices.
 *   flags & EVR_APPLY_COMPLEX   : interleaved complex128 psi (as _cplx).
 *   flags & EVR_APPLY_PLAIN     : one launch per term (as _plain).        */
#define EVR_APPLY_TRANSPOSE 1
#define EVR_APPLY_COMPLEX 2
#define EVR_APPLY_PLAIN 4
int evr_sg4_apply(evr_sg4_ctx* c, int flags, int nrhs, const double* psi, long long ldpsi, double* hpsi,
                  long long ldh, double E0, double Esc, void* stream);

/* Host-pointer variant: copies psi to the device, runs evr_sg4_hpsi,
 * copies the result back and synchronises (what a Fortran caller holding
 * RvecB in host memory calls). */
int evr_sg4_hpsi_host(evr_sg4_ctx* c, int nrhs, const double* psi, long long ldpsi, double* hpsi,
                      long long ldh, double E0, double Esc);

/* H.psi that allocates no device memory (no counterpart in the reference).
 * For callers that cannot call cudaMalloc -- a host program whose own
 * allocator owns the device memory, a real-time loop that must stay out of
 * the driver's allocator -- this runs the same persistent kernel as
 * evr_sg4_hpsi with its scratch (work counter, work list, per-term
 * contributions, slabs for terms larger than shared memory) carved from one
 * fixed file-scope device array of EVR_SG4_NOALLOC_SCRATCH_BYTES, which every
 * GPU that loads the library holds until the process exits.  Sizes that need
 * more scratch are rejected with EVR_ERR_ARG.  The first call on a device
 * looks up the array's device address (cudaGetSymbolAddress).  All calls
 * share the array: calls that
 * overlap on the GPU (two streams or two threads) race.  Real psi only;
 * device pointers; same result as evr_sg4_hpsi. */
#define EVR_SG4_NOALLOC_SCRATCH_BYTES (32u * 1024u * 1024u)
int evr_sg4_hpsi_noalloc(evr_sg4_ctx* c, int nrhs, const double* psi, long long ldpsi, double* hpsi,
                         long long ldh, double E0, double Esc, void* stream);

/* Device budget (bytes) for the operator fields of a context, applied by the
 * next evr_sg4_set_operator.  When fields given in analytic form (V as a
 * polynomial, G0/G1 affine) would exceed it, only their coefficients stay on
 * the device and every H.psi evaluates them per slice of consecutive Smolyak
 * terms (as much as fits the budget) just before that slice's work items run,
 * as the reference builds them term by term inside its term loop when they
 * are not kept in memory (get_OpGrid_type10_OF_ONEDP_FOR_SG4,
 * SRC/sub_Operator/sub_OpPsi_SG4.f90:2536, called at :1553).  The per-term
 * contributions and their ordered accumulation are unchanged, so results are
 * bit-identical to resident fields.  Grids passed as arrays are always
 * resident.  0 (the default): resident.  evr_sg4_hpsi/_cplx/_apply (not
 * _plain) and everything built on them accept streamed contexts; the
 * per-term path, the multi-context plans and evr_sg4_hpsi_noalloc return
 * EVR_ERR_STATE. */
int evr_sg4_set_field_budget(evr_sg4_ctx* c, long long bytes);
/* Number of field slices of the current operator (0: resident fields). */
int evr_sg4_field_slices(const evr_sg4_ctx* c, long long* nslices);

/* Plan knobs of a context, applied from its next H.psi (no reference
 * interface: the reference's tunable is the OpenMP thread count of
 * Tune_SG4threads_HPsi, SRC/sub_main/vib.f90:2013-2123):
 *   geo   : launch geometry, -1 automatic (per work plan), 0 wide (4 CTAs
 *           per SM), 1 narrow (8 per SM, D <= 6 only), 2 mid (6 per SM);
 *   rmax  : most right-hand sides one work item carries, 1..32 (0: the
 *           automatic plan's value);
 *   split : mode passes, 0 thread mapping chosen per pass, 1 one thread per
 *           fibre, 2 one thread per output element (-1: the automatic
 *           plan's value).
 * evr_sg4_set_plan(c, -1, 0, -1) restores the automatic plan.
 * Results do not depend on them: every setting runs the same arithmetic per
 * Smolyak term and right-hand side (the same bits). */
int evr_sg4_set_plan(evr_sg4_ctx* c, int geo, int rmax, int split);
int evr_sg4_get_plan(const evr_sg4_ctx* c, int* geo, int* rmax, int* split);

/* Autotuner (the counterpart of Tune_SG4threads_HPsi, SRC/sub_main/
 * vib.f90:2013-2123, which times H.psi for each OpenMP thread count and
 * keeps the fastest): times H.psi on nrhs vectors (flags: EVR_APPLY_COMPLEX
 * or 0) with the automatic plan and with every candidate (geometry x rmax in
 * {4, 8, 16, 32} x split mode; best of three, each after a 256 MB write that
 * clears L2, after one untimed call), and applies the fastest -- a candidate
 * replaces the best so far only when more than 1 % faster, and the winner is
 * then timed again against the automatic plan, alternately, five times each:
 * it is kept only if its median is more than 1 % faster.  With cache_path (a JSON file, created
 * if absent) the winner is recorded under a key of the workload's shape (D,
 * L, LB, type, channels, N, nrhs, complex, G given), and a later call with
 * the same shape applies the recorded plan without timing (from_cache = 1).
 * out may be NULL. */
typedef struct {
  int geo, rmax, split;  /* the plan applied */
  double ms;             /* its H.psi time (best of three) */
  double default_ms;     /* the automatic plan's H.psi time */
  int from_cache;        /* 1: read from cache_path, nothing timed */
} evr_tune_result;
int evr_sg4_tune_plan(evr_sg4_ctx* c, int nrhs, int flags, const char* cache_path, evr_tune_result* out);
/* Short form of evr_sg4_tune_plan without a cache: returns the winning rmax
 * and its time. */
int evr_sg4_tune(evr_sg4_ctx* c, int nrhs, int flags, int* best_rmax, double* best_ms);

/* Sizes of a context: out[0..7] as evr_sg4_desc_sizes, except out[0] = the
 * length of a vector, nb0 * N. */
int evr_sg4_ctx_sizes(const evr_sg4_ctx* c, long long* out);

/* Launch geometry of the context's current work plan (the last H.psi's RHS
 * count): geo 0 = wide (4 CTAs per SM), 1 = narrow (8 per SM; D <= 6 and at
 * least four waves of items), 2 = mid (6 per SM; D > 6 and at least four
 * waves).  ctas_per_sm may be NULL.  Replaces no reference interface (the
 * reference's OpenMP thread count, Tune_SG4threads_HPsi vib.f90:2013-2123,
 * is the nearest analogue). */
int evr_sg4_last_geometry(const evr_sg4_ctx* c, int* geo, int* ctas_per_sm);

/* ------------------------------------------------------------------------
 * Callers of the path, on the device.
 * ---------------------------------------------------------------------- */

/* Block Davidson for the lowest levels (sub_propagation_Davidson,
 * SRC/sub_propagation/sub_module_Davidson.f90:59-767: new block H.psi
 * sub_MakeHPsi_Davidson :896, projected H, sub_hermitic_H symmetrisation,
 * residuals MakeResidual_Davidson :1230, Davidson correction
 * sub_NewVec_Davidson :1306 with the H diagonal, restart at max_subspace).
 * With symmetrize = 1 the operator is (H + H^T)/2, applied exactly through
 * EVR_APPLY_TRANSPOSE, so the residual threshold is met for the symmetric
 * part the reference diagonalises.  guess: device N x nguess (or NULL: the
 * first nev packed functions); diag: device N (or NULL: plain residuals);
 * evals/resid: host nev; evecs: device N x nev or NULL.  Returns
 * EVR_ERR_NUMERIC if max_it is reached (evals/resid still filled). */
typedef struct {
  int nev;             /* number of lowest levels */
  int block;           /* directions added per iteration (0 = nev) */
  int max_subspace;    /* restart size (0 = max(3 nev, nev + 2 block)) */
  int max_it;          /* iterations */
  double conv_resi;    /* residual 2-norm threshold */
  int symmetrize;      /* 1: work on (H + H^T)/2 */
  int no_graph;        /* 0: each iteration is two recorded CUDA graphs (Ritz vectors,
                          residuals and their norms; then the expansion: correction,
                          Gram-Schmidt against the basis and within the block, H.psi,
                          projected matrix), replayed with the host's small dense
                          eigenproblem between them -- two host synchronisations per
                          iteration; 1: the same steps launched one by one */
} evr_davidson_opts;
int evr_sg4_davidson(evr_sg4_ctx* c, const evr_davidson_opts* o, const double* guess, int nguess,
                     const double* diag, double* evals, double* evecs, double* resid, int* iterations,
                     void* stream);

/* Exact diagonal of H on the device (diag: device N), the Davidson
 * preconditioner (the reference's correction uses the H diagonal,
 * sub_NewVec_Davidson, sub_module_Davidson.f90:1306).  Computed term by
 * term: each Smolyak term's diagonal is a grid->basis transform of its
 * fields with per-mode matrices (RBGwrho.D o (D.RGB)^T), one transform per
 * field term, then the weighted, term-ordered accumulation of H.psi.  Type 10
 * with Jac or rho grids, type 1 with coefficient grids, several channels and
 * streamed fields use evr_sg4_diagonal_by_apply. */
int evr_sg4_diagonal(evr_sg4_ctx* c, double* diag, void* stream);
/* The same diagonal from H applied to blocks of 64 unit vectors (N/64 H.psi
 * calls): valid for every operator, and the check of the term-wise form. */
int evr_sg4_diagonal_by_apply(evr_sg4_ctx* c, double* diag, void* stream);

/* Chebyshev propagation of complex wave packets (march_cheby,
 * SRC/sub_propagation/sub_module_propa_march.f90:4145-4437; coefficients
 * cof :5739): nsteps steps of dt, expansion order npoly on [Hmin, Hmax]
 * (E0, Esc of sub_scaledOpPsi fused into each H.psi), early exit when
 * |c_k| |w_k|^2 < poly_tol (poly_tol <= 0: always npoly terms), a step that
 * diverges (> 1e15) redone with Hmax raised by (Hmax-Hmin)/10 up to 10 times.
 * psi: device interleaved complex128 N x nrhs (ld N), propagated in place.
 * autocorr: host complex [(nsteps+1) x nrhs] = <psi0 | psi(t_k)> (psi0 NULL:
 * the initial psi), or NULL. */
typedef struct {
  double Hmin, Hmax;   /* spectral bounds of H */
  double dt;           /* time step (a.u.) */
  int npoly;           /* expansion order */
  int nsteps;          /* number of steps */
  double poly_tol;     /* convergence of the expansion, <= 0: fixed order */
  int no_graph;        /* fixed order: 0 replays each step as a CUDA graph recorded
                          once (no host work between launches); 1 launches eagerly */
} evr_cheby_opts;
int evr_sg4_cheby_propagate(evr_sg4_ctx* c, const evr_cheby_opts* o, int nrhs, double* psi, const double* psi0,
                            double* autocorr, int* npoly_used, void* stream);

/* Several independent Hamiltonians (contexts of any D, L and operator type)
 * applied in ONE persistent launch: the (context, term, rhs block) items of
 * all of them are merged into one cost-sorted work list, followed by each
 * context's ordered accumulation (1 + 2n launches).  No counterpart in the
 * reference, which applies one para_Op per sub_TabOpPsi call
 * (SRC/sub_Operator/sub_OpPsi.f90:705); this batches its independent
 * Hamiltonians (the uneven-instance workload) on one GPU.
 *
 * evr_sg4_multi_create fixes the contexts, nrhs[k] per context and the flags
 * (EVR_APPLY_COMPLEX, EVR_APPLY_TRANSPOSE); the plan owns the per-call
 * scratch, so the contexts stay usable on their own.  Calling
 * evr_sg4_set_operator with another operator type on a context invalidates
 * the plan (evr_sg4_multi_hpsi returns EVR_ERR_STATE).
 * evr_sg4_multi_hpsi: per context k, psi[k] (ld ldpsi[k], device) ->
 * hpsi[k] (ld ldh[k]), scaled by E0[k], Esc[k] (NULL arrays: 0 and 1);
 * psi[k] == NULL skips context k in this call.  A plan is used from one
 * stream at a time.
 * Launch groups: the contexts with D <= 6 run narrow in a launch of their
 * own when their items fill enough waves and other contexts exist; else one
 * launch takes every context; a group of more than 64 contexts is split into
 * launches of at most 64 (the contexts' parameters travel by value in the
 * launch).  A group's geometry is automatic unless every context in it names
 * the same one through evr_sg4_set_plan before evr_sg4_multi_create.
 * evr_sg4_multi_groups reports the launch groups: their count, and for the
 * first min(count, cap) the geometry (0 wide, 1 narrow, 2 mid) and the number
 * of work items (geo and n_items may be NULL). */
typedef struct evr_sg4_multi evr_sg4_multi;
int evr_sg4_multi_create(int n, evr_sg4_ctx* const* ctxs, const int* nrhs, int flags, evr_sg4_multi** out);
int evr_sg4_multi_hpsi(evr_sg4_multi* m, const double* const* psi, const long long* ldpsi, double* const* hpsi,
                       const long long* ldh, const double* E0, const double* Esc, void* stream);
int evr_sg4_multi_last_launches(const evr_sg4_multi* m, long long* n);
int evr_sg4_multi_groups(const evr_sg4_multi* m, int cap, int* n_groups, int* geo, long long* n_items);
int evr_sg4_multi_destroy(evr_sg4_multi* m);
/* Chebyshev propagation (evr_sg4_cheby_propagate's fixed-order form) of the
 * packets of every context of a plan created with EVR_APPLY_COMPLEX, in
 * lock-step: each expansion order is ONE evr_sg4_multi_hpsi over all
 * contexts.  o[k]: options of context k (own Hmin, Hmax; dt, npoly, nsteps
 * equal for all, poly_tol <= 0).  A context whose step diverges redoes it
 * with Hmax raised by (Hmax-Hmin)/10, up to 10 times.  psi[k]: device
 * interleaved complex128 N_k x nrhs_k, propagated in place; autocorr[k]: host
 * complex [(nsteps+1) x nrhs_k] = <psi_k(0) | psi_k(t_j)>, or NULL.  Unless
 * o[0].no_graph, a step with every context in it (each order's merged launch,
 * the ordered accumulations and recurrence updates of every context) is
 * recorded once as a CUDA graph and replayed while the bounds stay the same;
 * diverged contexts are redone eagerly (the same kernels, the same bits). */
int evr_sg4_multi_cheby_propagate(evr_sg4_multi* m, const evr_cheby_opts* o, double* const* psi,
                                  double* const* autocorr, int* npoly_used, void* stream);
/* One-shot form: create, apply, synchronize the stream, destroy. */
int evr_sg4_hpsi_multi(int n, evr_sg4_ctx* const* ctxs, const int* nrhs, const double* const* psi,
                       const long long* ldpsi, double* const* hpsi, const long long* ldh, const double* E0,
                       const double* Esc, int flags, void* stream);

/* Field-driven RK4 propagation of one complex packet (march_RK4_field,
 * SRC/sub_propagation/sub_module_propa_march.f90:397-548; fcn_field
 * :1439-1520): dpsi/dt = -i (H0 - E(t) mu) psi with E held at E[k] over
 * field interval k ('grid' field), each interval integrated with nsub RK4
 * steps.  H0 and mu are contexts on the same basis (mu a type-0 operator).
 * psi: device complex128 N, propagated in place. */
typedef struct {
  double dt;           /* time step (a.u.) */
  int nsteps;          /* number of steps = number of field samples */
  int checkpoint;      /* oc_gradient: keep psi every `checkpoint` steps */
  double E0;           /* energy shift: stages use H0 - E0, then psi *= exp(-i E0 dt)
                          (fcn_field's para_H%E0; mid-spectrum keeps RK4 stable) */
  int nsub;            /* RK4 steps per field interval (dt/nsub each, E held) */
  int no_graph;        /* 0: every field interval (nsub steps x 4 stages, each one H0/mu
                          launch, one chunk-sum launch and one stage update) is recorded
                          once as a CUDA graph and replayed, the interval index kept on
                          the device; 1: the same kernels launched one by one (same bits) */
} evr_rk4_opts;
int evr_sg4_rk4_field(evr_sg4_ctx* H0, evr_sg4_ctx* mu, const evr_rk4_opts* o, const double* E, double* psi,
                      void* stream);
/* nb packets propagated together, packet b under its own field E[k*nb + b]
 * (E: host [nsteps*nb]); psi: device complex128 N x nb (ld N), in place.
 * One H0/mu launch per stage serves all packets (the reference propagates
 * its nb_WP packets together, sub_propagation25, sub_control.f90).  Each
 * packet gets the same bits as evr_sg4_rk4_field under its own field (the
 * same per-column arithmetic and accumulation order). */
int evr_sg4_rk4_field_batch(evr_sg4_ctx* H0, evr_sg4_ctx* mu, const evr_rk4_opts* o, int nb, const double* E,
                            double* psi, void* stream);

/* Optimal-control objective J = |<target|psi(T)>|^2 after the RK4 propagation
 * above from psi0, and its exact gradient dJ/dE[k] for every field sample,
 * by the adjoint (costate) of the discrete RK4 steps; psi is checkpointed
 * every o->checkpoint steps and recomputed.  This is the derivative the
 * reference's field update uses in continuous form (build_field,
 * SRC/sub_propagation/sub_control.f90:907-1010).  psi0/target: device
 * complex128 N; E, grad: host [nsteps]; J: host scalar. */
int evr_sg4_oc_gradient(evr_sg4_ctx* H0, evr_sg4_ctx* mu, const evr_rk4_opts* o, const double* E,
                        const double* psi0, const double* target, double* J, double* grad, void* stream);

/* Algorithmic FP64 operation count of one H.psi per right-hand side for the
 * current operator (flop, counted from the term sizes, with the basis<->grid
 * passes in the mode order the kernels use, which never needs more
 * multiply-adds than the reference's order 1..D). */
int evr_sg4_flops_per_rhs(const evr_sg4_ctx* c, double* flops);

/* Number of kernel launches the last hpsi call issued. */
int evr_sg4_last_launches(const evr_sg4_ctx* c, long long* n);

/* Message of the last failure on the calling thread ("" if none). */
const char* evr_sg4_last_error(void);

/* Measured FP64 FMA throughput of the current device in TFLOP/s (a short
 * in-bounds DFMA loop; used as the roofline denominator). */
int evr_probe_fp64_peak(double* tflops);

/* The FP64 pipes of the current device, each in TFLOP/s: the DFMA loop
 * above, FP64 tensor-core MMA alone (mma.sync m8n8k4 f64, registers only),
 * and MMA with DFMA chains interleaved in the same warps (their sum, which
 * shows whether the two run on separate units or share one). */
int evr_probe_fp64_pipes(double* dfma_tflops, double* dmma_tflops, double* mixed_tflops);

#ifdef __cplusplus
}
#endif
#endif
