// sg4_items.cuh -- the persistent H.psi work-item kernels (device code shared
// by the per-geometry translation units and the host code that plans and
// launches them).
#pragma once
#include <cuda_runtime.h>

#include "evr_sg4.h"
#include "sg4_internal.h"

namespace evr {

// ------------------------------------------------------------------ device
#ifndef EVR_FUSED_MAXD
#define EVR_FUSED_MAXD 12  // type-10 items with D <= 12 use the fused grid passes
#endif
// Persistent H.psi launch geometry, chosen per work plan (geo 0, 1, 2).
// Wide (0): four 128-thread CTAs per SM (54.75 KB of shared memory and 128
// registers a thread each), fused type-10 passes up to D = 12; it beat two
// 256-thread CTAs by 0.7 % on the 6-D benchmark and lets the ~600 items of a
// small operator run in one wave.  Plans of at least EVR_BIG_WAVES waves of
// items take more resident warps, which keep the FP64 pipe busier on large
// operators, while a small operator's one wave of items finishes sooner with
// the wide kernel's longer register budget:
//   narrow (1), D <= 6: eight CTAs per SM (26.5 KB and 64 registers each,
//     the fused passes instantiated only up to D = 6): +7 % on the 6-D
//     benchmark (7 and 6 CTAs, and four 256-thread CTAs, within 3 %);
//   mid (2), D > 6: six CTAs per SM (35.75 KB, 80 registers, fused passes up
//     to D = 12): 4-7 % on the 12-D streamed operator and the uneven
//     multi-instance draw.
// Each geometry's kernels are compiled in their own translation units
// (sg4_items.cu built with EVR_GEO = 0, 1, 2 and EVR_KIND = 0, 1, 2), in
// parallel.
#ifndef EVR_CTA_THREADS
#define EVR_CTA_THREADS 128
#endif
#ifndef EVR_WIDE_CTAS
#define EVR_WIDE_CTAS 4
#endif
#define EVR_WIDE_FMAX 12
#ifndef EVR_NARROW_CTAS
#define EVR_NARROW_CTAS 8
#endif
#define EVR_NARROW_FMAX 6
#ifndef EVR_MID_CTAS
#define EVR_MID_CTAS 6
#endif
#define EVR_MID_FMAX 12
#define EVR_BIG_WAVES 4
#ifndef EVR_NARROW_INC
#define EVR_NARROW_INC 0  // the narrow kernel takes the point digits from divisions
#endif
#ifndef EVR_FASTDIV
#define EVR_FASTDIV 1     // those divisions by multiply-high with per-item magic numbers
#endif
#ifndef EVR_SPLIT_RES
#define EVR_SPLIT_RES 1   // fused type 10: x in shared memory when the other arrays do not fit
#endif

struct TermInfo {
  long long off_nb;   // into map
  long long off_nq;   // into the operator fields
  int nb, nq;
  int r;              // right-hand sides per work item for this term
  float cost;
  double w;           // WeightSG
  unsigned char l[EVR_MAXD];
};

// Modes in ascending (nq-nb)/(nb*nq), ties by index (the basis->grid order
// that minimises multiply-adds; grid->basis runs it backwards).  Integer
// comparison: key(o) <= key(i) <=> (nq_o-nb_o) nb_i nq_i <= (nq_i-nb_i) nb_o nq_o.
// The flop count uses it on the host; each work item sorts its modes the
// same way on the device (one thread, D <= 12: cheaper there than reading a
// stored order, measured).
static inline void mode_order(const int* nb, const int* nq, int D, int* ord) {
  for (int i = 0; i < D; ++i) {
    int j = i;
    const int ni = nq[i] - nb[i], di = nb[i] * nq[i];
    while (j > 0) {
      const int o = ord[j - 1];
      if ((nq[o] - nb[o]) * di <= ni * (nb[o] * nq[o])) break;
      ord[j] = o;
      --j;
    }
    ord[j] = i;
  }
}

// a work item (host plans)
struct Item {
  int term;
  int rhs0;
};

// a work item of a launch: the context's slot in the launch's parameter
// block, the Smolyak term and the first right-hand side of the block
struct MItem {
  int ctx, term, rhs0, pad;
};

// 1-D matrices of (mode, level), row-major [nout][nin] for the kernel.
enum { M_BG = 0, M_GB = 1, M_D1 = 2, M_D2 = 3 };

struct OpFields {
  int type;
  const double* V;     // [sum_nq] or NULL
  const double* G;     // [sum_nq*D*D] (GGiq per term) or NULL = identity
  const double* Jac;   // [sum_nq] or NULL
  const double* sqRho; // [sum_nq] or NULL
  double F2[EVR_MAXD * EVR_MAXD];
  double F1[EVR_MAXD];
};

// A type-1 derivative term with its coefficient (CASE 1 with Q-dependent
// coefficients): coefficient * d_i d_j x, or * d_i x when j < 0; the
// coefficient is the grid t1grid[goff + point] or, when goff < 0, c.  With
// a >= 0 it couples channel b into channel a (GridOp(:,a,b,iterm)); a < 0:
// it acts on every channel alike.
struct T1Term {
  int i, j, a, b;
  long long goff;
  double c;
};

struct KParams {
  int D, Lp1;
  int nrhs_v;                // virtual right-hand sides (2*nrhs for complex)
  int cshift;                // 1 for interleaved complex, else 0
  const TermInfo* terms;
  const int* map;
  const double* mats;
  const int* mat_off;        // [D*Lp1*8]: forward set, then transposed set
  int transpose;             // 1: apply H^T (the adjoint of the real operator)
  const int* nb_of_l;
  const int* nq_of_l;
  const double* psi;
  long long ldpsi;           // in doubles, already scaled for complex
  double* hpsi;
  long long ldh;
  double scale;              // 1/Esc
  const double* V;
  const double* G;
  const double* Jac;
  const double* sqRho;
  const double* F2;          // device [D*D]
  const double* F1;          // device [D]
  int type;
  int nbuf;                  // work arrays per item
  int smem_doubles;
  double* gscratch;
  long long scratch_per_cta; // doubles
  double* contrib;           // [sum_nb][nrhs_v] weighted term contributions
  const double* cfac;        // [sum_nq] -1/2/(Jac sqRho) or NULL (= -1/2)
  long long sum_nb;
  long long fbase;           // grid point of the first field entry (term slices)
  int nb0;                   // channels (electronic states): a vector is nb0 blocks of Nfun
  long long Nfun;            // packed basis functions per channel
  long long vstride;         // V[(a*nb0 + b)*vstride + point] for nb0 > 1
  int t1_mixed;              // type 1: some F2_ij (i < j) or F1_i is non-zero
  int n_t1;                  // type 1 with coefficient grids: its terms (else 0)
  const T1Term* t1terms;     // [n_t1]
  const double* t1grid;      // their grids, sum_nq each
  int split;                 // mode passes: 0 per-pass choice, 1 one thread per fibre, 2 per output
};

struct ItemShared {
  int nb[EVR_MAXD], nq[EVR_MAXD];
  int ord[EVR_MAXD];          // basis->grid mode order
  int pos[EVR_MAXD];          // rank of each mode in that order (inverse of ord)
  int st[EVR_MAXD];           // grid stride of each mode (product of the nq before it)
  int mo[EVR_MAXD][4];
  unsigned mg[EVR_MAXD];      // ceil(2^32 / nq[i]) (0 for nq = 1): rem / nq[i] = umulhi(rem, mg) for rem < 2^28
  unsigned long long mgt;     // ceil(2^64 / nq_t) (0 for nq_t = 1): e / nq_t = umul64hi(e, mgt)
  long long off_nb, off_nq;
  int nb_t, nq_t, r, rhs0, term;
  double w;
  double* base;               // the work arrays: base holds the first (x), base2 the rest
  double* base2;
};

__device__ __forceinline__ long long vaddr(const KParams& p, int v, int n, long long ld) {
  // element n (0-based, packed index) of virtual right-hand side v: column
  // v >> cshift is channel a of right-hand side j (RvecB((a-1)*Max_nDI + n))
  const int col = v >> p.cshift;
  const int j = col / p.nb0, a = col - j * p.nb0;
  return (long long)j * ld + (((long long)a * p.Nfun + n) << p.cshift) + (v & p.cshift);
}

// y(j,a) = sum_b V_ab x(j,b) at grid point q for nb0 > 1: the electronic
// matrix of the operator (OpGrid(iterm)%Grid(:,a,b) of the reference) couples
// the channels of one right-hand side; the item holds whole channel groups.
__device__ __forceinline__ double vmat_apply(const KParams& p, const double* xs, int e, int nqt, long long oq,
                                             int rhs0) {
  const int q = e % nqt, jj = e / nqt;
  const int a = ((rhs0 + jj) >> p.cshift) % p.nb0;
  double y = 0.0;
  for (int b = 0; b < p.nb0; ++b) {
    const int jb = jj + ((b - a) << p.cshift);
    const int ab = p.transpose ? b * p.nb0 + a : a * p.nb0 + b;
    y = fma(__ldg(p.V + (long long)ab * p.vstride + oq + q), xs[jb * nqt + q], y);
  }
  return y;
}

// Type-10 prologue with coupled channels: VX = V.x (the electronic matrix
// of each point applied to the channels of a right-hand side, VPsi(:,ib0)
// of the reference), then x rescaled in place (by sqRho forward, by the
// -1/2/(Jac sqRho) factor for H^T), each over the NQR elements of an item.
// Out of line and separate from the one-channel loop: inlined, it shifted
// the register allocation of the one-channel kernels (0.6-0.8 % on the 6-D
// benchmark).
static __device__ __noinline__ void channels_prologue(const KParams& p, long long oq, int nqt, int rhs0, double* x,
                                                      double* VX, int NQR) {
  for (int e = threadIdx.x; e < NQR; e += blockDim.x) {
    if (!p.V) {
      VX[e] = 0.0;
      continue;
    }
    const int q = e % nqt, jj = e / nqt;
    const int a = ((rhs0 + jj) >> p.cshift) % p.nb0;
    double y = 0.0;
    for (int b = 0; b < p.nb0; ++b) {
      const int jb = jj + ((b - a) << p.cshift);
      const int ab = p.transpose ? b * p.nb0 + a : a * p.nb0 + b;
      y = fma(__ldg(p.V + (long long)ab * p.vstride + oq + q), x[jb * nqt + q], y);
    }
    VX[e] = y;
  }
  __syncthreads();
  for (int e = threadIdx.x; e < NQR; e += blockDim.x) {
    const int q = e % nqt;
    if (!p.transpose) {
      if (p.sqRho) x[e] *= __ldg(p.sqRho + oq + q);
    } else {
      x[e] *= p.cfac ? __ldg(p.cfac + oq + q) : -0.5;
    }
  }
}

// out[a + S*(k + nout*b)] (+)= scale * sum_m M[k*NIN+m] in[a + S*(m + NIN*b)]
// One thread per fibre (a, b); the NIN inputs of the fibre stay in registers,
// matrix loads are warp-uniform, and four outputs are formed at once as
// independent FMA chains (GB300's FP64 pipe has a long latency, one chain per
// warp cannot keep it busy).  MODE 0 stores, 1 adds, 2 adds scale times.
template <int NIN, int MODE>
__device__ __forceinline__ void mode_pass_t(const double* __restrict__ M, int nout, int S, int R,
                                            const double* in, double* out, double scale) {
  const int nf = S * R;
  for (int f = threadIdx.x; f < nf; f += blockDim.x) {
    const int b = f / S, a = f - b * S;
    const double* fi = in + a + S * NIN * b;
    double v[NIN];
#pragma unroll
    for (int m = 0; m < NIN; ++m) v[m] = fi[S * m];
    double* fo = out + a + S * nout * b;
    int k = 0;
    for (; k + 4 <= nout; k += 4) {
      const double* M0 = M + k * NIN;
      double s0 = 0.0, s1 = 0.0, s2 = 0.0, s3 = 0.0;
#pragma unroll
      for (int m = 0; m < NIN; ++m) {
        s0 = fma(__ldg(M0 + m), v[m], s0);
        s1 = fma(__ldg(M0 + NIN + m), v[m], s1);
        s2 = fma(__ldg(M0 + 2 * NIN + m), v[m], s2);
        s3 = fma(__ldg(M0 + 3 * NIN + m), v[m], s3);
      }
      if (MODE == 0) {
        fo[S * k] = s0; fo[S * (k + 1)] = s1; fo[S * (k + 2)] = s2; fo[S * (k + 3)] = s3;
      } else if (MODE == 1) {
        fo[S * k] += s0; fo[S * (k + 1)] += s1; fo[S * (k + 2)] += s2; fo[S * (k + 3)] += s3;
      } else {
        fo[S * k] = fma(scale, s0, fo[S * k]);
        fo[S * (k + 1)] = fma(scale, s1, fo[S * (k + 1)]);
        fo[S * (k + 2)] = fma(scale, s2, fo[S * (k + 2)]);
        fo[S * (k + 3)] = fma(scale, s3, fo[S * (k + 3)]);
      }
    }
    for (; k < nout; ++k) {
      const double* Mk = M + k * NIN;
      double s0 = 0.0;
#pragma unroll
      for (int m = 0; m < NIN; ++m) s0 = fma(__ldg(Mk + m), v[m], s0);
      if (MODE == 0) fo[S * k] = s0;
      else if (MODE == 1) fo[S * k] += s0;
      else fo[S * k] = fma(scale, s0, fo[S * k]);
    }
  }
}

// Few fibres (when one thread per fibre leaves a longer critical path than
// one thread per output element): one thread per output element, so the
// threads share the pass evenly.  Each output is one FMA chain over the
// fibre's inputs in the same order as above, so the bits are the same.  The
// typical basis<->grid pass of a small term has one or two fibres per
// thread; splitting made the 6-D benchmark 4.8 % faster.
template <int NIN, int MODE>
__device__ __forceinline__ void mode_pass_split(const double* __restrict__ M, int nout, int S, int R,
                                                const double* in, double* out, double scale) {
  const int nf = S * R;
  for (int u = threadIdx.x; u < nf * nout; u += blockDim.x) {
    const int k = u / nf, f = u - k * nf;
    const int b = f / S, a = f - b * S;
    const double* fi = in + a + S * NIN * b;
    const double* Mk = M + k * NIN;
    double s0 = 0.0;
#pragma unroll
    for (int m = 0; m < NIN; ++m) s0 = fma(__ldg(Mk + m), fi[S * m], s0);
    double* fo = out + a + S * (k + nout * b);
    if (MODE == 0) *fo = s0;
    else if (MODE == 1) *fo += s0;
    else *fo = fma(scale, s0, *fo);
  }
}

// split: 0 picks per pass (one thread per output element when that gives a
// shorter critical path), 1 keeps one thread per fibre, 2 splits whenever a
// fibre has more than one output (a plan knob of the autotuner; the FMA
// chain of every output is the same either way).
template <int MODE>
__device__ __noinline__ void mode_pass_m(const double* M, int nin, int nout, int S, int R, const double* in, double* out,
                            double scale, int split) {
  const int nf = S * R, T = blockDim.x;
  if (nout > 1 && split != 1 && (split == 2 || (nf * nout + T - 1) / T < ((nf + T - 1) / T) * nout)) {
    switch (nin) {
#define EVR_CASE(n) \
  case n:           \
    mode_pass_split<n, MODE>(M, nout, S, R, in, out, scale); return;
      EVR_CASE(1) EVR_CASE(2) EVR_CASE(3) EVR_CASE(4) EVR_CASE(5) EVR_CASE(6) EVR_CASE(7) EVR_CASE(8)
      EVR_CASE(9) EVR_CASE(10) EVR_CASE(11) EVR_CASE(12) EVR_CASE(13) EVR_CASE(14) EVR_CASE(15) EVR_CASE(16)
#undef EVR_CASE
      default: return;
    }
  }
  switch (nin) {
#define EVR_CASE(n) \
  case n:           \
    mode_pass_t<n, MODE>(M, nout, S, R, in, out, scale); break;
    EVR_CASE(1) EVR_CASE(2) EVR_CASE(3) EVR_CASE(4) EVR_CASE(5) EVR_CASE(6) EVR_CASE(7) EVR_CASE(8)
    EVR_CASE(9) EVR_CASE(10) EVR_CASE(11) EVR_CASE(12) EVR_CASE(13) EVR_CASE(14) EVR_CASE(15) EVR_CASE(16)
#undef EVR_CASE
    default: break;
  }
}

static __device__ void mode_pass(const double* M, int nin, int nout, int S, int R, const double* in, double* out,
                          bool acc, double scale, int split) {
  if (!acc) mode_pass_m<0>(M, nin, nout, S, R, in, out, 1.0, split);
  else if (scale == 1.0) mode_pass_m<1>(M, nin, nout, S, R, in, out, 1.0, split);
  else mode_pass_m<2>(M, nin, nout, S, R, in, out, scale, split);
}

// Derivative pass along mode i on the grid (DerivOp_TO_RDP_OF_SmolaykRep).
static __device__ void grid_deriv(const KParams& p, const ItemShared& it, int i, int which, const double* in,
                           double* out, bool acc, double scale) {
  int S = 1, R = it.r;
  for (int j = 0; j < p.D; ++j) {
    if (j < i) S *= it.nq[j];
    else if (j > i) R *= it.nq[j];
  }
  mode_pass(p.mats + it.mo[i][which], it.nq[i], it.nq[i], S, R, in, out, acc, scale, p.split);
}

// basis->grid (to_grid, BDP_TO_GDP) or grid->basis (GDP_TO_BDP).  The
// reference applies modes 1..D; the product of 1-D maps commutes, so the
// modes are taken in the order that minimises multiply-adds: basis->grid in
// ascending (nq-nb)/(nb*nq) (the modes that grow the array most go last),
// grid->basis in the reverse order (they shrink it first).
// The extents of the other modes at step k follow from their ranks in the
// order (a mode already passed has its output size), read from the item's
// shared block rather than kept in a per-thread array.
static __device__ double* transform(const KParams& p, const ItemShared& it, bool to_grid, double* a, double* b) {
  for (int k = 0; k < p.D; ++k) {
    const int i = it.ord[to_grid ? k : p.D - 1 - k];
    const int nin = to_grid ? it.nb[i] : it.nq[i];
    const int nout = to_grid ? it.nq[i] : it.nb[i];
    int S = 1, R = it.r;
    for (int j = 0; j < p.D; ++j) {
      const bool done = to_grid ? it.pos[j] < k : it.pos[j] > p.D - 1 - k;
      const int c = (done == to_grid) ? it.nq[j] : it.nb[j];
      if (j < i) S *= c;
      else if (j > i) R *= c;
    }
    mode_pass(p.mats + it.mo[i][to_grid ? M_BG : M_GB], nin, nout, S, R, a, b, false, 1.0, p.split);
    __syncthreads();
    double* t = a;
    a = b;
    b = t;
  }
  return a;
}

// Type-10 grid operator in two fused passes over the grid points of an item
// (D <= 12):
//   pass A, per point: phi_j = (d_j x)(point) for every mode j (D independent
//     FMA chains over the mode fibres through the point), then
//     U_i = Jac sum_j G_ji phi_j, stored;
//   pass B, per point: O = c * sum_i (d_i U_i)(point) + O  (O holds V.x), or,
//     without Jac and rho, O = V.x - 1/2 sum_i (d_i U_i)(point) written over x.
// The reference applies d_j to the whole grid mode by mode
// (DerivOp_TO_RDP_OF_SmolaykRep); the same products, with two barriers
// instead of 2D+2 and no phi arrays.  For H^T the matrices are transposed
// and c (= -1/2/(Jac s)) and s trade places (done by the caller).
// Position of element e = j*nqt + q of an item (q's digits along the modes,
// mode 1 fastest, and the right-hand side j), advanced by a fixed stride with
// mixed-radix carries so the loops over the grid do no integer division.
template <int DD>
struct GridPos {
  int dig[DD], sdig[DD];
  int e, j, sj;
  __device__ __forceinline__ void init(const int* nq, int nqt, int e0, int stride) {
    e = e0;
    j = e0 / nqt;
    int q = e0 - j * nqt;
    sj = stride / nqt;
    int s = stride - sj * nqt;
#pragma unroll
    for (int i = 0; i < DD; ++i) {
      dig[i] = q % nq[i];
      q /= nq[i];
      sdig[i] = s % nq[i];
      s /= nq[i];
    }
  }
  __device__ __forceinline__ void advance(const int* nq, int stride) {
    e += stride;
    int carry = 0;
#pragma unroll
    for (int i = 0; i < DD; ++i) {
      const int d = dig[i] + sdig[i] + carry;  // <= 2 nq - 1
      carry = d >= nq[i];
      dig[i] = carry ? d - nq[i] : d;
    }
    j += sj + carry;
  }
};

// The point's digits come from GridPos (INC, fewer instructions) or from
// divisions of the element index (fewer registers: the narrow geometry's
// 64-register budget spills less without the digit arrays).
template <int DD, bool INC, class MS>
__device__ __forceinline__ void point_digits(GridPos<DD>& gp, const MS& ms, int nqt, int e, int* idx, int& q) {
  if constexpr (INC) {
    q = e - gp.j * nqt;
#pragma unroll
    for (int i = 0; i < DD; ++i) idx[i] = gp.dig[i];
  } else {
#if EVR_FASTDIV
    // exact quotients by multiply-high: nq_t < 2^27 (checked at context
    // creation), so e < 2^32 and every digit quotient has rem < 2^28
    const unsigned long long mt = ms.mgt();
    const int j = mt ? (int)__umul64hi((unsigned long long)e, mt) : e;
    q = e - j * nqt;
    unsigned rem = (unsigned)q;
#pragma unroll
    for (int i = 0; i < DD; ++i) {
      const unsigned n = (unsigned)ms.nq(i), m = ms.mg(i);
      const unsigned quo = m ? __umulhi(rem, m) : rem;
      idx[i] = (int)(rem - quo * n);
      rem = quo;
    }
#else
    q = e % nqt;
    int rem = q;
#pragma unroll
    for (int i = 0; i < DD; ++i) {
      const int n = ms.nq(i);
      idx[i] = rem % n;
      rem /= n;
    }
#endif
  }
}

// Per-mode sizes, grid strides and derivative matrices: in registers for the
// wide geometry, read from the item's shared block for the narrow one (its
// 64-register budget cannot hold 4 D values beside the point's digits and
// the D partial sums; spilled copies would live in local memory that the
// full shared-memory carve-out leaves almost no L1 for).
template <int DD, bool REG>
struct ModeSizes;
template <int DD>
struct ModeSizes<DD, true> {
  int nq_[DD], st_[DD];
  const double* Md_[DD];
  __device__ __forceinline__ ModeSizes(const KParams& p, const ItemShared& it) {
#pragma unroll
    for (int i = 0; i < DD; ++i) {
      nq_[i] = it.nq[i];
      st_[i] = it.st[i];
      Md_[i] = p.mats + it.mo[i][M_D1];
    }
  }
  __device__ __forceinline__ int nq(int i) const { return nq_[i]; }
  __device__ __forceinline__ int st(int i) const { return st_[i]; }
  __device__ __forceinline__ const double* Md(int i) const { return Md_[i]; }
};
template <int DD>
struct ModeSizes<DD, false> {
  const volatile ItemShared& it;
  const double* mats;
  __device__ __forceinline__ ModeSizes(const KParams& p, const ItemShared& s) : it(s), mats(p.mats) {}
  __device__ __forceinline__ int nq(int i) const { return it.nq[i]; }
  __device__ __forceinline__ int st(int i) const { return it.st[i]; }
  __device__ __forceinline__ unsigned mg(int i) const { return it.mg[i]; }
  __device__ __forceinline__ unsigned long long mgt() const { return it.mgt; }
  __device__ __forceinline__ const double* Md(int i) const { return mats + it.mo[i][M_D1]; }
};

template <int DD, bool INC>
__device__ void type10_fused(const KParams& p, const ItemShared& it, const double* x, double* O, double* U,
                             int NQR, bool inplace) {
  const int nqt = it.nq_t;
  const long long oq = it.off_nq;
  const ModeSizes<DD, INC> ms(p, it);
  const long long GD = (long long)DD * DD;
  const long long si = p.transpose ? nqt : (long long)nqt * DD;  // G offset step of the output index
  const long long sj = p.transpose ? (long long)nqt * DD : nqt;  // ... and of the input index
  GridPos<DD> gp;
  if constexpr (INC) gp.init(ms.nq_, nqt, threadIdx.x, blockDim.x);
  for (int e = threadIdx.x; e < NQR; e += blockDim.x) {
    int idx[DD], q;
    point_digits<DD, INC>(gp, ms, nqt, e, idx, q);
    if constexpr (INC) gp.advance(ms.nq_, blockDim.x);
    const double* xr = x + (e - q);
    double phi[DD];
#pragma unroll
    for (int j = 0; j < DD; ++j) {
      const int n = ms.nq(j), sd = ms.st(j);
      const double* fib = xr + (q - idx[j] * sd);
      const double* row = ms.Md(j) + idx[j] * n;
      double a = 0.0;
      for (int m = 0; m < n; ++m) a = fma(__ldg(row + m), fib[m * sd], a);
      phi[j] = a;
    }
    const double jac = p.Jac ? __ldg(p.Jac + oq + q) : 1.0;
    const double* g = p.G ? p.G + oq * GD + q : nullptr;
#pragma unroll
    for (int i = 0; i < DD; ++i) {
      double u;
      if (g) {
        u = 0.0;
#pragma unroll
        for (int j = 0; j < DD; ++j) u = fma(__ldg(g + si * i + sj * j), phi[j], u);
      } else {
        u = phi[i];
      }
      U[(long long)i * NQR + e] = p.Jac ? u * jac : u;
    }
  }
  __syncthreads();
  if constexpr (INC) gp.init(ms.nq_, nqt, threadIdx.x, blockDim.x);
  for (int e = threadIdx.x; e < NQR; e += blockDim.x) {
    int idx[DD], q;
    point_digits<DD, INC>(gp, ms, nqt, e, idx, q);
    if constexpr (INC) gp.advance(ms.nq_, blockDim.x);
    // one FMA chain over the fibres of every mode (no partial sums to add:
    // the FP64 pipe, not latency, bounds the kernel)
    double sum = 0.0;
#pragma unroll
    for (int i = 0; i < DD; ++i) {
      const int n = ms.nq(i), sd = ms.st(i);
      const double* fib = U + (long long)i * NQR + (e - idx[i] * sd);
      const double* row = ms.Md(i) + idx[i] * n;
      for (int m = 0; m < n; ++m) sum = fma(__ldg(row + m), fib[m * sd], sum);
    }
    if (inplace) {  // O is x: V.x + (-1/2) sum, both directions
      const double vx = p.V ? __ldg(p.V + oq + q) * O[e] : 0.0;
      O[e] = fma(-0.5, sum, vx);
    } else {
      const double cf = !p.transpose ? (p.cfac ? __ldg(p.cfac + oq + q) : -0.5)
                                     : (p.sqRho ? __ldg(p.sqRho + oq + q) : 1.0);
      O[e] = fma(cf, sum, O[e]);
    }
  }
  __syncthreads();
}

// Type-1 grid operator (CASE 1 of sub_TabOpPsi_OF_ONEDP_FOR_SGtype4,
// y = V.x + sum_{i<=j} F2_ij d_i d_j x + sum_i F1_i d_i x; the reference
// applies each term as a derivative pass of its own) in fused passes over
// the grid points of an item:
//   pass A, per point: V.x + sum_i F2_ii (d2_i x)(point), and with mixed
//     terms also + sum_i F1_i (d_i x)(point) and U_i = sum_{j>i} F2_ij
//     (d_j x)(point), stored (the derivatives along different modes commute);
//   pass B (mixed terms only): O += sum_i (d_i U_i)(point), one FMA chain.
// One or two barriers instead of one or two per term.  For H^T the matrices
// are the transposed set (chosen with the item's matrix offsets).
template <int DD, bool INC>
__device__ void type1_fused(const KParams& p, const ItemShared& it, const double* x, double* O, double* U,
                            int NQR) {
  const int nqt = it.nq_t;
  const long long oq = it.off_nq;
  const ModeSizes<DD, INC> ms(p, it);
  const bool mixed = p.t1_mixed != 0;
  GridPos<DD> gp;
  if constexpr (INC) gp.init(ms.nq_, nqt, threadIdx.x, blockDim.x);
  for (int e = threadIdx.x; e < NQR; e += blockDim.x) {
    int idx[DD], q;
    point_digits<DD, INC>(gp, ms, nqt, e, idx, q);
    if constexpr (INC) gp.advance(ms.nq_, blockDim.x);
    const double* xr = x + (e - q);
    double acc = !p.V ? 0.0 : (p.nb0 == 1 ? __ldg(p.V + oq + q) * x[e] : vmat_apply(p, x, e, nqt, oq, it.rhs0));
    double phi[DD];
#pragma unroll
    for (int i = 0; i < DD; ++i) {
      const int n = ms.nq(i), sd = ms.st(i);
      const double* fib = xr + (q - idx[i] * sd);
      const double f2 = __ldg(p.F2 + i * DD + i);
      if (f2 != 0.0) {
        const double* row2 = p.mats + it.mo[i][M_D2] + idx[i] * n;
        double d = 0.0;
        for (int m = 0; m < n; ++m) d = fma(__ldg(row2 + m), fib[m * sd], d);
        acc = fma(f2, d, acc);
      }
      phi[i] = 0.0;
      if (mixed) {
        const double* row = ms.Md(i) + idx[i] * n;
        double a = 0.0;
        for (int m = 0; m < n; ++m) a = fma(__ldg(row + m), fib[m * sd], a);
        phi[i] = a;
        const double f1 = __ldg(p.F1 + i);
        if (f1 != 0.0) acc = fma(f1, a, acc);
      }
    }
    if (mixed) {
#pragma unroll
      for (int i = 0; i + 1 < DD; ++i) {
        double u = 0.0;
#pragma unroll
        for (int j = i + 1; j < DD; ++j) u = fma(__ldg(p.F2 + i * DD + j), phi[j], u);
        U[(long long)i * NQR + e] = u;
      }
    }
    O[e] = acc;
  }
  __syncthreads();
  if (!mixed) return;
  if constexpr (INC) gp.init(ms.nq_, nqt, threadIdx.x, blockDim.x);
  for (int e = threadIdx.x; e < NQR; e += blockDim.x) {
    int idx[DD], q;
    point_digits<DD, INC>(gp, ms, nqt, e, idx, q);
    if constexpr (INC) gp.advance(ms.nq_, blockDim.x);
    double sum = O[e];
#pragma unroll
    for (int i = 0; i + 1 < DD; ++i) {
      const int n = ms.nq(i), sd = ms.st(i);
      const double* fib = U + (long long)i * NQR + (e - idx[i] * sd);
      const double* row = ms.Md(i) + idx[i] * n;
      for (int m = 0; m < n; ++m) sum = fma(__ldg(row + m), fib[m * sd], sum);
    }
    O[e] = sum;
  }
  __syncthreads();
}

template <int FMAX>
__device__ void type1_fused_dispatch(const KParams& p, const ItemShared& it, const double* x, double* O, double* U,
                                     int NQR) {
  switch (p.D) {
#define EVR_T1(n)                                                                                          \
  case n:                                                                                                  \
    if constexpr (n <= FMAX) type1_fused<n, (FMAX > EVR_NARROW_FMAX) || EVR_NARROW_INC>(p, it, x, O, U, NQR); \
    break;
    EVR_T1(1) EVR_T1(2) EVR_T1(3) EVR_T1(4) EVR_T1(5) EVR_T1(6) EVR_T1(7) EVR_T1(8) EVR_T1(9)
    EVR_T1(10) EVR_T1(11) EVR_T1(12)
#undef EVR_T1
    default: break;
  }
}

template <int FMAX>
__device__ void type10_fused_dispatch(const KParams& p, const ItemShared& it, const double* x, double* O, double* U,
                                      int NQR, bool inplace) {
  switch (p.D) {
#define EVR_T10(n)                                                        \
  case n:                                                                 \
    if constexpr (n <= FMAX)                                              \
      type10_fused<n, (FMAX > EVR_NARROW_FMAX) || EVR_NARROW_INC>(p, it, x, O, U, NQR, inplace); \
    break;
    EVR_T10(1) EVR_T10(2) EVR_T10(3) EVR_T10(4) EVR_T10(5) EVR_T10(6) EVR_T10(7) EVR_T10(8) EVR_T10(9)
    EVR_T10(10) EVR_T10(11) EVR_T10(12)
#undef EVR_T10
    default: break;
  }
}

// The weighted term result WeightSG(l) * y_b goes to contrib[off_nb + k][v]
// (no atomics); the two reduce kernels add the contributions of each packed
// function in Smolyak-term order, as tabR_AT_iG_TO_tabPackedBasis
// accumulates them (sub_module_basis_BtoG_GtoB_SG4.f90:1255-1294).
static __device__ void store_contrib(const KParams& p, const ItemShared& it, const double* yb) {
  const int nbt = it.nb_t;
  const double wt = it.w;
  const int* map = p.map + it.off_nb;
  const int r = it.r;
  for (int e = threadIdx.x; e < nbt * r; e += blockDim.x) {
    const int k = e / r, j = e - k * r;
    if (__ldg(map + k) > 0) p.contrib[(it.off_nb + k) * p.nrhs_v + it.rhs0 + j] = wt * yb[j * nbt + k];
  }
  __syncthreads();
}

// CASE 1 with Q-dependent coefficients, term by term as the reference
// (sub_OpPsi_SG4.f90:1497-1520): each term's derivatives of x
// (DerivOp_TO_RDP_OF_SmolaykRep), then times its coefficient grid, added
// into Y, on every channel alike or from channel b into channel a
// (OpPsi(:,a) += GridOp(:,a,b,iterm) * Psi_ch(:,b)); consecutive entries of
// one term reuse its derivatives.  Channel c of the item's column k is
// ((rhs0 + k) >> cshift) % nb0 (items hold whole channel groups), so channel
// b of the same right-hand side is (b - a) << cshift columns away.  For H^T
// an entry is (g d_i d_j)^T = d_i^T d_j^T g from channel a into channel b
// (the transposed matrices of the item): the coefficient first, then the
// derivatives.  Buffers: x (X or T), Y = T + NQR, C = T + 2 NQR and the
// other of X / T.  (Not inlined, the call made the mid kernel keep a
// 888-byte stack frame; inlined it adds some spill code to the kernels for
// every operator type, not to the type-10 one.)
static __device__ __forceinline__ double* type1_grid_terms(const KParams& p, const ItemShared& it, double* x, double* X,
                                                           double* T, int NQR) {
  const int nqt = it.nq_t;
  const long long oq = it.off_nq;
  double* Y = T + NQR;
  double* C = T + 2 * NQR;
  double* C2 = (x == X) ? T : X;
  auto chan = [&](int e) { return ((it.rhs0 + e / nqt) >> p.cshift) % p.nb0; };
  for (int e = threadIdx.x; e < NQR; e += blockDim.x) {
    const int q = e % nqt;
    Y[e] = !p.V ? 0.0 : (p.nb0 == 1 ? __ldg(p.V + oq + q) * x[e] : vmat_apply(p, x, e, nqt, oq, it.rhs0));
  }
  __syncthreads();
  int pi = -2, pj = -2;  // the term whose derivatives C2 holds
  for (int t = 0; t < p.n_t1; ++t) {
    const T1Term tt = p.t1terms[t];
    const double* g = tt.goff >= 0 ? p.t1grid + tt.goff + oq : nullptr;
    const int shift = (tt.a >= 0 ? tt.b - tt.a : 0) << p.cshift;  // columns from channel a to channel b
    if (!p.transpose) {
      if (tt.i != pi || tt.j != pj) {
        if (tt.j < 0) {
          grid_deriv(p, it, tt.i, M_D1, x, C2, false, 1.0);
        } else if (tt.j == tt.i) {
          grid_deriv(p, it, tt.i, M_D2, x, C2, false, 1.0);
        } else {
          grid_deriv(p, it, tt.j, M_D1, x, C, false, 1.0);
          __syncthreads();
          grid_deriv(p, it, tt.i, M_D1, C, C2, false, 1.0);
        }
        __syncthreads();
        pi = tt.i;
        pj = tt.j;
      }
      for (int e = threadIdx.x; e < NQR; e += blockDim.x)
        if (tt.a < 0 || chan(e) == tt.a) Y[e] = fma(g ? __ldg(g + e % nqt) : tt.c, C2[e + shift * nqt], Y[e]);
    } else {
      for (int e = threadIdx.x; e < NQR; e += blockDim.x)
        C[e] = (tt.a < 0 || chan(e) == tt.b) ? (g ? __ldg(g + e % nqt) : tt.c) * x[e - shift * nqt] : 0.0;
      __syncthreads();
      if (tt.j < 0) {
        grid_deriv(p, it, tt.i, M_D1, C, Y, true, 1.0);
      } else if (tt.j == tt.i) {
        grid_deriv(p, it, tt.i, M_D2, C, Y, true, 1.0);
      } else {
        grid_deriv(p, it, tt.j, M_D1, C, C2, false, 1.0);
        __syncthreads();
        grid_deriv(p, it, tt.i, M_D1, C2, Y, true, 1.0);
      }
    }
    __syncthreads();
  }
  return Y;
}

// OPK: 0 every operator type, without type-1 coefficient grids; 1 every
// type, with them; 10 only type 10 with D <= FMAX (the fused passes), for
// launches whose contexts are all such (the other branches are not compiled
// in).  The host picks the kernel for the contexts of a launch.
template <int FMAX, int OPK>
__device__ void run_item(const KParams& p, ItemShared& it, double* smem, int term, int rhs0) {
  if (threadIdx.x == 0) {
    const TermInfo& T = p.terms[term];
    it.term = term;
    it.rhs0 = rhs0;
    it.r = min(T.r, p.nrhs_v - rhs0);
    it.off_nb = T.off_nb;
    it.off_nq = T.off_nq - p.fbase;
    it.nb_t = T.nb;
    it.nq_t = T.nq;
    it.w = T.w;
    const long long nqr = (long long)T.nq * it.r;
    const long long need = (long long)p.nbuf * nqr;
    double* slab = p.gscratch + (long long)blockIdx.x * p.scratch_per_cta;
    if (need <= p.smem_doubles) {  // every work array in shared memory
      it.base = smem;
      it.base2 = smem + nqr;
    } else if (EVR_SPLIT_RES && p.type == 10 && p.nbuf == p.D + 1 && p.D <= FMAX && nqr <= p.smem_doubles) {
      // x -- the array the fused pass A reads along every mode's fibres -- in
      // shared memory, U_1..U_D in the global-scratch slab
      it.base = smem;
      it.base2 = slab;
    } else {
      it.base = slab;
      it.base2 = slab + nqr;
    }
    it.mgt = T.nq > 1 ? 0xFFFFFFFFFFFFFFFFull / (unsigned long long)T.nq + 1ull : 0ull;
  }
  if (threadIdx.x < p.D) {
    const int i = threadIdx.x;
    const int l = p.terms[term].l[i];
    const int k = i * p.Lp1 + l;
    it.nb[i] = p.nb_of_l[k];
    it.nq[i] = p.nq_of_l[k];
    it.mg[i] = it.nq[i] > 1 ? 0xFFFFFFFFu / (unsigned)it.nq[i] + 1u : 0u;
    for (int q = 0; q < 4; ++q) it.mo[i][q] = p.mat_off[k * 8 + 4 * p.transpose + q];
  }
  __syncthreads();
  if (threadIdx.x == 0) {  // the modes in mode_order, and their grid strides
    for (int i = 0; i < p.D; ++i) {
      int j = i;
      const int ni = it.nq[i] - it.nb[i], di = it.nb[i] * it.nq[i];
      while (j > 0) {
        const int o = it.ord[j - 1];
        if ((it.nq[o] - it.nb[o]) * di <= ni * (it.nb[o] * it.nq[o])) break;
        it.ord[j] = o;
        --j;
      }
      it.ord[j] = i;
    }
    int stride = 1;
    for (int k = 0; k < p.D; ++k) {
      it.pos[it.ord[k]] = k;
      it.st[k] = stride;
      stride *= it.nq[k];
    }
  }
  __syncthreads();
  const int D = p.D, r = it.r, nbt = it.nb_t, nqt = it.nq_t;
  const int NQR = nqt * r;
  double* buf = it.base;
  double* X = buf;
  double* T = it.base2;  // buf + NQR unless x alone is in shared memory (fused type 10)
  const int* map = p.map + it.off_nb;

  // gather (tabPackedBasis_TO_tabR_AT_iG) into the buffer from which the D
  // ping-pong passes of basis->grid end in X
  double* G0 = (D & 1) ? T : X;
  for (int e = threadIdx.x; e < nbt * r; e += blockDim.x) {
    const int j = e / nbt, k = e - j * nbt;
    int n = __ldg(map + k);
    G0[e] = n > 0 ? p.psi[vaddr(p, it.rhs0 + j, n - 1, p.ldpsi)] : 0.0;
  }
  __syncthreads();
  double* x = transform(p, it, true, G0, G0 == X ? T : X);
  double* y;
  const long long oq = it.off_nq;

  if (OPK != 10 && p.type == 0) {
    // CASE 0: y = V.x
    if (p.nb0 == 1) {
      for (int e = threadIdx.x; e < NQR; e += blockDim.x) {
        const int q = e % nqt;
        x[e] = (p.V ? __ldg(p.V + oq + q) : 0.0) * x[e];
      }
      y = x;
    } else {  // channel coupling: into the other transform buffer
      y = (x == X) ? T : X;
      for (int e = threadIdx.x; e < NQR; e += blockDim.x) y[e] = p.V ? vmat_apply(p, x, e, nqt, oq, it.rhs0) : 0.0;
    }
    __syncthreads();
  } else if (OPK == 1 && p.type == 1 && p.n_t1 > 0) {
    y = type1_grid_terms(p, it, x, X, T, NQR);
  } else if (OPK != 10 && p.type == 1) {
    // CASE 1 through the fused grid passes in the wide and mid kernels (x in
    // X, O in T, then U_1..U_{D-1}); the narrow kernel keeps the term-by-term
    // passes: compiled into it, the fused code shifted its register
    // allocation and cost the type-10 benchmark 1.2 %
    if constexpr (FMAX > EVR_NARROW_FMAX) {
      double* O = T;
      type1_fused_dispatch<FMAX>(p, it, x, O, T + NQR, NQR);
      y = O;
    } else {
      // CASE 1: y = V.x + sum F2_ij d_i d_j x + sum F1_i d_i x, term by term
      double* Y = T + NQR;
      double* C = T + 2 * NQR;
      for (int e = threadIdx.x; e < NQR; e += blockDim.x) {
        const int q = e % nqt;
        Y[e] = !p.V ? 0.0 : (p.nb0 == 1 ? __ldg(p.V + oq + q) * x[e] : vmat_apply(p, x, e, nqt, oq, it.rhs0));
      }
      __syncthreads();
      for (int i = 0; i < D; ++i)
        for (int j = i; j < D; ++j) {
          double f = p.F2[i * D + j];
          if (f == 0.0) continue;
          if (i == j) {
            grid_deriv(p, it, i, M_D2, x, Y, true, f);
          } else {
            grid_deriv(p, it, i, M_D1, x, C, false, 1.0);
            __syncthreads();
            grid_deriv(p, it, j, M_D1, C, Y, true, f);
          }
          __syncthreads();
        }
      for (int i = 0; i < D; ++i) {
        double f = p.F1[i];
        if (f == 0.0) continue;
        grid_deriv(p, it, i, M_D1, x, Y, true, f);
        __syncthreads();
      }
      y = Y;
    }
  } else if (OPK == 10 || D <= FMAX) {
    // CASE 10 through the fused grid passes; x is in X.  Without Jac and rho
    // (D + 1 arrays) U_1..U_D follow X and pass B writes O = V.x + c.sum over
    // x itself (each point is read and written by one thread; the -1/2 of
    // H^T is applied there too: scaling by -1/2 is exact, so the result is
    // the same bits as scaling x first).  Otherwise x is rescaled in place
    // and O = V.x starts in T, with U_1..U_D after it (D + 2 arrays); with
    // several channels V couples them (VPsi(:,ib0) of the reference, formed
    // before the rescaling, so in a pass of its own).
    const bool inplace = p.nbuf == D + 1;
    double* O = inplace ? x : T;
    double* U = T + (inplace ? 0 : 1) * NQR;
    if (!inplace) {
      if (p.nb0 > 1) {
        channels_prologue(p, oq, nqt, it.rhs0, x, O, NQR);
      } else {
        for (int e = threadIdx.x; e < NQR; e += blockDim.x) {
          const int q = e % nqt;
          const double xv = x[e];
          O[e] = p.V ? __ldg(p.V + oq + q) * xv : 0.0;
          if (!p.transpose) {
            if (p.sqRho) x[e] = xv * __ldg(p.sqRho + oq + q);
          } else {
            x[e] = xv * (p.cfac ? __ldg(p.cfac + oq + q) : -0.5);
          }
        }
      }
      __syncthreads();
    }
    type10_fused_dispatch<FMAX>(p, it, x, O, U, NQR, inplace);
    double* yb = transform(p, it, false, O, inplace ? T : x);
    store_contrib(p, it, yb);
    return;
  } else {
    // CASE 10: -1/2 sum_i d_i(Jac sum_j G_ji d_j(s x)) / (Jac s) + V x
    double* VX = T + NQR;
    double* O = T + 2 * NQR;
    double* Phi = T + 3 * NQR;
    // forward: s.x first and -1/2/(Jac s) last; H^T swaps the two scalings;
    // coupled channels' V.x before the rescaling, in a pass of its own
    if (p.nb0 > 1) {
      channels_prologue(p, oq, nqt, it.rhs0, x, VX, NQR);
    } else {
      for (int e = threadIdx.x; e < NQR; e += blockDim.x) {
        const int q = e % nqt;
        double xv = x[e];
        VX[e] = p.V ? __ldg(p.V + oq + q) * xv : 0.0;
        if (!p.transpose) {
          if (p.sqRho) x[e] = xv * __ldg(p.sqRho + oq + q);
        } else {
          x[e] = xv * (p.cfac ? __ldg(p.cfac + oq + q) : -0.5);
        }
      }
    }
    __syncthreads();
    for (int j = 0; j < D; ++j) grid_deriv(p, it, j, M_D1, x, Phi + (long long)j * NQR, false, 1.0);
    __syncthreads();
    double* U = x;  // s.x is no longer needed
    const long long GD = (long long)D * D;
    for (int i = 0; i < D; ++i) {
      for (int e = threadIdx.x; e < NQR; e += blockDim.x) {
        const int q = e % nqt;
        double u = 0.0;
        if (p.G) {
          // output i, input j: G_ji = GGiq(q, j, i) forward, G_ij for H^T
          const double* g = p.G + oq * GD + q;
          const long long si = p.transpose ? nqt : (long long)nqt * D;
          const long long sj = p.transpose ? (long long)nqt * D : nqt;
          for (int j = 0; j < D; ++j)
            u = fma(__ldg(g + si * i + sj * j), Phi[(long long)j * NQR + e], u);
        } else {
          u = Phi[(long long)i * NQR + e];
        }
        if (p.Jac) u *= __ldg(p.Jac + oq + q);
        U[e] = u;
      }
      __syncthreads();
      grid_deriv(p, it, i, M_D1, U, O, i > 0, 1.0);
      __syncthreads();
    }
    // -1/2 O / (Jac s) + V x, with -1/2/(Jac s) formed once per operator
    for (int e = threadIdx.x; e < NQR; e += blockDim.x) {
      const int q = e % nqt;
      const double cf = !p.transpose ? (p.cfac ? __ldg(p.cfac + oq + q) : -0.5)
                                     : (p.sqRho ? __ldg(p.sqRho + oq + q) : 1.0);
      O[e] = fma(cf, O[e], VX[e]);
    }
    __syncthreads();
    y = O;
    // G->B ping-pongs between O and U
    double* yb = transform(p, it, false, O, U);
    store_contrib(p, it, yb);
    return;
  }
  double* other = (y == X) ? T : X;
  if (p.type == 1) other = (x == X) ? X : T;  // x is free after the operator
  double* yb = transform(p, it, false, y, other);
  store_contrib(p, it, yb);
}

// The parameter blocks of a launch, passed by value: EVR_PB_SMALL contexts
// (a single context, the field-driven pairs) or EVR_PB_LARGE (the
// multi-context plans split their contexts into launches of at most this
// many; 17.5 KB, inside the 32 KB kernel-parameter limit).
enum { EVR_PB_SMALL = 2, EVR_PB_LARGE = 64 };
template <int CAP>
struct ParamBlock {
  KParams p[CAP];
};
// the launch's other arguments take 32 bytes of the 32,764-byte limit
static_assert(sizeof(ParamBlock<EVR_PB_LARGE>) + 32 <= 32764, "parameter block beyond the kernel-parameter limit");

// The persistent H.psi kernel: every work item of a launch, of one or several
// contexts; each item names its context's slot in the parameter block.  The
// block is a __grid_constant__ kernel parameter, so a context's fields are
// read in place from the constant bank.  Measured against the alternatives
// (same bits): a copy of the context's parameters in registers spilled to
// local memory (3 % slower on the 64-instance draw, 17 % on its small
// contexts), and a kernel taking one context's parameters as a plain kernel
// argument was 1.3 % slower on the 6-D benchmark (more spill code).
// OPK 10 compiles only the fused type-10 path (launches whose contexts are
// all type 10 with D <= FMAX): less code and fewer spills, 1.2 % faster on
// the 6-D benchmark than the kernel for every type.  OPK 0 leaves out the
// type-1 coefficient grids (with them the wide kernel spilled and an RK4
// stage took 2 % longer); OPK 1 has them.
// With a counter the CTAs pull items until the list is empty; without one
// (the per-term path) CTA b runs item item_base + b.
template <int MINB, int FMAX, int CAP, int OPK>
__global__ void __launch_bounds__(EVR_CTA_THREADS, MINB) hpsi_items_kernel(const __grid_constant__ ParamBlock<CAP> P,
                                                              const MItem* __restrict__ items, int n_items,
                                                              int item_base, unsigned int* counter) {
  extern __shared__ double smem[];
  __shared__ ItemShared it;
  __shared__ int next;
  for (int round = 0;; ++round) {
    if (threadIdx.x == 0) next = counter ? (int)atomicAdd(counter, 1u) : (round == 0 ? item_base + (int)blockIdx.x : n_items);
    __syncthreads();
    const int idx = next;
    __syncthreads();
    if (idx >= n_items) break;
    const MItem m = items[idx];
    run_item<FMAX, OPK>(P.p[m.ctx], it, smem, m.term, m.rhs0);
  }
}

// One kernel of one launch geometry, each compiled in its own translation
// unit (sg4_items.cu with EVR_GEO = 0 wide, 1 narrow, 2 mid and EVR_KIND = 0
// the small parameter block without type-1 coefficient grids, 1 the large
// block, 2 the small block for type 10 only, 3 the small block with
// coefficient grids); the host code in sg4_device.cu assembles them per
// geometry.
template <int CAP>
struct MultiEntry {
  void (*launch)(unsigned grid, size_t smem, cudaStream_t s, const ParamBlock<CAP>& P, const MItem* items,
                 int n_items, int item_base, unsigned int* counter);
  cudaError_t (*static_smem)(size_t* bytes);  // static shared bytes
  cudaError_t (*set_smem)(int bytes);         // the dynamic shared-memory limit
};
extern const MultiEntry<EVR_PB_SMALL> multi_small_wide, multi_small_narrow, multi_small_mid;
extern const MultiEntry<EVR_PB_SMALL> multi_small10_wide, multi_small10_narrow, multi_small10_mid;
extern const MultiEntry<EVR_PB_SMALL> multi_small1g_wide, multi_small1g_narrow, multi_small1g_mid;
extern const MultiEntry<EVR_PB_LARGE> multi_large_wide, multi_large_narrow, multi_large_mid;

}  // namespace evr
