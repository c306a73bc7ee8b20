// sg4_device.cu -- GB300 (sm_103a) SG4 H.psi: context, operator fields and
// the FP64 kernels behind include/evr_sg4.h.
//
// The reference computes, for every Smolyak term l (sub_TabOpPsi_FOR_SGtype4,
// SRC/sub_Operator/sub_OpPsi_SG4.f90:681-977):
//   gather (tabPackedBasis_TO_tabR_AT_iG) -> sum-factorised basis->grid
//   (BDP_TO_GDP_OF_SmolyakRep) -> operator on the grid (CASE 0/1/10 of
//   sub_TabOpPsi_OF_ONEDP_FOR_SGtype4) -> grid->basis (GDP_TO_BDP) ->
//   weighted atomic scatter (tabR_AT_iG_TO_tabPackedBasis).
// Here one persistent kernel runs every (term, block of right-hand sides)
// work item of one H.psi, of one context or of several: CTAs pull items from
// a cost-sorted list through a global atomic counter, keep the term in
// shared memory (x in shared memory and the rest in a per-CTA slab of global
// scratch when a term does not fit), apply the 1-D matrices mode by mode
// (fused grid passes for the operators), and write each term's weighted
// result to a contribution buffer that two small kernels then sum per packed
// function in Smolyak-term order (compensated, deterministic, no atomics).
// The contexts' parameters travel by value in the launch (a __grid_constant__
// block).  GB300's FP64 pipe (~1.25 TFLOP/s measured) is the binding
// resource, so the kernel is organised to keep it busy: several CTAs per SM
// (four, six, or eight for D <= 6) so some compute while the others gather or
// synchronise, right-hand sides grouped per item so the 1-D matrices and the
// operator fields are loaded once per point for the group, and no FP64 work
// spent on anything but the algorithm's own multiply-adds.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <numeric>
#include <string>
#include <vector>

#include "evr_sg4.h"
#include "sg4_internal.h"
#include "sg4_reduce.cuh"

namespace evr {

static thread_local std::string g_err;

int set_error(int code, const char* fmt, ...) {
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_err = buf;
  return code;
}

#define CUDA_TRY(call)                                                                          \
  do {                                                                                          \
    cudaError_t e_ = (call);                                                                    \
    if (e_ != cudaSuccess)                                                                      \
      return set_error(EVR_ERR_CUDA, "%s:%d %s: %s", __FILE__, __LINE__, #call, cudaGetErrorString(e_)); \
  } while (0)

int desc_sizes(const evr_sg4_desc* d, DescSizes* z) {
  if (!d) return set_error(EVR_ERR_ARG, "descriptor is NULL");
  if (d->D < 1 || d->D > EVR_MAXD) return set_error(EVR_ERR_ARG, "D=%d outside [1,%d]", d->D, EVR_MAXD);
  if (d->L < 0) return set_error(EVR_ERR_ARG, "L < 0");
  if (d->nb0 < 1 || d->nb0 > EVR_MAXNB0) return set_error(EVR_ERR_ARG, "nb0=%d outside [1,%d]", d->nb0, EVR_MAXNB0);
  if (d->nb_SG < 1 || d->N < 1) return set_error(EVR_ERR_ARG, "empty basis (nb_SG=%lld, N=%lld)", d->nb_SG, d->N);
  if (!d->nb_of_l || !d->nq_of_l || !d->tab_l || !d->weight || !d->map)
    return set_error(EVR_ERR_ARG, "descriptor has NULL tables");
  for (int k = 0; k < d->D * (d->L + 1); ++k) {
    int nb = d->nb_of_l[k], nq = d->nq_of_l[k];
    if (nb < 1 || nq < 1 || nb > EVR_MAXN || nq > EVR_MAXN)
      return set_error(EVR_ERR_ARG, "nb/nq of (mode,level) %d = %d/%d outside [1,%d]", k, nb, nq, EVR_MAXN);
    if (nb > nq)  // sub_read_data.f90:804: the basis may not outgrow its grid
      return set_error(EVR_ERR_ARG, "nb=%d > nq=%d at (mode,level) %d", nb, nq, k);
  }
  z->sum_nb = z->sum_nq = z->max_nb = z->max_nq = 0;
  for (long long t = 0; t < d->nb_SG; ++t) {
    long long nb = 1, nq = 1;
    for (int i = 0; i < d->D; ++i) {
      int l = d->tab_l[t * d->D + i];
      if (l < 0 || l > d->L) return set_error(EVR_ERR_ARG, "term %lld has level %d outside [0,L]", t, l);
      nb *= d->nb_of_l[i * (d->L + 1) + l];
      nq *= d->nq_of_l[i * (d->L + 1) + l];
    }
    if (nq >= (1LL << 27))  // the kernels' exact multiply-high divisions assume nq_t < 2^27
      return set_error(EVR_ERR_ARG, "term %lld has %lld grid points (at most 2^27 - 1 per term)", t, nq);
    z->sum_nb += nb;
    z->sum_nq += nq;
    z->max_nb = std::max(z->max_nb, nb);
    z->max_nq = std::max(z->max_nq, nq);
  }
  return EVR_OK;
}

}  // namespace evr

#include "sg4_items.cuh"

// The automatic launch plan's knobs (evr_sg4_set_plan): the most right-hand
// sides per work item, and the mode-pass thread mapping (0 chosen per pass,
// 1 one thread per fibre, 2 one thread per output element).  Four columns per
// item and one thread per output element were the autotuner's choice for the
// 6-D benchmark and for 55 of the 64 uneven instances; as the automatic plan
// they measured faster than (32, per-pass choice) on every timed path: the
// benchmark 1.8 %, the RK4 stage 4.2 %, the OC gradient 3.8 %, Chebyshev 3 %,
// the 64-instance draw 1.6 %, the per-term path 2-5 %, Davidson 0.5 %, the
// streamed 12-D operator 0.2 % (same bits).
#ifndef EVR_AUTO_RMAX
#define EVR_AUTO_RMAX 4
#endif
#ifndef EVR_AUTO_SPLIT
#define EVR_AUTO_SPLIT 2
#endif

namespace evr {

// The kernels of launch geometry geo (0 wide, 1 narrow, 2 mid).
struct GeoKernels {
  int ctas;  // resident CTAs per SM
  int fmax;  // largest D of its fused passes
  const MultiEntry<EVR_PB_SMALL>* small;
  const MultiEntry<EVR_PB_LARGE>* large;
  const MultiEntry<EVR_PB_SMALL>* small10;  // type 10 with D <= fmax only
  const MultiEntry<EVR_PB_SMALL>* small1g;  // with type-1 coefficient grids
};
static const GeoKernels& geo_kernels(int geo) {
  static const GeoKernels t[3] = {
      {EVR_WIDE_CTAS, EVR_WIDE_FMAX, &multi_small_wide, &multi_large_wide, &multi_small10_wide, &multi_small1g_wide},
      {EVR_NARROW_CTAS, EVR_NARROW_FMAX, &multi_small_narrow, &multi_large_narrow, &multi_small10_narrow,
       &multi_small1g_narrow},
      {EVR_MID_CTAS, EVR_MID_FMAX, &multi_small_mid, &multi_large_mid, &multi_small10_mid, &multi_small1g_mid}};
  return t[geo == 1 ? 1 : (geo == 2 ? 2 : 0)];
}

// A launch over n_ctx <= EVR_PB_LARGE contexts whose parameters are
// ps[0..n_ctx) (host memory; items name their slot).  The launch copies the
// block, so ps may change as soon as this returns, and a CUDA graph that
// records the launch keeps the values of the recording.
static void launch_multi(int geo, unsigned grid, size_t smem, cudaStream_t s, const KParams* ps, int n_ctx,
                         const MItem* items, int n_items, int item_base, unsigned int* counter) {
  const GeoKernels& k = geo_kernels(geo);
  if (n_ctx <= EVR_PB_SMALL) {
    ParamBlock<EVR_PB_SMALL> P;
    std::copy(ps, ps + n_ctx, P.p);
    bool t10 = true, grids = false;  // the kernel compiled for the contexts' operators
    for (int j = 0; j < n_ctx; ++j) {
      t10 = t10 && ps[j].type == 10 && ps[j].D <= k.fmax;
      grids = grids || (ps[j].type == 1 && ps[j].n_t1 > 0);
    }
    (t10 ? k.small10 : (grids ? k.small1g : k.small))->launch(grid, smem, s, P, items, n_items, item_base, counter);
  } else {
    static thread_local ParamBlock<EVR_PB_LARGE> P;  // 17.5 KB: not on the stack
    std::copy(ps, ps + n_ctx, P.p);
    k.large->launch(grid, smem, s, P, items, n_items, item_base, counter);
  }
}

// One context's persistent launch: the CTAs pull items[0..n_items) through
// the counter (zeroed by the caller).
static void launch_single(int geo, unsigned grid, size_t smem, cudaStream_t s, const KParams& p, const MItem* items,
                          int n_items, unsigned int* counter) {
  launch_multi(geo, grid, smem, s, &p, 1, items, n_items, 0, counter);
}

static int geo_ctas(int geo) { return geo_kernels(geo).ctas; }

// Static shared memory plus the 1 KB the driver reserves per CTA, rounded up
// to 256 bytes (queried once): the largest of a geometry's kernels, so all
// of them keep the geometry's CTAs per SM.
static int smem_slack(int geo) {
  static const std::vector<int> slack = [] {
    std::vector<int> v(3, 4096);
    for (int g = 0; g < 3; ++g) {
      size_t a = 0, b = 0, c = 0, d = 0;
      const GeoKernels& k = geo_kernels(g);
      if (k.small->static_smem(&a) != cudaSuccess || k.large->static_smem(&b) != cudaSuccess ||
          k.small10->static_smem(&c) != cudaSuccess || k.small1g->static_smem(&d) != cudaSuccess) {
        cudaGetLastError();
        continue;
      }
      v[g] = (int)((std::max(std::max(a, b), std::max(c, d)) + 1024 + 255) / 256 * 256);
    }
    return v;
  }();
  return slack[geo];
}

// dynamic shared memory per CTA: the SM's 228 KB split between the resident
// CTAs, less the slack above, so all of them fit (54.75 KB wide, 26.5 KB
// narrow, 35.75 KB mid)
static int geo_smem_bytes(int geo) { return (228 * 1024 / geo_ctas(geo) - smem_slack(geo)) / 256 * 256; }

// dynamic shared memory of every geometry's kernels (set at context creation)
static cudaError_t set_smem_attributes() {
  cudaError_t e = cudaSuccess;
  for (int g = 0; g < 3 && e == cudaSuccess; ++g) {
    const GeoKernels& k = geo_kernels(g);
    const int bytes = geo_smem_bytes(g);
    e = k.small->set_smem(bytes);
    if (e == cudaSuccess) e = k.large->set_smem(bytes);
    if (e == cudaSuccess) e = k.small10->set_smem(bytes);
    if (e == cudaSuccess) e = k.small1g->set_smem(bytes);
  }
  return e;
}

__device__ __forceinline__ void neumaier_add(double& s, double& c, double x) {
  const double t = s + x;
  c += (fabs(s) >= fabs(x)) ? ((s - t) + x) : ((x - t) + s);
  s = t;
}

// Neumaier sum of contrib[inv_idx[q] * nrhs_v + v] over q in [q0, q1), in
// order, with the indices and values loaded eight at a time ahead of the
// additions (each value sits behind an index load: a short list is
// latency-bound); the additions are those of the plain loop, in its order.
__device__ __forceinline__ void chunk_sum(const double* __restrict__ contrib, const long long* __restrict__ inv_idx,
                                          long long q0, long long q1, int nrhs_v, int v, double& s, double& c) {
  long long q = q0;
  for (; q + 8 <= q1; q += 8) {
    long long id[8];
    double x[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) id[k] = inv_idx[q + k];
#pragma unroll
    for (int k = 0; k < 8; ++k) x[k] = contrib[id[k] * nrhs_v + v];
#pragma unroll
    for (int k = 0; k < 8; ++k) neumaier_add(s, c, x[k]);
  }
  for (; q < q1; ++q) neumaier_add(s, c, contrib[inv_idx[q] * nrhs_v + v]);
}

__device__ __forceinline__ void out_value(double* hpsi, const double* psi, long long n, int v, int cshift,
                                          long long ldpsi, long long ldh, double sum, double E0, double Esc,
                                          int nb0, long long Nfun) {
  const int col = v >> cshift;
  const int j = col / nb0, a = col - j * nb0;
  const long long in = ((long long)a * Nfun + n) << cshift | (v & cshift);
  const long long oh = (long long)j * ldh + in;
  if (E0 == 0.0 && Esc == 1.0) {
    hpsi[oh] = sum;
  } else {
    hpsi[oh] = (sum - E0 * psi[(long long)j * ldpsi + in]) / Esc;
  }
}

// hpsi(n, v) = (sum_t contrib(k_t(n), v) - E0 psi(n, v)) / Esc, the sum over
// the terms holding packed function n (inv_ptr/inv_idx is the inverse of
// tab_iB_OF_SRep_TO_iB, in Smolyak-term order), in two phases so no thread
// runs a long serial chain (the ground state is held by every term).  Each
// packed function's list is cut into at most EVR_RED_CHUNKS chunks of at
// least 16 entries:
//   phase 1: one thread per (chunk, right-hand side) adds its chunk in term
//            order with Neumaier compensation -> (s, c) partials;
//   phase 2: one thread per (function, right-hand side) joins its chunk
//            partials in order with TwoSum and writes (sum - E0 psi)/Esc.
// The chunking is fixed at set-up, so results are deterministic, and the
// compensated sums keep them independent of the sign pattern of the Smolyak
// weights.
#define EVR_RED_CHUNKS 32
__global__ void __launch_bounds__(256) hpsi_reduce_chunks_kernel(
    const double* __restrict__ contrib, const long long* __restrict__ chunk_q, long long n_chunks,
    const long long* __restrict__ inv_idx, int nrhs_v, double2* __restrict__ part) {
  const long long total = n_chunks * nrhs_v;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
       t += (long long)gridDim.x * blockDim.x) {
    const long long ch = t / nrhs_v;
    const int v = (int)(t - ch * nrhs_v);
    double s = 0.0, c = 0.0;
    chunk_sum(contrib, inv_idx, chunk_q[ch], chunk_q[ch + 1], nrhs_v, v, s, c);
    part[t] = make_double2(s, c);
  }
}

__global__ void __launch_bounds__(256) hpsi_reduce_join_kernel(
    const double2* __restrict__ part, const long long* __restrict__ fun_chunk, long long N, int nrhs_v, int cshift,
    const double* psi, long long ldpsi, double* hpsi, long long ldh, double E0, double Esc, int nb0) {
  const long long total = N * nrhs_v;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
       t += (long long)gridDim.x * blockDim.x) {
    const long long n = t / nrhs_v;
    const int v = (int)(t - n * nrhs_v);
    out_value(hpsi, psi, n, v, cshift, ldpsi, ldh, join_chunks(part, fun_chunk[n], fun_chunk[n + 1], nrhs_v, v), E0,
              Esc, nb0, N);
  }
}

// Operator fields on the term grids: V from a polynomial, G from the affine
// form (get_OpGrid_type10_OF_ONEDP_FOR_SG4 evaluates them point by point).
__device__ void point_coords(const int* nq_of_l, const double* xcat, const int* x_off, int D, int Lp1,
                             const TermInfo& T, long long q, double* Q) {
  for (int i = 0; i < D; ++i) {
    int k = i * Lp1 + T.l[i];
    int nqi = nq_of_l[k];
    long long iq = q % nqi;
    q /= nqi;
    Q[i] = xcat[x_off[k] + iq];
  }
}

// V polynomial terms as up to EVR_VFAC (mode << 8 | exponent) factors in
// ascending mode order (-1 ends a term): the same products, in the same
// order, as the dense exponent table, without its D loop per term.
#define EVR_VFAC 8

// Fields of the grid points [gp0, gp1) (whole terms), written from index 0.
__global__ void fields_kernel(const TermInfo* terms, long long nb_SG, const long long* pt_term_start,
                              const int* nq_of_l, const double* xcat, const int* x_off, int D, int Lp1,
                              int V_nterms, const double* V_coef, const int* V_fac, double* V,
                              const double* G0, const double* G1, double* G, long long gp0, long long gp1, int nb0,
                              long long vstride, int Gsym) {
  for (long long gp = gp0 + blockIdx.x * (long long)blockDim.x + threadIdx.x; gp < gp1;
       gp += (long long)gridDim.x * blockDim.x) {
    // binary search of the term owning global point gp
    long long lo = 0, hi = nb_SG - 1;
    while (lo < hi) {
      long long mid = (lo + hi + 1) / 2;
      if (pt_term_start[mid] <= gp) lo = mid; else hi = mid - 1;
    }
    const TermInfo& T = terms[lo];
    long long q = gp - T.off_nq;
    double Q[EVR_MAXD];
    point_coords(nq_of_l, xcat, x_off, D, Lp1, T, q, Q);
    if (V) {
      // with nb0 > 1 channels, element (a, b) of the electronic matrix has its
      // own coefficients over the same monomials (get_d0MatOp_AT_Qact gives
      // the nb0 x nb0 matrix at each point)
      for (int ab = 0; ab < nb0 * nb0; ++ab) {
        const double* cf = V_coef + (long long)ab * V_nterms;
        double v = 0.0;
        for (int t = 0; t < V_nterms; ++t) {
          double m = cf[t];
          for (int f = 0; f < EVR_VFAC; ++f) {
            const int code = V_fac[t * EVR_VFAC + f];
            if (code < 0) break;
            const double x = Q[code >> 8];
            for (int k = 0; k < (code & 255); ++k) m *= x;
          }
          v += m;
        }
        V[(long long)ab * vstride + gp - gp0] = v;
      }
    }
    if (G) {
      // a symmetric affine form (G0 and G1 symmetric in i, j, bit for bit)
      // gives G_ji the same FMA chain as G_ij: formed once, stored twice
      const long long nqt = T.nq;
      double* Gt = G + (T.off_nq - gp0) * D * D + q;
      for (int i = 0; i < D; ++i)
        for (int j = Gsym ? i : 0; j < D; ++j) {
          double g = G0 ? G0[i * D + j] : (i == j ? 1.0 : 0.0);
          if (G1)
            for (int k = 0; k < D; ++k) g = fma(G1[((long long)i * D + j) * D + k], Q[k], g);
          // GGiq(iq, j, i) of the term
          Gt[nqt * ((long long)D * i + j)] = g;
          if (Gsym) Gt[nqt * ((long long)D * j + i)] = g;
        }
    }
  }
}

// In-bounds DFMA loop used to measure the FP64 peak.
__global__ void dfma_peak_kernel(double* out, int iters, double a, double b) {
  double x0 = threadIdx.x, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6,
         x7 = x0 + 7;
  for (int i = 0; i < iters; ++i) {
    x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
    x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}

// FP64 tensor-core probe: mma.sync m8n8k4 f64 (DMMA; 512 flops per warp
// instruction) on four independent accumulator tiles per warp, in registers
// only.  With `dfma` > 0 each step also runs that many DFMA chains per thread
// beside the MMAs (the mixed probe: do DMMA and DFMA add up, or share a pipe).
__device__ __forceinline__ void dmma_m8n8k4(double& d0, double& d1, double a, double b) {
  asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1}, {%2}, {%3}, {%0,%1};\n"
               : "+d"(d0), "+d"(d1)
               : "d"(a), "d"(b));
}

__global__ void dmma_peak_kernel(double* out, int iters, int dfma, double a, double b) {
  double c[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) c[k] = threadIdx.x + k;
  double x0 = threadIdx.x, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3;
  const double av = a * (1 + (threadIdx.x & 3)), bv = b * (1 + (threadIdx.x >> 3));
  for (int i = 0; i < iters; ++i) {
    dmma_m8n8k4(c[0], c[1], av, bv);
    dmma_m8n8k4(c[2], c[3], av, bv);
    dmma_m8n8k4(c[4], c[5], av, bv);
    dmma_m8n8k4(c[6], c[7], av, bv);
    if (dfma) {
      x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
    }
  }
  double t = x0 + x1 + x2 + x3;
#pragma unroll
  for (int k = 0; k < 8; ++k) t += c[k];
  out[blockIdx.x * blockDim.x + threadIdx.x] = t;
}

}  // namespace evr

using namespace evr;

// ----------------------------------------------------------------- context
struct evr_sg4_ctx {
  int D = 0, L = 0, LB = 0;
  long long N = 0, nb_SG = 0;   // N: packed basis functions per channel
  int nb0 = 1;                  // channels (electronic states)
  long long nvec = 0;           // length of a vector: nb0 * N
  DescSizes z;
  int device = 0, num_sms = 0;
  std::vector<int> nb_of_l, nq_of_l, mat_off, x_off;
  std::vector<int> diag_off;            // [D*(L+1)*5] offsets of the diagonal pattern matrices
  int* d_diag_off = nullptr;
  std::vector<TermInfo> terms;  // host copy (r filled per nrhs)
  // device
  int* d_map = nullptr;
  double* d_mats = nullptr;
  int* d_mat_off = nullptr;
  int* d_nb_of_l = nullptr;
  int* d_nq_of_l = nullptr;
  double* d_x = nullptr;
  int* d_x_off = nullptr;
  TermInfo* d_terms = nullptr;
  MItem* d_items = nullptr;          // the plan's items, decreasing cost (slot 0)
  MItem* d_plain_items = nullptr;    // term-ordered (context 0) items for the per-term path
  size_t items_cap = 0;
  int items_nrhs = -1;               // items built for this virtual nrhs
  int n_items = 0;
  std::vector<int> term_item_start;  // plain path
  unsigned int* d_counter = nullptr;
  long long* d_inv_ptr = nullptr;    // [N+1] packed function -> contributions
  long long* d_inv_idx = nullptr;    // [count(map>0)] global DP indices, term order
  long long* d_chunk_q = nullptr;    // [n_chunks+1] list positions where chunks start
  long long* d_fun_chunk = nullptr;  // [N+1] first chunk of every packed function
  long long n_chunks = 0;
  double* d_part = nullptr;          // [n_chunks][nrhs_v] chunk partials (s, c)
  size_t part_cap = 0;
  double* d_contrib = nullptr;       // [sum_nb][nrhs_v]
  size_t contrib_cap = 0;
  double* d_scratch = nullptr;
  long long scratch_per_cta = 0;     // doubles per CTA slab of the current plan
  size_t scratch_cap = 0;            // doubles allocated
  int grid = 0;
  int smem_doubles = 0;
  int geo = 0;                       // launch geometry (1: narrow, D <= EVR_NARROW_FMAX)
  int rmax = EVR_AUTO_RMAX;          // most right-hand sides per work item (plan knob)
  int geo_override = -1;             // launch geometry (plan knob; -1 automatic)
  int split = EVR_AUTO_SPLIT;        // mode-pass thread mapping (plan knob)
  // operator
  bool have_op = false;
  int type = -1;
  double* d_V = nullptr;
  double* d_G = nullptr;
  double* d_Jac = nullptr;
  double* d_sqRho = nullptr;
  double* d_cfac = nullptr;
  double* d_F2 = nullptr;
  double* d_F1 = nullptr;
  double F2[EVR_MAXD * EVR_MAXD] = {0};
  double F1[EVR_MAXD] = {0};
  int n_t1 = 0;                       // type-1 terms with coefficient grids (0: constant F2 / F1)
  std::vector<T1Term> t1_terms;       // host copy
  T1Term* d_t1terms = nullptr;
  double* d_t1grid = nullptr;
  // streamed operator fields: analytic V / G kept as coefficients and
  // evaluated per slice of Smolyak terms just before the slice's items run
  long long field_budget = 0;         // bytes; 0: fields stay resident
  bool streamed = false;
  int V_nterms = 0;
  double* d_Vcoef = nullptr;
  int* d_Vfac = nullptr;
  double* d_G0 = nullptr;
  double* d_G1 = nullptr;
  int G_sym = 0;                      // the affine G is symmetric bit for bit (G_ji formed once)
  long long* d_pt_start = nullptr;    // [nb_SG] first grid point of every term
  std::vector<long long> slice_term;  // [nslices+1] term ranges
  std::vector<int> slice_item;        // [nslices+1] ranges of the sorted work list
  // host-pointer path buffers
  double* d_io = nullptr;
  size_t io_cap = 0;
  long long last_launches = 0;
};

// Work arrays per item and grid point.  The fused type-10 passes need x and
// U_1..U_D, plus a separate V.x array when x is rescaled in place (Jac or rho
// given) or when V couples channels (a point's value needs the other
// channels' x): otherwise pass B writes O over x (D + 1 arrays, so more
// items keep their arrays in shared memory).
// Type 1 with an off-diagonal F2 or an F1 term (the fused passes then stage
// U_1..U_{D-1}).
static bool t1_mixed(const evr_sg4_ctx* c) {
  const int D = c->D;
  for (int i = 0; i < D; ++i) {
    if (c->F1[i] != 0.0) return true;
    for (int j = i + 1; j < D; ++j)
      if (c->F2[i * D + j] != 0.0) return true;
  }
  return false;
}

static int nbuf_for(const evr_sg4_ctx* c) {
  const int D = c->D;
  if (c->type == 0) return 2;
  // type 1: the fused passes of the wide and mid kernels take x, O and, with
  // mixed terms, U_1..U_{D-1}; the narrow kernel's term-by-term passes X, T,
  // Y, C (a plan's geometry is chosen after its split, so room for both)
  if (c->type == 1) return std::max(4, 2 + (t1_mixed(c) ? D - 1 : 0));
  if (D > EVR_FUSED_MAXD) return D + 4;
  return (c->d_Jac || c->d_sqRho || c->nb0 > 1) ? D + 2 : D + 1;
}

static void free_ctx(evr_sg4_ctx* c) {
  void* ptrs[] = {c->d_map, c->d_mats, c->d_mat_off, c->d_diag_off, c->d_nb_of_l, c->d_nq_of_l, c->d_x, c->d_x_off,
                  c->d_terms, c->d_items, c->d_plain_items, c->d_counter, c->d_inv_ptr,
                  c->d_inv_idx, c->d_contrib, c->d_chunk_q, c->d_fun_chunk, c->d_part,
                  c->d_scratch, c->d_V, c->d_G, c->d_Jac, c->d_cfac,
                  c->d_sqRho, c->d_F2, c->d_F1, c->d_io, c->d_Vcoef, c->d_Vfac, c->d_G0, c->d_G1,
                  c->d_pt_start, c->d_t1terms, c->d_t1grid};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  delete c;
}

template <class T>
static int upload(T** dst, const T* src, size_t n) {
  if (n == 0) n = 1;
  CUDA_TRY(cudaMalloc((void**)dst, n * sizeof(T)));
  if (src) CUDA_TRY(cudaMemcpy(*dst, src, n * sizeof(T), cudaMemcpyHostToDevice));
  return EVR_OK;
}

extern "C" const char* evr_sg4_last_error(void) { return g_err.c_str(); }

extern "C" int evr_sg4_create(const evr_sg4_desc* d, evr_sg4_ctx** out) {
  if (!out) return set_error(EVR_ERR_ARG, "evr_sg4_create: out is NULL");
  *out = nullptr;
  DescSizes z;
  int rc = desc_sizes(d, &z);
  if (rc) return rc;
  if (!d->RGB || !d->RBGwrho || !d->d1GG || !d->d2GG || !d->x)
    return set_error(EVR_ERR_ARG, "evr_sg4_create: descriptor has NULL matrices");
  if (d->N > 2147483647LL) return set_error(EVR_ERR_ARG, "evr_sg4_create: N exceeds int32");
  for (long long k = 0; k < z.sum_nb; ++k)
    if (d->map[k] < 0 || d->map[k] > d->N)
      return set_error(EVR_ERR_ARG, "evr_sg4_create: map[%lld]=%d outside [0,N]", k, d->map[k]);
  evr_sg4_ctx* c = new evr_sg4_ctx();
  c->D = d->D;
  c->L = d->L;
  c->LB = d->LB;
  c->N = d->N;
  c->nb0 = d->nb0;
  c->nvec = (long long)d->nb0 * d->N;
  c->nb_SG = d->nb_SG;
  c->z = z;
  const int D = d->D, Lp1 = d->L + 1;
  cudaError_t e = cudaGetDevice(&c->device);
  if (e != cudaSuccess) {
    free_ctx(c);
    return set_error(EVR_ERR_CUDA, "evr_sg4_create: no CUDA device (%s)", cudaGetErrorString(e));
  }
  cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, c->device);
  c->nb_of_l.assign(d->nb_of_l, d->nb_of_l + D * Lp1);
  c->nq_of_l.assign(d->nq_of_l, d->nq_of_l + D * Lp1);
  // matrices, re-laid out row-major [nout][nin]
  std::vector<double> mats;
  c->mat_off.resize((size_t)D * Lp1 * 8);
  c->x_off.resize((size_t)D * Lp1);
  size_t o_rgb = 0, o_gb = 0, o_gg = 0, o_x = 0;
  for (int k = 0; k < D * Lp1; ++k) {
    int nb = c->nb_of_l[k], nq = c->nq_of_l[k];
    c->x_off[k] = (int)o_x;
    o_x += nq;
    // forward set: RGB [nq][nb], RBGwrho [nb][nq], d1GG, d2GG [nq][nq] (row-major)
    c->mat_off[k * 8 + M_BG] = (int)mats.size();
    for (int q = 0; q < nq; ++q)
      for (int b = 0; b < nb; ++b) mats.push_back(d->RGB[o_rgb + q + (size_t)nq * b]);
    c->mat_off[k * 8 + M_GB] = (int)mats.size();
    for (int b = 0; b < nb; ++b)
      for (int q = 0; q < nq; ++q) mats.push_back(d->RBGwrho[o_gb + b + (size_t)nb * q]);
    c->mat_off[k * 8 + M_D1] = (int)mats.size();
    for (int r = 0; r < nq; ++r)
      for (int s = 0; s < nq; ++s) mats.push_back(d->d1GG[o_gg + r + (size_t)nq * s]);
    c->mat_off[k * 8 + M_D2] = (int)mats.size();
    for (int r = 0; r < nq; ++r)
      for (int s = 0; s < nq; ++s) mats.push_back(d->d2GG[o_gg + r + (size_t)nq * s]);
    // transposed set (H^T = B->G with RBGwrho^T, G->B with RGB^T, d^T):
    c->mat_off[k * 8 + 4 + M_BG] = (int)mats.size();
    for (int q = 0; q < nq; ++q)
      for (int b = 0; b < nb; ++b) mats.push_back(d->RBGwrho[o_gb + b + (size_t)nb * q]);
    c->mat_off[k * 8 + 4 + M_GB] = (int)mats.size();
    for (int b = 0; b < nb; ++b)
      for (int q = 0; q < nq; ++q) mats.push_back(d->RGB[o_rgb + q + (size_t)nq * b]);
    c->mat_off[k * 8 + 4 + M_D1] = (int)mats.size();
    for (int r = 0; r < nq; ++r)
      for (int s = 0; s < nq; ++s) mats.push_back(d->d1GG[o_gg + s + (size_t)nq * r]);
    c->mat_off[k * 8 + 4 + M_D2] = (int)mats.size();
    for (int r = 0; r < nq; ++r)
      for (int s = 0; s < nq; ++s) mats.push_back(d->d2GG[o_gg + s + (size_t)nq * r]);
    // the diagonal's pattern matrices, [nb][nq] row-major (see diag_kernel):
    //   E = B o C^T, L1 = (B d1) o C^T, R1 = B o (d1 C)^T, LR = (B d1) o (d1 C)^T,
    //   L2 = (B d2) o C^T,  with B = RBGwrho, C = RGB, o the elementwise product
    {
      auto B = [&](int b, int q) { return d->RBGwrho[o_gb + b + (size_t)nb * q]; };
      auto C = [&](int q, int b) { return d->RGB[o_rgb + q + (size_t)nq * b]; };
      auto d1 = [&](int r, int s2) { return d->d1GG[o_gg + r + (size_t)nq * s2]; };
      auto d2 = [&](int r, int s2) { return d->d2GG[o_gg + r + (size_t)nq * s2]; };
      std::vector<double> Bd1((size_t)nb * nq), Bd2((size_t)nb * nq), d1C((size_t)nq * nb);
      for (int b = 0; b < nb; ++b)
        for (int q = 0; q < nq; ++q) {
          double a1 = 0.0, a2 = 0.0;
          for (int r = 0; r < nq; ++r) {
            a1 += B(b, r) * d1(r, q);
            a2 += B(b, r) * d2(r, q);
          }
          Bd1[(size_t)b * nq + q] = a1;
          Bd2[(size_t)b * nq + q] = a2;
        }
      for (int q = 0; q < nq; ++q)
        for (int b = 0; b < nb; ++b) {
          double a = 0.0;
          for (int r = 0; r < nq; ++r) a += d1(q, r) * C(r, b);
          d1C[(size_t)q * nb + b] = a;
        }
      if (c->diag_off.empty()) c->diag_off.resize((size_t)D * Lp1 * 5);
      for (int pat = 0; pat < 5; ++pat) {
        c->diag_off[(size_t)k * 5 + pat] = (int)mats.size();
        for (int b = 0; b < nb; ++b)
          for (int q = 0; q < nq; ++q) {
            const double l = (pat == 1 || pat == 3) ? Bd1[(size_t)b * nq + q] : (pat == 4 ? Bd2[(size_t)b * nq + q] : B(b, q));
            const double r = (pat == 2 || pat == 3) ? d1C[(size_t)q * nb + b] : C(q, b);
            mats.push_back(l * r);
          }
      }
    }
    o_rgb += (size_t)nq * nb;
    o_gb += (size_t)nq * nb;
    o_gg += (size_t)nq * nq;
  }
  c->terms.resize(d->nb_SG);
  long long onb = 0, onq = 0;
  for (long long t = 0; t < d->nb_SG; ++t) {
    TermInfo& T = c->terms[t];
    memset(&T, 0, sizeof(T));
    long long nb = 1, nq = 1;
    for (int i = 0; i < D; ++i) {
      int l = d->tab_l[t * D + i];
      T.l[i] = (unsigned char)l;
      nb *= c->nb_of_l[i * Lp1 + l];
      nq *= c->nq_of_l[i * Lp1 + l];
    }
    T.off_nb = onb;
    T.off_nq = onq;
    T.nb = (int)nb;
    T.nq = (int)nq;
    T.w = d->weight[t];
    onb += nb;
    onq += nq;
  }
  // inverse of the gather map: for each packed function, its DP entries in term order
  std::vector<long long> inv_ptr(d->N + 1, 0), inv_idx;
  for (long long k = 0; k < z.sum_nb; ++k)
    if (d->map[k] > 0) inv_ptr[d->map[k]]++;
  for (long long n = 0; n < d->N; ++n) inv_ptr[n + 1] += inv_ptr[n];
  inv_idx.resize(inv_ptr[d->N] > 0 ? inv_ptr[d->N] : 1);
  {
    std::vector<long long> fill(inv_ptr.begin(), inv_ptr.end() - 1);
    for (long long k = 0; k < z.sum_nb; ++k)
      if (d->map[k] > 0) inv_idx[fill[d->map[k] - 1]++] = k;
  }
  // chunks of each function's contribution list: at most EVR_RED_CHUNKS per function
  std::vector<long long> chunk_q, fun_chunk(d->N + 1, 0);
  for (long long n = 0; n < d->N; ++n) {
    fun_chunk[n] = (long long)chunk_q.size();
    const long long len = inv_ptr[n + 1] - inv_ptr[n];
    const long long csz = std::max<long long>(16, (len + EVR_RED_CHUNKS - 1) / EVR_RED_CHUNKS);
    for (long long q = inv_ptr[n]; q < inv_ptr[n + 1]; q += csz) chunk_q.push_back(q);
  }
  fun_chunk[d->N] = (long long)chunk_q.size();
  c->n_chunks = (long long)chunk_q.size();
  chunk_q.push_back(inv_ptr[d->N]);
  // launch geometry: persistent CTAs per SM sharing ~220 KB of shared memory
  // (wide until a work plan chooses otherwise)
  c->geo = 0;
  c->smem_doubles = geo_smem_bytes(0) / 8;
  c->grid = geo_ctas(0) * c->num_sms;
  if ((rc = upload(&c->d_map, d->map, (size_t)z.sum_nb)) ||
      (rc = upload(&c->d_mats, mats.data(), mats.size())) ||
      (rc = upload(&c->d_mat_off, c->mat_off.data(), c->mat_off.size())) ||
      (rc = upload(&c->d_diag_off, c->diag_off.data(), c->diag_off.size())) ||
      (rc = upload(&c->d_nb_of_l, c->nb_of_l.data(), c->nb_of_l.size())) ||
      (rc = upload(&c->d_nq_of_l, c->nq_of_l.data(), c->nq_of_l.size())) ||
      (rc = upload(&c->d_x, d->x, o_x)) ||
      (rc = upload(&c->d_x_off, c->x_off.data(), c->x_off.size())) ||
      (rc = upload<TermInfo>(&c->d_terms, nullptr, c->terms.size())) ||
      (rc = upload<unsigned int>(&c->d_counter, nullptr, 1)) ||
      (rc = upload(&c->d_inv_ptr, inv_ptr.data(), inv_ptr.size())) ||
      (rc = upload(&c->d_inv_idx, inv_idx.data(), inv_idx.size())) ||
      (rc = upload(&c->d_chunk_q, chunk_q.data(), chunk_q.size())) ||
      (rc = upload(&c->d_fun_chunk, fun_chunk.data(), fun_chunk.size()))) {
    free_ctx(c);
    return rc;
  }
  e = set_smem_attributes();
  if (e != cudaSuccess) {
    free_ctx(c);
    return set_error(EVR_ERR_CUDA, "evr_sg4_create: shared-memory attribute: %s", cudaGetErrorString(e));
  }
  *out = c;
  return EVR_OK;
}

extern "C" int evr_sg4_destroy(evr_sg4_ctx* c) {
  if (!c) return set_error(EVR_ERR_ARG, "evr_sg4_destroy: NULL context");
  cudaDeviceSynchronize();
  free_ctx(c);
  return EVR_OK;
}

// V (polynomial) and/or G (affine) on the grid points [g0, g1) (whole terms) into
// the context's field arrays, from index 0.
static int eval_fields(evr_sg4_ctx* c, long long g0, long long g1, bool V, bool G, cudaStream_t s) {
  if (g1 <= g0) return EVR_OK;
  const long long blocks = std::max<long long>(1, std::min<long long>((g1 - g0 + 255) / 256, 8LL * c->num_sms));
  fields_kernel<<<(unsigned)blocks, 256, 0, s>>>(c->d_terms, c->nb_SG, c->d_pt_start, c->d_nq_of_l, c->d_x,
                                                 c->d_x_off, c->D, c->L + 1, V ? c->V_nterms : 0, c->d_Vcoef,
                                                 c->d_Vfac, V ? c->d_V : nullptr, c->d_G0, c->d_G1,
                                                 G ? c->d_G : nullptr, g0, g1, c->nb0, c->z.sum_nq, c->G_sym);
  CUDA_TRY(cudaGetLastError());
  return EVR_OK;
}

extern "C" int evr_sg4_set_field_budget(evr_sg4_ctx* c, long long bytes) {
  if (!c) return set_error(EVR_ERR_ARG, "set_field_budget: NULL context");
  if (bytes < 0) return set_error(EVR_ERR_ARG, "set_field_budget: negative budget");
  c->field_budget = bytes;
  return EVR_OK;
}

extern "C" int evr_sg4_field_slices(const evr_sg4_ctx* c, long long* nslices) {
  if (!c || !nslices) return set_error(EVR_ERR_ARG, "field_slices: NULL argument");
  *nslices = c->streamed ? (long long)c->slice_term.size() - 1 : 0;
  return EVR_OK;
}

extern "C" int evr_sg4_set_operator(evr_sg4_ctx* c, const evr_sg4_op_desc* op) {
  if (!c || !op) return set_error(EVR_ERR_ARG, "evr_sg4_set_operator: NULL argument");
  if (op->type != 0 && op->type != 1 && op->type != 10)
    return set_error(EVR_ERR_ARG, "evr_sg4_set_operator: type_Op=%d not in {0,1,10}", op->type);
  const int D = c->D;
  const long long snq = c->z.sum_nq;
  for (double** p : {&c->d_V, &c->d_G, &c->d_Jac, &c->d_sqRho, &c->d_cfac, &c->d_F2, &c->d_F1, &c->d_Vcoef, &c->d_G0,
                     &c->d_G1, &c->d_t1grid})
    if (*p) {
      cudaFree(*p);
      *p = nullptr;
    }
  if (c->d_t1terms) cudaFree(c->d_t1terms);
  c->d_t1terms = nullptr;
  c->n_t1 = 0;
  c->t1_terms.clear();
  if (c->d_Vfac) cudaFree(c->d_Vfac);
  if (c->d_pt_start) cudaFree(c->d_pt_start);
  c->d_Vfac = nullptr;
  c->d_pt_start = nullptr;
  c->streamed = false;
  c->slice_term.clear();
  c->V_nterms = 0;
  c->have_op = false;
  c->type = op->type;
  c->items_nrhs = -1;  // work split depends on the operator's buffer count and the slices
  int rc;
  const long long nvg = snq * c->nb0 * c->nb0;  // V_grid entries
  const bool polyV = !op->V_grid && op->V_nterms > 0;
  const bool affG = op->type == 10 && !op->G_grid && (op->G0 || op->G1);
  std::vector<int> vfac;
  if (polyV) {
    if (!op->V_coef || !op->V_expo) return set_error(EVR_ERR_ARG, "V polynomial without coef/expo");
    vfac.assign((size_t)op->V_nterms * EVR_VFAC, -1);
    for (int t = 0; t < op->V_nterms; ++t) {
      int f = 0;
      for (int i = 0; i < D; ++i) {
        const int ex = op->V_expo[t * D + i];
        if (ex < 0 || ex > 16) return set_error(EVR_ERR_ARG, "V exponent outside [0,16]");
        if (ex == 0) continue;
        if (f == EVR_VFAC) return set_error(EVR_ERR_ARG, "V term %d depends on more than %d modes", t, EVR_VFAC);
        vfac[(size_t)t * EVR_VFAC + f++] = (i << 8) | ex;
      }
    }
  }
  // fields given in analytic form are streamed per term slice when they exceed the budget
  const bool grids = op->V_grid || (op->type == 10 && (op->G_grid || op->Jac_grid || op->sqRho_grid)) ||
                     (op->type == 1 && (op->F2_grid || op->F1_grid));
  const double bpp = 8.0 * (polyV ? 1 : 0) + 8.0 * D * D * (affG ? 1 : 0);  // bytes per grid point
  const bool stream = c->field_budget > 0 && !grids && (polyV || affG) && bpp * (double)snq > (double)c->field_budget;
  if (stream && c->nb0 > 1)
    return set_error(EVR_ERR_ARG, "field budget: streamed fields take one channel (nb0 = %d)", c->nb0);
  long long slice_pts = snq;
  if (stream) {
    const long long cap = (long long)((double)c->field_budget / bpp);
    c->slice_term.push_back(0);
    long long pts = 0;
    slice_pts = 0;
    for (long long t = 0; t < c->nb_SG; ++t) {
      const long long q = c->terms[t].nq;
      if (q > cap)
        return set_error(EVR_ERR_ARG, "field budget %lld B is below the fields of term %lld (%lld points)",
                         c->field_budget, t, q);
      if (pts + q > cap) {
        c->slice_term.push_back(t);
        pts = 0;
      }
      pts += q;
      slice_pts = std::max(slice_pts, pts);
    }
    c->slice_term.push_back(c->nb_SG);
  }
  if (op->V_grid) {
    for (long long k = 0; k < nvg; ++k)
      if (!std::isfinite(op->V_grid[k])) return set_error(EVR_ERR_NUMERIC, "V_grid[%lld] is not finite", k);
    if ((rc = upload(&c->d_V, op->V_grid, (size_t)nvg))) return rc;
  }
  if (polyV) CUDA_TRY(cudaMalloc(&c->d_V, (size_t)slice_pts * 8 * c->nb0 * c->nb0));
  if (op->type == 10) {
    if (op->G_grid) {
      if ((rc = upload(&c->d_G, op->G_grid, (size_t)snq * D * D))) return rc;
    } else if (affG) {
      CUDA_TRY(cudaMalloc(&c->d_G, (size_t)slice_pts * D * D * 8));
    }
    if (op->Jac_grid) {
      for (long long k = 0; k < snq; ++k)
        if (!(op->Jac_grid[k] != 0.0) || !std::isfinite(op->Jac_grid[k]))
          return set_error(EVR_ERR_NUMERIC, "Jac_grid[%lld] is zero or not finite", k);
      if ((rc = upload(&c->d_Jac, op->Jac_grid, (size_t)snq))) return rc;
    }
    if (op->sqRho_grid) {
      for (long long k = 0; k < snq; ++k)
        if (!(op->sqRho_grid[k] != 0.0) || !std::isfinite(op->sqRho_grid[k]))
          return set_error(EVR_ERR_NUMERIC, "sqRho_grid[%lld] is zero or not finite", k);
      if ((rc = upload(&c->d_sqRho, op->sqRho_grid, (size_t)snq))) return rc;
    }
    if (op->Jac_grid || op->sqRho_grid) {  // -1/2 / (Jac sqRhoOVERJac) per point
      std::vector<double> cf((size_t)snq);
      for (long long k = 0; k < snq; ++k)
        cf[k] = -0.5 / ((op->Jac_grid ? op->Jac_grid[k] : 1.0) * (op->sqRho_grid ? op->sqRho_grid[k] : 1.0));
      if ((rc = upload(&c->d_cfac, cf.data(), cf.size()))) return rc;
    }
  }
  memset(c->F2, 0, sizeof(c->F2));
  memset(c->F1, 0, sizeof(c->F1));
  if (op->type == 1) {
    if (op->F2)
      for (int i = 0; i < D; ++i)
        for (int j = i; j < D; ++j) c->F2[i * D + j] = op->F2[i * D + j];
    if (op->F1)
      for (int i = 0; i < D; ++i) c->F1[i] = op->F1[i];
  }
  if (op->type == 1 && (op->F2_grid || op->F1_grid)) {
    // Q-dependent coefficients: the term list in Init_TypeOp order, (i, j >= i)
    // then (i, 0), with the channel pairs (a, b) of each term inside (several
    // channels: one grid per pair, GridOp(:,a,b,iterm)); a grid that is zero
    // everywhere is skipped (grid_zero), a term without a grid keeps its
    // constant on every channel alike
    const int nc = c->nb0 * c->nb0;
    std::vector<T1Term> tl;
    std::vector<const double*> src;
    auto add = [&](int i, int j, const double* g, double cst) -> int {
      if (!g) {
        if (cst != 0.0) tl.push_back(T1Term{i, j, -1, -1, -1, cst});
        return EVR_OK;
      }
      for (int ab = 0; ab < nc; ++ab) {
        const double* ga = g + (size_t)ab * snq;
        bool zero = true;
        for (long long k = 0; k < snq; ++k) {
          if (!std::isfinite(ga[k]))
            return set_error(EVR_ERR_NUMERIC, "type-1 coefficient grid (%d, %d) is not finite", i, j);
          if (ga[k] != 0.0) zero = false;
        }
        if (zero) continue;
        tl.push_back(T1Term{i, j, c->nb0 > 1 ? ab / c->nb0 : -1, c->nb0 > 1 ? ab % c->nb0 : -1,
                            (long long)src.size() * snq, 0.0});
        src.push_back(ga);
      }
      return EVR_OK;
    };
    for (int i = 0; i < D; ++i)
      for (int j = i; j < D; ++j)
        if ((rc = add(i, j, op->F2_grid ? op->F2_grid + (size_t)(i * D + j) * nc * snq : nullptr, c->F2[i * D + j])))
          return rc;
    for (int i = 0; i < D; ++i)
      if ((rc = add(i, -1, op->F1_grid ? op->F1_grid + (size_t)i * nc * snq : nullptr, c->F1[i]))) return rc;
    memset(c->F2, 0, sizeof(c->F2));  // every term is in the list
    memset(c->F1, 0, sizeof(c->F1));
    if (!src.empty()) {
      CUDA_TRY(cudaMalloc(&c->d_t1grid, src.size() * (size_t)snq * 8));
      for (size_t k = 0; k < src.size(); ++k)
        CUDA_TRY(cudaMemcpy(c->d_t1grid + k * snq, src[k], (size_t)snq * 8, cudaMemcpyHostToDevice));
    }
    if (!tl.empty()) {
      CUDA_TRY(cudaMalloc(&c->d_t1terms, tl.size() * sizeof(T1Term)));
      CUDA_TRY(cudaMemcpy(c->d_t1terms, tl.data(), tl.size() * sizeof(T1Term), cudaMemcpyHostToDevice));
    }
    c->n_t1 = (int)tl.size();  // 0: every term zero, V alone remains (the constant path)
    c->t1_terms = tl;
  }
  if ((rc = upload(&c->d_F2, c->F2, (size_t)D * D)) || (rc = upload(&c->d_F1, c->F1, (size_t)D))) return rc;
  if (polyV || affG) {  // the analytic forms stay on the device (evaluated again per slice when streamed)
    std::vector<long long> start(c->nb_SG);
    for (long long t = 0; t < c->nb_SG; ++t) start[t] = c->terms[t].off_nq;
    CUDA_TRY(cudaMemcpy(c->d_terms, c->terms.data(), c->terms.size() * sizeof(TermInfo), cudaMemcpyHostToDevice));
    if ((rc = upload(&c->d_pt_start, start.data(), start.size()))) return rc;
    if (polyV && ((rc = upload(&c->d_Vcoef, op->V_coef, (size_t)op->V_nterms * c->nb0 * c->nb0)) ||
                  (rc = upload(&c->d_Vfac, vfac.data(), vfac.size()))))
      return rc;
    c->V_nterms = polyV ? op->V_nterms : 0;
    c->G_sym = 0;
    if (affG) {
      bool sym = true;
      for (int i = 0; i < D && sym; ++i)
        for (int j = 0; j < D && sym; ++j) {
          if (op->G0 && memcmp(&op->G0[i * D + j], &op->G0[j * D + i], sizeof(double)) != 0) sym = false;
          for (int k = 0; k < D && sym && op->G1; ++k)
            if (memcmp(&op->G1[((size_t)i * D + j) * D + k], &op->G1[((size_t)j * D + i) * D + k], sizeof(double)))
              sym = false;
        }
      c->G_sym = sym ? 1 : 0;
    }
    if (affG && op->G0 && (rc = upload(&c->d_G0, op->G0, (size_t)D * D))) return rc;
    if (affG && op->G1 && (rc = upload(&c->d_G1, op->G1, (size_t)D * D * D))) return rc;
    if (!stream) {
      if ((rc = eval_fields(c, 0, snq, polyV, affG, 0))) return rc;
      CUDA_TRY(cudaDeviceSynchronize());
    }
  }
  c->streamed = stream;
  c->have_op = true;
  return EVR_OK;
}


// Work list of one H.psi over nrhs_v virtual right-hand sides: (term, rhs
// block) items in term order with their costs, and the term table with each
// term's block size r for this nrhs_v (the context itself is not modified).
static void plan_work(const evr_sg4_ctx* c, int nrhs_v, int smem_doubles, std::vector<TermInfo>& terms,
                      std::vector<Item>& items, std::vector<float>& cost, long long& max_need) {
  const int nbuf = nbuf_for(c);
  const int Rmax = c->rmax;
  max_need = 0;
  items.clear();
  cost.clear();
  if (&terms != &c->terms) terms = c->terms;
  for (long long t = 0; t < c->nb_SG; ++t) {
    TermInfo& T = terms[t];
    long long per = (long long)nbuf * T.nq;
    int r = (int)std::min<long long>(std::min(nrhs_v, Rmax), std::max<long long>(1, smem_doubles / per));
    if (c->nb0 > 1) {  // whole channel groups (both halves of complex columns): 2 nb0 columns
      const int g = 2 * c->nb0;
      r = std::max(g, r / g * g);
    }
    T.r = r;
    max_need = std::max(max_need, per * r);
    double fl = 0;  // cost ~ grid size times the 1-D lengths
    for (int i = 0; i < c->D; ++i) fl += c->nq_of_l[i * (c->L + 1) + T.l[i]];
    T.cost = (float)(fl * T.nq);
    for (int r0 = 0; r0 < nrhs_v; r0 += r) {
      items.push_back(Item{(int)t, r0});
      cost.push_back(T.cost * std::min(r, nrhs_v - r0));
    }
  }
}

// Geometry of a plan with n_wide items planned for the wide kernel: plans of
// at least EVR_BIG_WAVES waves go narrow (D <= 6) or mid (D > 6).
static int choose_geo(int D, size_t n_wide, int num_sms) {
  if (n_wide < (size_t)EVR_BIG_WAVES * geo_ctas(0) * num_sms) return 0;
  return D <= EVR_NARROW_FMAX ? 1 : 2;
}

// The same list sorted by decreasing cost (the persistent kernel then ends
// balanced), with each term's block size written into `terms`, and the
// launch geometry chosen for this plan (the context is not modified).
static void plan_sorted(const evr_sg4_ctx* c, int nrhs_v, std::vector<TermInfo>& terms, std::vector<Item>& items,
                        std::vector<Item>& sorted, long long& max_need, int& geo) {
  std::vector<float> cost;
  plan_work(c, nrhs_v, geo_smem_bytes(0) / 8, terms, items, cost, max_need);
  geo = c->geo_override >= 0 ? c->geo_override : choose_geo(c->D, items.size(), c->num_sms);
  if (geo) plan_work(c, nrhs_v, geo_smem_bytes(geo) / 8, terms, items, cost, max_need);
  std::vector<int> order(items.size());
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return cost[a] > cost[b]; });
  sorted.resize(items.size());
  for (size_t k = 0; k < order.size(); ++k) sorted[k] = items[order[k]];
}

// plan_sorted into the context's own term table and launch geometry
// (c->terms, c->geo, c->smem_doubles, c->grid).
static void plan_items(evr_sg4_ctx* c, int nrhs_v, std::vector<Item>& items, std::vector<Item>& sorted,
                       long long& max_need) {
  int geo = 0;
  plan_sorted(c, nrhs_v, c->terms, items, sorted, max_need, geo);
  c->geo = geo;
  c->smem_doubles = geo_smem_bytes(geo) / 8;
  c->grid = geo_ctas(geo) * c->num_sms;
}

// a single context's device work list: every item in slot 0
static std::vector<MItem> slot0_items(const std::vector<Item>& items) {
  std::vector<MItem> out(items.size());
  for (size_t k = 0; k < items.size(); ++k) out[k] = MItem{0, items[k].term, items[k].rhs0, 0};
  return out;
}

static int build_items(evr_sg4_ctx* c, int nrhs_v) {
  if (c->items_nrhs == nrhs_v) return EVR_OK;
  std::vector<Item> items, sorted;
  long long max_need = 0;
  plan_items(c, nrhs_v, items, sorted, max_need);
  // streamed fields: the list runs slice by slice (decreasing cost within a slice)
  c->slice_item.assign(1, 0);
  if (c->streamed) {
    auto slice_of = [&](int term) {
      return (int)(std::upper_bound(c->slice_term.begin(), c->slice_term.end(), (long long)term) -
                   c->slice_term.begin()) - 1;
    };
    std::stable_sort(sorted.begin(), sorted.end(),
                     [&](const Item& a, const Item& b) { return slice_of(a.term) < slice_of(b.term); });
    const int ns = (int)c->slice_term.size() - 1;
    size_t q = 0;
    for (int k = 0; k < ns; ++k) {
      while (q < sorted.size() && slice_of(sorted[q].term) == k) ++q;
      c->slice_item.push_back((int)q);
    }
  } else {
    c->slice_item.push_back((int)sorted.size());
  }
  c->term_item_start.assign(c->nb_SG + 1, 0);
  for (size_t k = 0; k < items.size(); ++k) c->term_item_start[items[k].term + 1]++;
  for (long long t = 0; t < c->nb_SG; ++t) c->term_item_start[t + 1] += c->term_item_start[t];
  size_t need = std::max<size_t>(1, items.size());
  if (need > c->items_cap) {
    if (c->d_items) cudaFree(c->d_items);
    c->d_items = nullptr;
    CUDA_TRY(cudaMalloc(&c->d_items, need * sizeof(MItem)));
    c->items_cap = need;
  }
  {
    const std::vector<MItem> ms = slot0_items(sorted);
    CUDA_TRY(cudaMemcpy(c->d_items, ms.data(), ms.size() * sizeof(MItem), cudaMemcpyHostToDevice));
  }
  {
    const std::vector<MItem> pl = slot0_items(items);
    if (c->d_plain_items) cudaFree(c->d_plain_items);
    c->d_plain_items = nullptr;
    CUDA_TRY(cudaMalloc(&c->d_plain_items, std::max<size_t>(1, pl.size()) * sizeof(MItem)));
    CUDA_TRY(cudaMemcpy(c->d_plain_items, pl.data(), pl.size() * sizeof(MItem), cudaMemcpyHostToDevice));
  }
  CUDA_TRY(cudaMemcpy(c->d_terms, c->terms.data(), c->terms.size() * sizeof(TermInfo), cudaMemcpyHostToDevice));
  c->n_items = (int)items.size();
  // global scratch for terms that do not fit in shared memory
  long long per_cta = max_need > c->smem_doubles ? max_need : 0;
  if ((size_t)per_cta * c->grid > c->scratch_cap) {
    if (c->d_scratch) cudaFree(c->d_scratch);
    c->d_scratch = nullptr;
    CUDA_TRY(cudaMalloc(&c->d_scratch, (size_t)per_cta * c->grid * 8));
    c->scratch_cap = (size_t)per_cta * c->grid;
  }
  c->scratch_per_cta = per_cta;
  size_t pneed = (size_t)c->n_chunks * nrhs_v * 2;
  if (pneed > c->part_cap) {
    if (c->d_part) cudaFree(c->d_part);
    c->d_part = nullptr;
    CUDA_TRY(cudaMalloc(&c->d_part, pneed * 8));
    c->part_cap = pneed;
  }
  size_t cneed = (size_t)c->z.sum_nb * nrhs_v;
  if (cneed > c->contrib_cap) {
    if (c->d_contrib) cudaFree(c->d_contrib);
    c->d_contrib = nullptr;
    CUDA_TRY(cudaMalloc(&c->d_contrib, cneed * 8));
    c->contrib_cap = cneed;
  }
  c->items_nrhs = nrhs_v;
  return EVR_OK;
}

static int launch_reduce(evr_sg4_ctx* c, const double* contrib, double2* part, int nrhs_v, int cshift,
                         const double* psi, long long ldpsi, double* hpsi, long long ldh, double E0, double Esc,
                         cudaStream_t s) {
  // 64-thread blocks, up to 64 per SM: every thread runs a serial chain of
  // FP64 additions, and GB300's FP64 pipe (about two operations per clock
  // per SM) wants small reductions spread over all SMs
  const long long t1 = c->n_chunks * nrhs_v, t2 = c->N * nrhs_v;
  const long long b1 = std::max<long long>(1, std::min<long long>((t1 + 63) / 64, 64LL * c->num_sms));
  const long long b2 = std::max<long long>(1, std::min<long long>((t2 + 63) / 64, 64LL * c->num_sms));
  hpsi_reduce_chunks_kernel<<<(unsigned)b1, 64, 0, s>>>(contrib, c->d_chunk_q, c->n_chunks, c->d_inv_idx, nrhs_v,
                                                       part);
  hpsi_reduce_join_kernel<<<(unsigned)b2, 64, 0, s>>>(part, c->d_fun_chunk, c->N, nrhs_v, cshift, psi, ldpsi, hpsi,
                                                     ldh, E0, Esc, c->nb0);
  CUDA_TRY(cudaGetLastError());
  return EVR_OK;
}

static KParams make_params(evr_sg4_ctx* c, int nrhs_v, int cshift, const double* psi, long long ldpsi,
                           double* hpsi, long long ldh, double scale) {
  KParams p;
  memset(&p, 0, sizeof(p));
  p.D = c->D;
  p.Lp1 = c->L + 1;
  p.nrhs_v = nrhs_v;
  p.cshift = cshift;
  p.terms = c->d_terms;
  p.map = c->d_map;
  p.mats = c->d_mats;
  p.mat_off = c->d_mat_off;
  p.nb_of_l = c->d_nb_of_l;
  p.nq_of_l = c->d_nq_of_l;
  p.psi = psi;
  p.ldpsi = ldpsi;
  p.hpsi = hpsi;
  p.ldh = ldh;
  p.scale = scale;
  p.V = c->d_V;
  p.G = c->d_G;
  p.Jac = c->d_Jac;
  p.sqRho = c->d_sqRho;
  p.F2 = c->d_F2;
  p.F1 = c->d_F1;
  p.t1_mixed = c->type == 1 && t1_mixed(c) ? 1 : 0;
  p.n_t1 = c->type == 1 ? c->n_t1 : 0;
  p.t1terms = c->d_t1terms;
  p.t1grid = c->d_t1grid;
  p.split = c->split;
  p.type = c->type;
  p.nbuf = nbuf_for(c);
  p.smem_doubles = c->smem_doubles;
  p.gscratch = c->d_scratch;
  p.scratch_per_cta = c->scratch_per_cta;
  p.contrib = c->d_contrib;
  p.cfac = c->d_cfac;
  p.sum_nb = c->z.sum_nb;
  p.nb0 = c->nb0;
  p.Nfun = c->N;
  p.vstride = c->z.sum_nq;
  return p;
}

static int hpsi_common(evr_sg4_ctx* c, int nrhs, int cshift, const double* psi, long long ldpsi,
                       double* hpsi, long long ldh, double E0, double Esc, void* stream, bool plain,
                       bool transpose = false) {
  if (!c) return set_error(EVR_ERR_ARG, "hpsi: NULL context");
  if (!c->have_op) return set_error(EVR_ERR_STATE, "hpsi: set_operator was not called");
  if (plain && c->streamed)
    return set_error(EVR_ERR_STATE, "hpsi: the per-term path needs resident operator fields (the budget streams them)");
  if (nrhs < 1) return set_error(EVR_ERR_ARG, "hpsi: nrhs=%d (size(Psi)=0 stops the reference)", nrhs);
  if (!psi || !hpsi) return set_error(EVR_ERR_ARG, "hpsi: NULL vector");
  if (ldpsi < c->nvec || ldh < c->nvec)
    return set_error(EVR_ERR_ARG, "hpsi: leading dimension < nb0*N=%lld", c->nvec);
  if (!(Esc != 0.0) || !std::isfinite(Esc) || !std::isfinite(E0))
    return set_error(EVR_ERR_ARG, "hpsi: Esc must be finite and non-zero");
  cudaPointerAttributes a1, a2;
  if (cudaPointerGetAttributes(&a1, psi) != cudaSuccess || cudaPointerGetAttributes(&a2, hpsi) != cudaSuccess ||
      a1.type != cudaMemoryTypeDevice || a2.type != cudaMemoryTypeDevice) {
    cudaGetLastError();
    return set_error(EVR_ERR_ARG, "hpsi: psi and hpsi must be device pointers (use evr_sg4_hpsi_host)");
  }
  const int nrhs_v = (nrhs * c->nb0) << cshift;  // one virtual column per (rhs, channel, re/im)
  int rc = build_items(c, nrhs_v);
  if (rc) return rc;
  cudaStream_t s = (cudaStream_t)stream;
  const long long ldv_psi = ldpsi << cshift, ldv_h = ldh << cshift;
  KParams p = make_params(c, nrhs_v, cshift, psi, ldv_psi, hpsi, ldv_h, 1.0);
  p.transpose = transpose ? 1 : 0;
  const size_t smem = (size_t)c->smem_doubles * 8;
  long long launches = 0;
  if (!plain && c->streamed) {  // per slice: its fields, then its items
    for (size_t k = 0; k + 1 < c->slice_term.size(); ++k) {
      const long long t0 = c->slice_term[k], t1 = c->slice_term[k + 1];
      const long long g0 = c->terms[t0].off_nq, g1 = t1 < c->nb_SG ? c->terms[t1].off_nq : c->z.sum_nq;
      if ((rc = eval_fields(c, g0, g1, c->V_nterms > 0, c->d_G1 || c->d_G0, s))) return rc;
      CUDA_TRY(cudaMemsetAsync(c->d_counter, 0, sizeof(unsigned int), s));
      KParams q = p;
      q.fbase = g0;
      launch_single(c->geo, c->grid, smem, s, q, c->d_items + c->slice_item[k],
                    c->slice_item[k + 1] - c->slice_item[k], c->d_counter);
      CUDA_TRY(cudaGetLastError());
      launches += 2;
    }
  } else if (!plain) {
    CUDA_TRY(cudaMemsetAsync(c->d_counter, 0, sizeof(unsigned int), s));
    launch_single(c->geo, c->grid, smem, s, p, c->d_items, c->n_items, c->d_counter);
    CUDA_TRY(cudaGetLastError());
    launches = 1;
  } else {
    for (long long t = 0; t < c->nb_SG; ++t) {  // one launch per Smolyak term
      const int b0 = c->term_item_start[t], b1 = c->term_item_start[t + 1];
      launch_multi(c->geo, b1 - b0, smem, s, &p, 1, c->d_plain_items, b1, b0, nullptr);
      ++launches;
    }
    CUDA_TRY(cudaGetLastError());
  }
  if ((rc = launch_reduce(c, c->d_contrib, (double2*)c->d_part, nrhs_v, cshift, psi, ldv_psi, hpsi, ldv_h, E0, Esc,
                          s)))
    return rc;
  CUDA_TRY(cudaGetLastError());
  c->last_launches = launches + 2;
  return EVR_OK;
}

extern "C" int evr_sg4_hpsi(evr_sg4_ctx* c, int nrhs, const double* psi, long long ldpsi, double* hpsi,
                            long long ldh, double E0, double Esc, void* stream) {
  return hpsi_common(c, nrhs, 0, psi, ldpsi, hpsi, ldh, E0, Esc, stream, false);
}

extern "C" int evr_sg4_hpsi_plain(evr_sg4_ctx* c, int nrhs, const double* psi, long long ldpsi, double* hpsi,
                                  long long ldh, void* stream) {
  return hpsi_common(c, nrhs, 0, psi, ldpsi, hpsi, ldh, 0.0, 1.0, stream, true);
}

extern "C" int evr_sg4_hpsi_cplx(evr_sg4_ctx* c, int nrhs, const double* psi, long long ldpsi, double* hpsi,
                                 long long ldh, double E0, double Esc, void* stream) {
  return hpsi_common(c, nrhs, 1, psi, ldpsi, hpsi, ldh, E0, Esc, stream, false);
}

extern "C" int evr_sg4_apply(evr_sg4_ctx* c, int flags, int nrhs, const double* psi, long long ldpsi,
                             double* hpsi, long long ldh, double E0, double Esc, void* stream) {
  if (flags & ~(EVR_APPLY_TRANSPOSE | EVR_APPLY_COMPLEX | EVR_APPLY_PLAIN))
    return set_error(EVR_ERR_ARG, "apply: unknown flags 0x%x", flags);
  const bool plain = (flags & EVR_APPLY_PLAIN) != 0;
  if (plain && ((flags & EVR_APPLY_COMPLEX) || E0 != 0.0 || Esc != 1.0))
    return set_error(EVR_ERR_ARG, "apply: the per-term path takes real psi with E0=0, Esc=1");
  return hpsi_common(c, nrhs, (flags & EVR_APPLY_COMPLEX) ? 1 : 0, psi, ldpsi, hpsi, ldh, E0, Esc, stream, plain,
                     (flags & EVR_APPLY_TRANSPOSE) != 0);
}

extern "C" int evr_sg4_hpsi_host(evr_sg4_ctx* c, int nrhs, const double* psi, long long ldpsi, double* hpsi,
                                 long long ldh, double E0, double Esc) {
  if (!c) return set_error(EVR_ERR_ARG, "hpsi_host: NULL context");
  if (nrhs < 1 || !psi || !hpsi || ldpsi < c->nvec || ldh < c->nvec)
    return set_error(EVR_ERR_ARG, "hpsi_host: bad sizes or NULL vectors");
  size_t n = (size_t)c->nvec * nrhs;
  if (2 * n > c->io_cap) {
    if (c->d_io) cudaFree(c->d_io);
    c->d_io = nullptr;
    CUDA_TRY(cudaMalloc(&c->d_io, 2 * n * 8));
    c->io_cap = 2 * n;
  }
  double* dpsi = c->d_io;
  double* dh = c->d_io + n;
  CUDA_TRY(cudaMemcpy2DAsync(dpsi, (size_t)c->nvec * 8, psi, (size_t)ldpsi * 8, (size_t)c->nvec * 8, nrhs,
                             cudaMemcpyHostToDevice, 0));
  int rc = evr_sg4_hpsi(c, nrhs, dpsi, c->nvec, dh, c->nvec, E0, Esc, nullptr);
  if (rc) return rc;
  CUDA_TRY(cudaMemcpy2DAsync(hpsi, (size_t)ldh * 8, dh, (size_t)c->nvec * 8, (size_t)c->nvec * 8, nrhs,
                             cudaMemcpyDeviceToHost, 0));
  CUDA_TRY(cudaStreamSynchronize(0));
  return EVR_OK;
}

extern "C" int evr_sg4_flops_per_rhs(const evr_sg4_ctx* c, double* flops) {
  if (!c || !flops) return set_error(EVR_ERR_ARG, "flops: NULL argument");
  if (!c->have_op) return set_error(EVR_ERR_STATE, "flops: set_operator was not called");
  const int D = c->D, Lp1 = c->L + 1;
  double F = 0.0;
  for (const TermInfo& T : c->terms) {
    int nb[EVR_MAXD], nq[EVR_MAXD];
    for (int i = 0; i < D; ++i) {
      nb[i] = c->nb_of_l[i * Lp1 + T.l[i]];
      nq[i] = c->nq_of_l[i * Lp1 + T.l[i]];
    }
    // B->G and G->B in the mode order the kernel uses (ascending
    // (nq-nb)/(nb*nq), ties by index; G->B reversed): 2 nin nout flops per fibre
    int ord[EVR_MAXD];
    mode_order(nb, nq, D, ord);
    double f = 0.0;
    for (int dir = 0; dir < 2; ++dir) {
      int cur[EVR_MAXD];
      for (int i = 0; i < D; ++i) cur[i] = dir == 0 ? nb[i] : nq[i];
      for (int k = 0; k < D; ++k) {
        const int i = ord[dir == 0 ? k : D - 1 - k];
        double rest = 1.0;
        for (int j = 0; j < D; ++j)
          if (j != i) rest *= cur[j];
        f += 2.0 * nb[i] * nq[i] * rest;
        cur[i] = dir == 0 ? nq[i] : nb[i];
      }
    }
    double sum_nqi = 0;
    for (int i = 0; i < D; ++i) sum_nqi += nq[i];
    const double q = T.nq;
    // V.x: one product per point, or a row of the nb0 x nb0 electronic matrix
    const double vq = c->d_V ? (c->nb0 > 1 ? 2.0 * c->nb0 * q : q) : 0.0;
    if (c->type == 0) {
      f += vq;
    } else if (c->type == 1 && c->n_t1 > 0) {  // term by term: derivative passes, then coefficient x result
      f += vq;
      int pi = -2, pj = -2;
      for (const T1Term& t : c->t1_terms) {
        if (t.i != pi || t.j != pj) f += 2.0 * q * nq[t.i] + (t.j > t.i ? 2.0 * q * nq[t.j] : 0.0);
        pi = t.i;
        pj = t.j;
        f += t.a < 0 ? 2.0 * q : 2.0 * q / c->nb0;  // per column: a channel-pair grid acts on one channel of nb0
      }
    } else if (c->type == 1) {  // the fused passes (type1_fused; the same for a diagonal F2 term by term)
      f += vq;
      for (int i = 0; i < D; ++i)
        if (c->F2[i * D + i] != 0.0) f += 2.0 * q * nq[i] + 2.0 * q;  // F2_ii d2_i x
      if (t1_mixed(c)) {
        for (int i = 0; i < D; ++i) {
          f += 2.0 * q * nq[i];                                       // d_i x
          if (c->F1[i] != 0.0) f += 2.0 * q;                          // F1_i d_i x
        }
        f += 2.0 * q * (D * (D - 1) / 2);                             // U_i = sum_{j>i} F2_ij d_j x
        for (int i = 0; i + 1 < D; ++i) f += 2.0 * q * nq[i];         // d_i U_i
      }
    } else {
      f += 4.0 * q * sum_nqi;                       // D derivative passes, twice
      f += c->d_G ? 2.0 * D * D * q : 0.0;           // G contraction
      f += (c->d_Jac ? 2.0 * D * q : 0.0) + (c->d_sqRho ? 2.0 * q : 0.0);
      f += vq + 2.0 * q;                            // V.x and the final multiply-add
    }
    f += 2.0 * T.nb;                                // weighted scatter
    F += f;
  }
  *flops = F;
  return EVR_OK;
}

extern "C" int evr_sg4_ctx_sizes(const evr_sg4_ctx* c, long long* out) {
  if (!c || !out) return set_error(EVR_ERR_ARG, "ctx_sizes: NULL argument");
  out[0] = c->nvec;
  out[1] = c->nb_SG;
  out[2] = c->z.sum_nb;
  out[3] = c->z.sum_nq;
  out[4] = c->z.max_nb;
  out[5] = c->z.max_nq;
  out[6] = c->D;
  out[7] = c->L;
  return EVR_OK;
}

extern "C" int evr_sg4_last_geometry(const evr_sg4_ctx* c, int* geo, int* ctas_per_sm) {
  if (!c || !geo) return set_error(EVR_ERR_ARG, "last_geometry: NULL argument");
  *geo = c->geo;
  if (ctas_per_sm) *ctas_per_sm = geo_ctas(c->geo);
  return EVR_OK;
}

extern "C" int evr_sg4_last_launches(const evr_sg4_ctx* c, long long* n) {
  if (!c || !n) return set_error(EVR_ERR_ARG, "last_launches: NULL argument");
  *n = c->last_launches;
  return EVR_OK;
}

extern "C" int evr_probe_fp64_peak(double* tflops) {
  if (!tflops) return set_error(EVR_ERR_ARG, "probe: NULL argument");
  int dev = 0, sms = 0;
  CUDA_TRY(cudaGetDevice(&dev));
  CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  const int blocks = 4 * sms, threads = 256, iters = 2048;
  double* d = nullptr;
  CUDA_TRY(cudaMalloc(&d, sizeof(double) * blocks * threads));
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  dfma_peak_kernel<<<blocks, threads>>>(d, 64, 1.0000001, 1e-9);
  float best = 1e30f;
  for (int rep = 0; rep < 3; ++rep) {
    cudaEventRecord(e0);
    dfma_peak_kernel<<<blocks, threads>>>(d, iters, 1.0000001, 1e-9);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    best = std::min(best, ms);
  }
  cudaError_t e = cudaGetLastError();
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(d);
  if (e != cudaSuccess) return set_error(EVR_ERR_CUDA, "probe: %s", cudaGetErrorString(e));
  *tflops = 2.0 * 8 * iters * (double)blocks * threads / (best * 1e-3) / 1e12;
  return EVR_OK;
}

extern "C" int evr_probe_fp64_pipes(double* dfma_tflops, double* dmma_tflops, double* mixed_tflops) {
  if (!dfma_tflops || !dmma_tflops || !mixed_tflops) return set_error(EVR_ERR_ARG, "probe: NULL argument");
  int rc = evr_probe_fp64_peak(dfma_tflops);
  if (rc) return rc;
  int dev = 0, sms = 0;
  CUDA_TRY(cudaGetDevice(&dev));
  CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  const int blocks = 4 * sms, threads = 256, iters = 4096;
  double* d = nullptr;
  CUDA_TRY(cudaMalloc(&d, sizeof(double) * blocks * threads));
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  float best[2] = {1e30f, 1e30f};
  for (int mixed = 0; mixed < 2; ++mixed) {
    dmma_peak_kernel<<<blocks, threads>>>(d, 64, mixed, 1.0000001, 1e-9);
    for (int rep = 0; rep < 3; ++rep) {
      cudaEventRecord(e0);
      dmma_peak_kernel<<<blocks, threads>>>(d, iters, mixed, 1.0000001, 1e-9);
      cudaEventRecord(e1);
      cudaEventSynchronize(e1);
      float ms = 0;
      cudaEventElapsedTime(&ms, e0, e1);
      best[mixed] = std::min(best[mixed], ms);
    }
  }
  cudaError_t e = cudaGetLastError();
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(d);
  if (e != cudaSuccess) return set_error(EVR_ERR_CUDA, "probe: %s", cudaGetErrorString(e));
  const double warps = (double)blocks * threads / 32.0;
  const double mma_flops = 4.0 * 512.0 * iters * warps;           // four m8n8k4 per step per warp
  const double fma_flops = 2.0 * 4.0 * iters * blocks * threads;  // four DFMA per step per thread
  *dmma_tflops = mma_flops / (best[0] * 1e-3) / 1e12;
  *mixed_tflops = (mma_flops + fma_flops) / (best[1] * 1e-3) / 1e12;
  return EVR_OK;
}

// ------------------------------------------------------------------------
// H.psi without device allocation.
//
// Some callers cannot call cudaMalloc: code running inside a caller-owned
// memory budget (a host program whose allocator owns every device byte and
// forbids allocations behind its back), or a real-time loop that must stay
// out of the driver's allocator, whose calls can synchronise the device.
// evr_sg4_hpsi_noalloc gives them the persistent kernel with all of its scratch
// -- the work counter, the term table of this call's plan, the work list,
// the per-term contributions, the chunk partials of the ordered accumulation
// and the per-CTA slabs for terms larger than shared memory -- carved from
// one fixed, file-scope device array instead of device allocations.
//
// The array (EVR_SG4_NOALLOC_SCRATCH_BYTES) exists on every device that
// loads this library and stays resident until the process exits.  Every
// call shares it and it keeps the previous call's contents: the counter is
// cleared at the start of each call and every other byte a call reads is
// written by that call first.  Two calls whose kernels overlap on the GPU
// (different streams, or different host threads) race on the array: keep
// calls on one stream, or serialise them.  The call plans into local copies
// (term table, geometry), so the context's own cached plan for evr_sg4_hpsi
// is left as it was.
// ------------------------------------------------------------------------
static __device__ __align__(256) unsigned char g_noalloc_scratch[EVR_SG4_NOALLOC_SCRATCH_BYTES];

namespace evr {
static std::mutex g_noalloc_mu;
static unsigned char* g_noalloc_ptr[64];  // device address of the array, per device
}  // namespace evr

extern "C" int evr_sg4_hpsi_noalloc(evr_sg4_ctx* c, int nrhs, const double* psi, long long ldpsi,
                                    double* hpsi, long long ldh, double E0, double Esc, void* stream) {
  if (!c) return set_error(EVR_ERR_ARG, "hpsi_noalloc: NULL context");
  if (!c->have_op) return set_error(EVR_ERR_STATE, "hpsi_noalloc: set_operator was not called");
  if (c->streamed) return set_error(EVR_ERR_STATE, "hpsi_noalloc: the operator fields are streamed (use evr_sg4_hpsi)");
  if (nrhs < 1) return set_error(EVR_ERR_ARG, "hpsi_noalloc: nrhs=%d", nrhs);
  if (!psi || !hpsi) return set_error(EVR_ERR_ARG, "hpsi_noalloc: NULL vector");
  if (ldpsi < c->nvec || ldh < c->nvec)
    return set_error(EVR_ERR_ARG, "hpsi_noalloc: leading dimension < nb0*N=%lld", c->nvec);
  if (!(Esc != 0.0) || !std::isfinite(Esc) || !std::isfinite(E0))
    return set_error(EVR_ERR_ARG, "hpsi_noalloc: Esc must be finite and non-zero");
  int dev = 0;
  CUDA_TRY(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64 || dev != c->device)
    return set_error(EVR_ERR_STATE, "hpsi_noalloc: current device %d is not the context's device %d", dev, c->device);
  unsigned char* base = nullptr;
  {
    // set-up, once per device with that device current: the device address of
    // the array (its host-side name is only a stand-in, never passed to a kernel)
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    if (!g_noalloc_ptr[dev]) {
      void* ptr = nullptr;
      cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
      if (e != cudaSuccess || !ptr)
        return set_error(EVR_ERR_CUDA, "hpsi_noalloc: cudaGetSymbolAddress: %s", cudaGetErrorString(e));
      g_noalloc_ptr[dev] = (unsigned char*)ptr;
    }
    base = g_noalloc_ptr[dev];
  }
  cudaPointerAttributes a1, a2;
  if (cudaPointerGetAttributes(&a1, psi) != cudaSuccess || cudaPointerGetAttributes(&a2, hpsi) != cudaSuccess ||
      a1.type != cudaMemoryTypeDevice || a2.type != cudaMemoryTypeDevice) {
    cudaGetLastError();
    return set_error(EVR_ERR_ARG, "hpsi_noalloc: psi and hpsi must be device pointers");
  }
  const int nrhs_v = nrhs * c->nb0;
  // this call's plan, in local copies: the context's cached plan stays as it is
  std::vector<TermInfo> terms;
  std::vector<Item> items, sorted;
  long long max_need = 0;
  int geo = 0;
  plan_sorted(c, nrhs_v, terms, items, sorted, max_need, geo);
  const int smem_doubles = geo_smem_bytes(geo) / 8;
  // carve: [counter | terms | items | contributions | chunk partials | large-term slabs], 256-byte aligned
  auto up = [](size_t x) { return (x + 255) & ~(size_t)255; };
  const size_t off_terms = 256;
  const size_t off_items = off_terms + up(terms.size() * sizeof(TermInfo));
  const size_t off_contrib = off_items + up(sorted.size() * sizeof(MItem));
  const size_t off_part = off_contrib + up((size_t)c->z.sum_nb * nrhs_v * 8);
  const size_t off_slabs = off_part + up((size_t)c->n_chunks * nrhs_v * 16);
  const long long per_cta = max_need > smem_doubles ? max_need : 0;
  // with large-term slabs, launch only as many CTAs as the array has slabs for
  int grid = geo_ctas(geo) * c->num_sms;
  if (per_cta > 0 && off_slabs < (size_t)EVR_SG4_NOALLOC_SCRATCH_BYTES)
    grid = (int)std::min<long long>(grid, ((size_t)EVR_SG4_NOALLOC_SCRATCH_BYTES - off_slabs) / ((size_t)per_cta * 8));
  const size_t total = off_slabs + (size_t)per_cta * std::max(grid, 1) * 8;
  if (grid < 1 || total > (size_t)EVR_SG4_NOALLOC_SCRATCH_BYTES)
    return set_error(EVR_ERR_ARG,
                     "hpsi_noalloc: this operator and nrhs=%d need %zu bytes of scratch, more than the fixed "
                     "%u-byte array; use evr_sg4_hpsi or fewer right-hand sides",
                     nrhs, total, (unsigned)EVR_SG4_NOALLOC_SCRATCH_BYTES);
  cudaStream_t s = (cudaStream_t)stream;
  // both host lists are pageable: cudaMemcpyAsync stages them before it
  // returns, so they may go out of scope when this call does
  CUDA_TRY(cudaMemcpyAsync(base + off_terms, terms.data(), terms.size() * sizeof(TermInfo), cudaMemcpyHostToDevice,
                           s));
  const std::vector<MItem> ms = slot0_items(sorted);
  CUDA_TRY(cudaMemcpyAsync(base + off_items, ms.data(), ms.size() * sizeof(MItem), cudaMemcpyHostToDevice, s));
  CUDA_TRY(cudaMemsetAsync(base, 0, sizeof(unsigned int), s));
  KParams p = make_params(c, nrhs_v, 0, psi, ldpsi, hpsi, ldh, 1.0);
  p.terms = (const TermInfo*)(base + off_terms);
  p.smem_doubles = smem_doubles;
  p.contrib = (double*)(base + off_contrib);
  p.gscratch = per_cta ? (double*)(base + off_slabs) : nullptr;
  p.scratch_per_cta = per_cta;
  launch_single(geo, grid, (size_t)smem_doubles * 8, s, p, (const MItem*)(base + off_items), (int)ms.size(),
                (unsigned int*)base);
  CUDA_TRY(cudaGetLastError());
  int rc = launch_reduce(c, p.contrib, (double2*)(base + off_part), nrhs_v, 0, psi, ldpsi, hpsi, ldh, E0, Esc, s);
  if (rc) return rc;
  CUDA_TRY(cudaGetLastError());
  c->last_launches = 3;
  return EVR_OK;
}

// ------------------------------------------------------------------------
// Several independent Hamiltonians in one persistent launch.  The plan owns
// everything that depends on the right-hand-side count (term blocks, the
// per-term contributions, chunk partials, one global-scratch slab per CTA
// shared by all contexts) and the merged cost-sorted item list; the contexts
// lend their read-only tables and operator grids.
// ------------------------------------------------------------------------
// One persistent launch of a plan: the merged items of its contexts (at most
// EVR_PB_LARGE), in one launch geometry.
struct MGroup {
  int geo = 0, grid = 0, smem_doubles = 0;
  std::vector<int> ctx_of;       // slot in the launch's parameter block -> context
  std::vector<MItem> sorted;     // its contexts' items (ctx = slot), decreasing cost
  MItem* d_items = nullptr;      // the full list
  MItem* d_sub = nullptr;        // a filtered list (some contexts skipped)
  unsigned int* d_counter = nullptr;
  long long scratch_per_cta = 0;
};

struct evr_sg4_multi {
  int n = 0, cshift = 0, transpose = 0;
  std::vector<evr_sg4_ctx*> ctxs;
  std::vector<int> nrhs_v, type, nbuf;  // per context; type and work arrays per point fix the plan
  std::vector<int> group;        // per context: its launch group
  std::vector<int> slot;         // per context: its slot in that group's parameter block
  std::vector<MGroup> groups;    // one, or two when D <= 6 contexts fill a narrow launch of their own;
                                 // each split into launches of at most EVR_PB_LARGE contexts
  std::vector<TermInfo*> d_terms;
  std::vector<double*> d_contrib;
  std::vector<double*> d_part;
  double* d_scratch = nullptr;   // global-scratch slabs, shared by the groups (launched in turn)
  std::vector<KParams> pslot[2]; // parameters bound to fixed vectors (multi_bind), per context
  long long last_launches = 0;
};

void evr::multi_shape(const evr_sg4_multi* m, std::vector<evr_sg4_ctx*>* ctxs, std::vector<int>* nrhs,
                      int* cshift, int* transpose) {
  *ctxs = m->ctxs;
  nrhs->resize(m->n);
  for (int k = 0; k < m->n; ++k) (*nrhs)[k] = (m->nrhs_v[k] >> m->cshift) / m->ctxs[k]->nb0;
  *cshift = m->cshift;
  *transpose = m->transpose;
}

static void free_multi(evr_sg4_multi* m) {
  for (TermInfo* p : m->d_terms) if (p) cudaFree(p);
  for (double* p : m->d_contrib) if (p) cudaFree(p);
  for (double* p : m->d_part) if (p) cudaFree(p);
  for (MGroup& g : m->groups) {
    void* gp[] = {g.d_items, g.d_sub, g.d_counter};
    for (void* q : gp) if (q) cudaFree(q);
  }
  if (m->d_scratch) cudaFree(m->d_scratch);
  delete m;
}

extern "C" int evr_sg4_multi_create(int n, evr_sg4_ctx* const* ctxs, const int* nrhs, int flags,
                                    evr_sg4_multi** out) {
  if (!out) return set_error(EVR_ERR_ARG, "multi_create: NULL output");
  *out = nullptr;
  if (n < 1 || !ctxs || !nrhs) return set_error(EVR_ERR_ARG, "multi_create: NULL argument or n < 1");
  if (flags & ~(EVR_APPLY_TRANSPOSE | EVR_APPLY_COMPLEX)) return set_error(EVR_ERR_ARG, "multi_create: bad flags");
  for (int k = 0; k < n; ++k) {
    if (!ctxs[k] || !ctxs[k]->have_op) return set_error(EVR_ERR_STATE, "multi_create: context %d has no operator", k);
    if (ctxs[k]->streamed)
      return set_error(EVR_ERR_STATE, "multi_create: context %d streams its operator fields (use evr_sg4_hpsi)", k);
    if (nrhs[k] < 1) return set_error(EVR_ERR_ARG, "multi_create: nrhs[%d]=%d < 1", k, nrhs[k]);
    if (ctxs[k]->device != ctxs[0]->device) return set_error(EVR_ERR_ARG, "multi_create: contexts on different devices");
  }
  evr_sg4_multi* m = new evr_sg4_multi();
  m->n = n;
  m->cshift = (flags & EVR_APPLY_COMPLEX) ? 1 : 0;
  m->transpose = (flags & EVR_APPLY_TRANSPOSE) ? 1 : 0;
  m->ctxs.assign(ctxs, ctxs + n);
  m->nrhs_v.resize(n);
  m->type.resize(n);
  m->nbuf.resize(n);
  m->d_terms.assign(n, nullptr);
  m->d_contrib.assign(n, nullptr);
  m->d_part.assign(n, nullptr);
  auto fail = [&](int rc) { free_multi(m); return rc; };
  // Launch groups.  The contexts with D <= 6 run narrow in a launch of their
  // own when their items fill enough waves and other contexts exist;
  // otherwise one launch takes every context, in the geometry of the merged
  // wide plan (wide; narrow if every D <= 6, else mid, once it has enough
  // waves of items).
  std::vector<size_t> n_wide(n);
  for (int k = 0; k < n; ++k) {
    evr_sg4_ctx* c = ctxs[k];
    std::vector<TermInfo> terms;
    std::vector<Item> items;
    std::vector<float> cost;
    long long need = 0;
    plan_work(c, (nrhs[k] * c->nb0) << m->cshift, geo_smem_bytes(0) / 8, terms, items, cost, need);
    n_wide[k] = items.size();
  }
  const int sms = ctxs[0]->num_sms;
  size_t small_items = 0, all_items = 0;
  int dmax = 0, n_small = 0;
  for (int k = 0; k < n; ++k) {
    all_items += n_wide[k];
    dmax = std::max(dmax, ctxs[k]->D);
    if (ctxs[k]->D <= EVR_NARROW_FMAX) {
      small_items += n_wide[k];
      ++n_small;
    }
  }
  m->group.assign(n, 0);
  if (n_small > 0 && n_small < n && choose_geo(EVR_NARROW_FMAX, small_items, sms) == 1) {
    int dbig = 0;
    for (int k = 0; k < n; ++k)
      if (ctxs[k]->D > EVR_NARROW_FMAX) {
        m->group[k] = 1;
        dbig = std::max(dbig, ctxs[k]->D);
      }
    m->groups.resize(2);
    m->groups[0].geo = 1;
    m->groups[1].geo = choose_geo(dbig, all_items - small_items, sms);
  } else {
    m->groups.resize(1);
    m->groups[0].geo = choose_geo(dmax, all_items, sms);
  }
  {  // each group split into launches of at most EVR_PB_LARGE contexts, in context order
    std::vector<MGroup> split;
    std::vector<int> to(n, 0);
    for (size_t gi = 0; gi < m->groups.size(); ++gi) {
      int cnt = 0;
      for (int k = 0; k < n; ++k) {
        if (m->group[k] != (int)gi) continue;
        if (cnt++ % EVR_PB_LARGE == 0) {
          split.emplace_back();
          split.back().geo = m->groups[gi].geo;
        }
        to[k] = (int)split.size() - 1;
      }
    }
    m->groups.swap(split);
    m->group.swap(to);
  }
  m->slot.assign(n, 0);
  for (int k = 0; k < n; ++k) {
    MGroup& g = m->groups[m->group[k]];
    m->slot[k] = (int)g.ctx_of.size();
    g.ctx_of.push_back(k);
  }
  const int ng = (int)m->groups.size();
  // a geometry named by evr_sg4_set_plan on every context of a group is the
  // group's (set_plan keeps the narrow geometry to D <= 6)
  for (int gi = 0; gi < ng; ++gi) {
    int want = -2;
    for (int k = 0; k < n; ++k)
      if (m->group[k] == gi) want = (want == -2 || want == ctxs[k]->geo_override) ? ctxs[k]->geo_override : -1;
    if (want >= 0) m->groups[gi].geo = want;
  }
  std::vector<std::vector<MItem>> all(ng);
  std::vector<std::vector<float>> allcost(ng);
  long long scratch_doubles = 0;
  for (MGroup& g : m->groups) {
    g.smem_doubles = geo_smem_bytes(g.geo) / 8;
    g.grid = geo_ctas(g.geo) * sms;
  }
  for (int k = 0; k < n; ++k) {
    evr_sg4_ctx* c = ctxs[k];
    const int gk = m->group[k];
    MGroup& g = m->groups[gk];
    const int nv = (nrhs[k] * c->nb0) << m->cshift;
    m->nrhs_v[k] = nv;
    m->type[k] = c->type;
    m->nbuf[k] = nbuf_for(c);
    std::vector<TermInfo> terms;
    std::vector<Item> items;
    std::vector<float> cost;
    long long need = 0;
    plan_work(c, nv, g.smem_doubles, terms, items, cost, need);
    if (need > g.smem_doubles) g.scratch_per_cta = std::max(g.scratch_per_cta, need);
    for (size_t q = 0; q < items.size(); ++q) {
      all[gk].push_back(MItem{m->slot[k], items[q].term, items[q].rhs0, 0});
      allcost[gk].push_back(cost[q]);
    }
    if (cudaMalloc(&m->d_terms[k], terms.size() * sizeof(TermInfo)) != cudaSuccess ||
        cudaMemcpy(m->d_terms[k], terms.data(), terms.size() * sizeof(TermInfo), cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMalloc(&m->d_contrib[k], (size_t)c->z.sum_nb * nv * 8) != cudaSuccess ||
        cudaMalloc(&m->d_part[k], (size_t)c->n_chunks * nv * 16) != cudaSuccess) {
      cudaGetLastError();
      return fail(set_error(EVR_ERR_CUDA, "multi_create: device allocation for context %d failed", k));
    }
  }
  for (int gi = 0; gi < ng; ++gi) {
    MGroup& g = m->groups[gi];
    std::vector<int> order(all[gi].size());
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return allcost[gi][a] > allcost[gi][b]; });
    g.sorted.resize(all[gi].size());
    for (size_t q = 0; q < order.size(); ++q) g.sorted[q] = all[gi][order[q]];
    scratch_doubles = std::max(scratch_doubles, g.scratch_per_cta * g.grid);
    const size_t ni = std::max<size_t>(1, g.sorted.size());
    if (cudaMalloc(&g.d_items, ni * sizeof(MItem)) != cudaSuccess ||
        cudaMalloc(&g.d_sub, ni * sizeof(MItem)) != cudaSuccess ||
        cudaMalloc(&g.d_counter, sizeof(unsigned int)) != cudaSuccess ||
        cudaMemcpy(g.d_items, g.sorted.data(), g.sorted.size() * sizeof(MItem), cudaMemcpyHostToDevice) !=
            cudaSuccess) {
      cudaGetLastError();
      return fail(set_error(EVR_ERR_CUDA, "multi_create: device allocation failed"));
    }
  }
  if (scratch_doubles && cudaMalloc(&m->d_scratch, (size_t)scratch_doubles * 8) != cudaSuccess) {
    cudaGetLastError();
    return fail(set_error(EVR_ERR_CUDA, "multi_create: device allocation failed"));
  }
  *out = m;
  return EVR_OK;
}

extern "C" int evr_sg4_multi_groups(const evr_sg4_multi* m, int cap, int* n_groups, int* geo, long long* n_items) {
  if (!m || !n_groups || cap < 0) return set_error(EVR_ERR_ARG, "multi_groups: NULL argument or cap < 0");
  *n_groups = (int)m->groups.size();
  for (size_t g = 0; g < m->groups.size() && (int)g < cap; ++g) {
    if (geo) geo[g] = m->groups[g].geo;
    if (n_items) n_items[g] = (long long)m->groups[g].sorted.size();
  }
  return EVR_OK;
}

extern "C" int evr_sg4_multi_destroy(evr_sg4_multi* m) {
  if (!m) return set_error(EVR_ERR_ARG, "multi_destroy: NULL plan");
  cudaDeviceSynchronize();
  free_multi(m);
  return EVR_OK;
}

// One launch group's merged items: the parameters of its contexts (by
// context) gathered into the group's slots.
static void launch_group(const MGroup& g, const std::vector<KParams>& params, const MItem* items, int n_items,
                         cudaStream_t s) {
  std::vector<KParams> slots(g.ctx_of.size());
  for (size_t j = 0; j < g.ctx_of.size(); ++j) slots[j] = params[g.ctx_of[j]];
  launch_multi(g.geo, g.grid, (size_t)g.smem_doubles * 8, s, slots.data(), (int)slots.size(), items, n_items, 0,
               g.d_counter);
}

extern "C" int evr_sg4_multi_hpsi(evr_sg4_multi* m, const double* const* psi, const long long* ldpsi,
                                  double* const* hpsi, const long long* ldh, const double* E0, const double* Esc,
                                  void* stream) {
  if (!m || !psi || !hpsi || !ldpsi || !ldh) return set_error(EVR_ERR_ARG, "multi_hpsi: NULL argument");
  cudaStream_t s = (cudaStream_t)stream;
  std::vector<KParams> params(m->n);
  int active = 0;
  for (int k = 0; k < m->n; ++k) {
    evr_sg4_ctx* c = m->ctxs[k];
    if (!psi[k]) continue;  // context k is skipped in this call
    if (!c->have_op || c->type != m->type[k] || nbuf_for(c) != m->nbuf[k] || c->streamed)
      return set_error(EVR_ERR_STATE, "multi_hpsi: the operator of context %d changed since multi_create", k);
    if (!hpsi[k] || ldpsi[k] < c->nvec || ldh[k] < c->nvec)
      return set_error(EVR_ERR_ARG, "multi_hpsi: bad output or leading dimension for context %d", k);
    const double e0 = E0 ? E0[k] : 0.0, esc = Esc ? Esc[k] : 1.0;
    if (!(esc != 0.0) || !std::isfinite(esc) || !std::isfinite(e0))
      return set_error(EVR_ERR_ARG, "multi_hpsi: Esc of context %d must be finite and non-zero", k);
    KParams& p = params[k];
    p = make_params(c, m->nrhs_v[k], m->cshift, psi[k], ldpsi[k] << m->cshift, hpsi[k], ldh[k] << m->cshift, 1.0);
    const MGroup& g = m->groups[m->group[k]];
    p.transpose = m->transpose;
    p.smem_doubles = g.smem_doubles;  // the plan's geometry, not the context's own last plan
    p.terms = m->d_terms[k];
    p.contrib = m->d_contrib[k];
    p.gscratch = m->d_scratch;
    p.scratch_per_cta = g.scratch_per_cta;
    ++active;
  }
  if (active == 0) return set_error(EVR_ERR_ARG, "multi_hpsi: every context is skipped");
  int launched = 0;
  for (MGroup& g : m->groups) {  // one after the other: they share the scratch slabs
    const MItem* items = g.d_items;
    int n_items = (int)g.sorted.size();
    if (active < m->n) {  // the sorted list without the skipped contexts
      std::vector<MItem> sub;
      sub.reserve(g.sorted.size());
      for (const MItem& q : g.sorted)
        if (psi[g.ctx_of[q.ctx]]) sub.push_back(q);
      if (!sub.empty())
        CUDA_TRY(cudaMemcpyAsync(g.d_sub, sub.data(), sub.size() * sizeof(MItem), cudaMemcpyHostToDevice, s));
      CUDA_TRY(cudaStreamSynchronize(s));  // `sub` leaves scope
      items = g.d_sub;
      n_items = (int)sub.size();
    }
    if (n_items == 0) continue;
    CUDA_TRY(cudaMemsetAsync(g.d_counter, 0, sizeof(unsigned int), s));
    launch_group(g, params, items, n_items, s);
    CUDA_TRY(cudaGetLastError());
    ++launched;
  }
  for (int k = 0; k < m->n; ++k) {
    if (!psi[k]) continue;
    int rc = launch_reduce(m->ctxs[k], m->d_contrib[k], (double2*)m->d_part[k], m->nrhs_v[k], m->cshift, psi[k],
                           ldpsi[k] << m->cshift, hpsi[k], ldh[k] << m->cshift, E0 ? E0[k] : 0.0,
                           Esc ? Esc[k] : 1.0, s);
    if (rc) return rc;
  }
  m->last_launches = launched + 2LL * active;
  return EVR_OK;
}

// Parameters of every context bound to fixed vectors (psi[k] -> hpsi[k],
// ld = nb0*N, in binding 0 or 1), formed once: multi_launch_bound then
// enqueues kernels and memsets only, so a caller can record it in a CUDA graph
// (the recording keeps the launches' parameter blocks by value).  The same
// parameters, items and kernels as evr_sg4_multi_hpsi with every context
// active, so the same bits.
int evr::multi_bind(evr_sg4_multi* m, int slot, const double* const* psi, double* const* hpsi) {
  if (!m || slot < 0 || slot > 1 || !psi || !hpsi) return set_error(EVR_ERR_ARG, "multi_bind: bad arguments");
  std::vector<KParams> params(m->n);
  for (int k = 0; k < m->n; ++k) {
    evr_sg4_ctx* c = m->ctxs[k];
    if (!psi[k] || !hpsi[k]) return set_error(EVR_ERR_ARG, "multi_bind: NULL vector of context %d", k);
    KParams& p = params[k];
    p = make_params(c, m->nrhs_v[k], m->cshift, psi[k], c->nvec << m->cshift, hpsi[k], c->nvec << m->cshift, 1.0);
    const MGroup& g = m->groups[m->group[k]];
    p.transpose = m->transpose;
    p.smem_doubles = g.smem_doubles;
    p.terms = m->d_terms[k];
    p.contrib = m->d_contrib[k];
    p.gscratch = m->d_scratch;
    p.scratch_per_cta = g.scratch_per_cta;
  }
  m->pslot[slot].swap(params);
  return EVR_OK;
}

int evr::multi_launch_bound(evr_sg4_multi* m, int slot, const double* const* psi, double* const* hpsi,
                            const double* E0, const double* Esc, void* stream) {
  cudaStream_t s = (cudaStream_t)stream;
  if (slot < 0 || slot > 1 || m->pslot[slot].empty())
    return set_error(EVR_ERR_STATE, "multi_launch_bound: binding %d is not set", slot);
  for (MGroup& g : m->groups) {
    CUDA_TRY(cudaMemsetAsync(g.d_counter, 0, sizeof(unsigned int), s));
    launch_group(g, m->pslot[slot], g.d_items, (int)g.sorted.size(), s);
    CUDA_TRY(cudaGetLastError());
  }
  for (int k = 0; k < m->n; ++k) {
    const long long ld = m->ctxs[k]->nvec << m->cshift;
    int rc = launch_reduce(m->ctxs[k], m->d_contrib[k], (double2*)m->d_part[k], m->nrhs_v[k], m->cshift, psi[k], ld,
                           hpsi[k], ld, E0[k], Esc[k], s);
    if (rc) return rc;
  }
  return EVR_OK;
}

extern "C" int evr_sg4_multi_last_launches(const evr_sg4_multi* m, long long* n) {
  if (!m || !n) return set_error(EVR_ERR_ARG, "multi_last_launches: NULL argument");
  *n = m->last_launches;
  return EVR_OK;
}

extern "C" int evr_sg4_hpsi_multi(int n, evr_sg4_ctx* const* ctxs, const int* nrhs, const double* const* psi,
                                  const long long* ldpsi, double* const* hpsi, const long long* ldh, const double* E0,
                                  const double* Esc, int flags, void* stream) {
  evr_sg4_multi* m = nullptr;
  int rc = evr_sg4_multi_create(n, ctxs, nrhs, flags, &m);
  if (rc) return rc;
  rc = evr_sg4_multi_hpsi(m, psi, ldpsi, hpsi, ldh, E0, Esc, stream);
  if (!rc && cudaStreamSynchronize((cudaStream_t)stream) != cudaSuccess)
    rc = set_error(EVR_ERR_CUDA, "hpsi_multi: %s", cudaGetErrorString(cudaGetLastError()));
  if (!rc)
    for (int k = 0; k < n; ++k) ctxs[k]->last_launches = m->last_launches;
  free_multi(m);
  return rc;
}

// ------------------------------------------------------------------------
// A fixed H.psi: one context applied to fixed device buffers (nrhs real
// columns, psi -> hpsi, ld = nb0*N, E0 = 0, Esc = 1), with a plan, work list
// and scratch of its own and its parameter block uploaded once, so a launch
// is kernels only and can be recorded in a CUDA graph (the context's own
// cached plan, which other calls re-plan, is not involved).  Same items and
// arithmetic as evr_sg4_apply, so the same bits.
// ------------------------------------------------------------------------
struct evr::BoundApply {
  evr_sg4_ctx* c = nullptr;
  KParams p{};                  // the plan's parameters (terms, scratch of its own)
  int geo = 0, grid = 0, nrhs_v = 0, n_items = 0;
  TermInfo* d_terms = nullptr;
  MItem* d_items = nullptr;
  unsigned int* d_counter = nullptr;
  double* d_contrib = nullptr;
  double* d_part = nullptr;
  double* d_scratch = nullptr;
  const double* psi = nullptr;
  double* hpsi = nullptr;
  long long ld = 0;
};

// The same work list, geometry and kernel as evr_sg4_apply's plan for
// nrhs columns (plan_sorted), in buffers of its own.
int evr::bound_apply_create(evr_sg4_ctx* c, int nrhs, int transpose, const double* psi, double* hpsi,
                            BoundApply** out) {
  *out = nullptr;
  if (!c || nrhs < 1 || !psi || !hpsi) return set_error(EVR_ERR_ARG, "bound apply: bad arguments");
  if (!c->have_op) return set_error(EVR_ERR_STATE, "bound apply: set_operator was not called");
  if (c->streamed) return set_error(EVR_ERR_STATE, "bound apply: the operator fields are streamed");
  BoundApply* b = new BoundApply();
  b->c = c;
  b->psi = psi;
  b->hpsi = hpsi;
  b->ld = c->nvec;
  b->nrhs_v = nrhs * c->nb0;
  std::vector<TermInfo> terms;
  std::vector<Item> items, sorted;
  long long max_need = 0;
  plan_sorted(c, b->nrhs_v, terms, items, sorted, max_need, b->geo);
  const int smem_doubles = geo_smem_bytes(b->geo) / 8;
  b->grid = geo_ctas(b->geo) * c->num_sms;
  const long long per_cta = max_need > smem_doubles ? max_need : 0;
  auto fail = [&](const char* what) {
    cudaGetLastError();
    bound_apply_destroy(b);
    return set_error(EVR_ERR_CUDA, "bound apply: %s", what);
  };
  if (cudaMalloc(&b->d_terms, terms.size() * sizeof(TermInfo)) != cudaSuccess ||
      cudaMalloc(&b->d_items, std::max<size_t>(1, sorted.size()) * sizeof(MItem)) != cudaSuccess ||
      cudaMalloc(&b->d_counter, sizeof(unsigned int)) != cudaSuccess ||
      cudaMalloc(&b->d_contrib, (size_t)c->z.sum_nb * b->nrhs_v * 8) != cudaSuccess ||
      cudaMalloc(&b->d_part, (size_t)c->n_chunks * b->nrhs_v * 16) != cudaSuccess ||
      (per_cta && cudaMalloc(&b->d_scratch, (size_t)per_cta * b->grid * 8) != cudaSuccess))
    return fail("device allocation failed");
  if (cudaMemcpy(b->d_terms, terms.data(), terms.size() * sizeof(TermInfo), cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(b->d_items, slot0_items(sorted).data(), sorted.size() * sizeof(MItem), cudaMemcpyHostToDevice) !=
          cudaSuccess)
    return fail("upload failed");
  b->n_items = (int)sorted.size();
  KParams p = make_params(c, b->nrhs_v, 0, psi, b->ld, hpsi, b->ld, 1.0);
  p.transpose = transpose ? 1 : 0;
  p.terms = b->d_terms;
  p.smem_doubles = smem_doubles;
  p.contrib = b->d_contrib;
  p.gscratch = b->d_scratch;
  p.scratch_per_cta = per_cta;
  b->p = p;
  *out = b;
  return EVR_OK;
}

void evr::bound_apply_destroy(BoundApply* b) {
  if (!b) return;
  void* ptrs[] = {b->d_terms, b->d_items, b->d_counter, b->d_contrib, b->d_part, b->d_scratch};
  for (void* q : ptrs)
    if (q) cudaFree(q);
  delete b;
}

int evr::bound_apply_launch(BoundApply* b, void* stream) {
  cudaStream_t s = (cudaStream_t)stream;
  CUDA_TRY(cudaMemsetAsync(b->d_counter, 0, sizeof(unsigned int), s));
  launch_single(b->geo, b->grid, (size_t)b->p.smem_doubles * 8, s, b->p, b->d_items, b->n_items, b->d_counter);
  CUDA_TRY(cudaGetLastError());
  return launch_reduce(b->c, b->d_contrib, (double2*)b->d_part, b->nrhs_v, 0, b->psi, b->ld, b->hpsi, b->ld, 0.0,
                       1.0, s);
}

// ------------------------------------------------------------------------
// Two operators of one basis (H0 and mu of a field-driven propagation)
// applied to one complex vector in one persistent launch, up to the chunk
// partials of their ordered accumulations; the caller joins them (and fuses
// its own element-wise update into that join).  The parameter blocks point
// at a vector owned by the pair, so an apply uploads nothing and launches
// two kernels: the merged item list, then the chunk sums of both operators
// (which also rearms the work counter).
// ------------------------------------------------------------------------
struct evr::FieldPair {
  evr_sg4_multi* m = nullptr;
  double* x = nullptr;         // [nrhs][N] complex input
  double2* part = nullptr;     // [2][n_chunks][2 nrhs]
  int grid = 0;
  int nrhs = 1;
  long long N = 0;
  KParams ps[2];               // the pair's parameters (slots 0 and 1 of its one launch group)
};

// Chunk sums of both operators: thread t = (op, chunk, virtual column v),
// op-major, then chunk, then column (nrhs_v = 2 nrhs: re/im of each packet).
__global__ void __launch_bounds__(256) pair_chunks_kernel(const double* __restrict__ contrib0,
                                                          const double* __restrict__ contrib1,
                                                          const long long* __restrict__ chunk_q, long long n_chunks,
                                                          const long long* __restrict__ inv_idx, int nrhs_v,
                                                          double2* __restrict__ part, unsigned int* counter) {
  if (blockIdx.x == 0 && threadIdx.x == 0) *counter = 0u;  // the item kernel before this one has finished
  const long long per = n_chunks * nrhs_v, total = 2 * per;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
       t += (long long)gridDim.x * blockDim.x) {
    const int op = t >= per ? 1 : 0;
    const long long r = t - op * per;
    const long long ch = r / nrhs_v;
    const int v = (int)(r - ch * nrhs_v);
    const double* contrib = op ? contrib1 : contrib0;
    double s = 0.0, c = 0.0;
    chunk_sum(contrib, inv_idx, chunk_q[ch], chunk_q[ch + 1], nrhs_v, v, s, c);
    part[t] = make_double2(s, c);
  }
}

int evr::field_pair_create(evr_sg4_ctx* a, evr_sg4_ctx* b, int transpose, int nrhs, FieldPair** out) {
  *out = nullptr;
  if (!a || !b) return set_error(EVR_ERR_ARG, "field pair: NULL context");
  if (nrhs < 1) return set_error(EVR_ERR_ARG, "field pair: nrhs < 1");
  if (a->N != b->N || a->nb_SG != b->nb_SG || a->z.sum_nb != b->z.sum_nb || a->n_chunks != b->n_chunks)
    return set_error(EVR_ERR_ARG, "field pair: the two operators are on different bases");
  if (a->nb0 != 1 || b->nb0 != 1) return set_error(EVR_ERR_ARG, "field pair: one channel (nb0 = 1) only");
  evr_sg4_ctx* cs[2] = {a, b};
  const int nr[2] = {nrhs, nrhs};
  FieldPair* f = new FieldPair();
  int rc = evr_sg4_multi_create(2, cs, nr, EVR_APPLY_COMPLEX | (transpose ? EVR_APPLY_TRANSPOSE : 0), &f->m);
  if (rc) {
    delete f;
    return rc;
  }
  f->N = a->N;
  f->nrhs = nrhs;
  if (cudaMalloc(&f->x, (size_t)a->N * nrhs * 16) != cudaSuccess ||
      cudaMalloc(&f->part, (size_t)a->n_chunks * 4 * nrhs * sizeof(double2)) != cudaSuccess) {
    cudaGetLastError();
    field_pair_destroy(f);
    return set_error(EVR_ERR_CUDA, "field pair: device allocation failed");
  }
  evr_sg4_multi* m = f->m;
  const MGroup& g = m->groups[0];  // one basis, one launch group: context k in slot k
  KParams* ps = f->ps;
  for (int k = 0; k < 2; ++k) {
    ps[k] = make_params(cs[k], 2 * nrhs, 1, f->x, 2 * a->N, nullptr, 2 * a->N, 1.0);
    ps[k].transpose = m->transpose;
    ps[k].smem_doubles = g.smem_doubles;
    ps[k].terms = m->d_terms[k];
    ps[k].contrib = m->d_contrib[k];
    ps[k].gscratch = m->d_scratch;
    ps[k].scratch_per_cta = g.scratch_per_cta;
  }
  if (cudaMemset(g.d_counter, 0, sizeof(unsigned int)) != cudaSuccess) {
    cudaGetLastError();
    field_pair_destroy(f);
    return set_error(EVR_ERR_CUDA, "field pair: counter reset failed");
  }
  // enough CTAs for every item, so small operators leave SMs to other streams
  f->grid = (int)std::min<size_t>((size_t)g.grid, std::max<size_t>(1, g.sorted.size()));
  *out = f;
  return EVR_OK;
}

void evr::field_pair_destroy(FieldPair* f) {
  if (!f) return;
  if (f->m) free_multi(f->m);
  if (f->x) cudaFree(f->x);
  if (f->part) cudaFree(f->part);
  delete f;
}

int evr::field_pair_apply(FieldPair* f, void* stream) {
  cudaStream_t s = (cudaStream_t)stream;
  evr_sg4_multi* m = f->m;
  evr_sg4_ctx* c = m->ctxs[0];
  const MGroup& g = m->groups[0];
  launch_multi(g.geo, f->grid, (size_t)g.smem_doubles * 8, s, f->ps, 2, g.d_items, (int)g.sorted.size(), 0,
               g.d_counter);
  // 64-thread blocks: the Neumaier sums are FP64 chains, and GB300's FP64
  // pipe (about two operations per clock per SM) wants them on many SMs
  const int nrhs_v = 2 * f->nrhs;
  const long long t1 = c->n_chunks * 2 * nrhs_v;
  const long long b1 = std::max<long long>(1, std::min<long long>((t1 + 63) / 64, 64LL * c->num_sms));
  pair_chunks_kernel<<<(unsigned)b1, 64, 0, s>>>(m->d_contrib[0], m->d_contrib[1], c->d_chunk_q, c->n_chunks,
                                                 c->d_inv_idx, nrhs_v, f->part, g.d_counter);
  CUDA_TRY(cudaGetLastError());
  return EVR_OK;
}

evr::FieldPairView evr::field_pair_view(const FieldPair* f) {
  FieldPairView v;
  const evr_sg4_ctx* c = f->m->ctxs[0];
  v.N = f->N;
  v.n_chunks = c->n_chunks;
  v.nrhs = f->nrhs;
  v.fun_chunk = c->d_fun_chunk;
  v.part = f->part;
  v.x = f->x;
  return v;
}



// ------------------------------------------------------------------------
// diag(H) term by term.  The term operator is B A C (C = RGB basis->grid,
// B = RBGwrho grid->basis, Kronecker products over the modes), and
// A = V + sum of terms f(q) D_i D_j with D_i a 1-D matrix on mode i, so its
// diagonal element at DP index k is
//   sum_q f(q) prod_l P_l[k_l][q_l],  P_l = (B_l M1_l) o (M2_l C_l)^T,
// M1_l = the outer 1-D matrix on mode l (d1GG or d2GG, else I), M2_l the
// inner one: a grid->basis transform of the field f with the "pattern"
// matrices P_l in place of RBGwrho.  Per term: one transform per pattern
// (V; D^2 G_ij terms for type 10, -1/2 each; F2/F1 terms for type 1), the
// weighted result into the contribution buffer, then the ordered
// accumulation of evr_sg4_hpsi.  A few H.psi-equivalents of work instead of
// N/64 H.psi calls on blocks of unit vectors.  Type 10 with Jac or rho (the
// -1/2/(Jac s) factor does not factor per mode), several channels and
// streamed fields keep the unit-vector method.
// ------------------------------------------------------------------------
namespace evr {

struct DiagPat {
  int field;   // 0: V, 1: ones, 2: G(i, j)
  int i, j;    // modes with an outer / inner 1-D matrix (-1: none)
  int pi, pj;  // their pattern sets (1 L1, 2 R1, 3 LR, 4 L2); 0 = E elsewhere
  double coef;
};

__global__ void __launch_bounds__(128) diag_kernel(KParams p, const int* __restrict__ diag_off,
                                                   const DiagPat* __restrict__ pats, int npat,
                                                   const int* __restrict__ order, int nterms, unsigned int* counter) {
  extern __shared__ double smem[];
  __shared__ ItemShared it;
  __shared__ int next;
  for (;;) {
    if (threadIdx.x == 0) next = (int)atomicAdd(counter, 1u);
    __syncthreads();
    const int idx = next;
    __syncthreads();
    if (idx >= nterms) break;
    const int term = order[idx];
    if (threadIdx.x == 0) {
      const TermInfo& T = p.terms[term];
      it.term = term;
      it.rhs0 = 0;
      it.r = 1;
      it.off_nb = T.off_nb;
      it.off_nq = T.off_nq;
      it.nb_t = T.nb;
      it.nq_t = T.nq;
      it.w = T.w;
      const long long need = 3LL * T.nq;
      it.base = (need <= p.smem_doubles) ? smem : p.gscratch + (long long)blockIdx.x * p.scratch_per_cta;
    }
    if (threadIdx.x < p.D) {
      const int i = threadIdx.x;
      const int k = i * p.Lp1 + p.terms[term].l[i];
      it.nb[i] = p.nb_of_l[k];
      it.nq[i] = p.nq_of_l[k];
    }
    __syncthreads();
    if (threadIdx.x == 0) {  // the mode order of the grid->basis passes, as run_item
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
      for (int k = 0; k < p.D; ++k) it.pos[it.ord[k]] = k;
    }
    __syncthreads();
    const int nqt = it.nq_t, nbt = it.nb_t;
    double* A = it.base;
    double* Bf = A + nqt;
    double* acc = A + 2 * nqt;
    for (int e = threadIdx.x; e < nbt; e += blockDim.x) acc[e] = 0.0;
    const long long oq = it.off_nq;
    const long long GD = (long long)p.D * p.D;
    for (int t = 0; t < npat; ++t) {
      const DiagPat pt = pats[t];
      for (int q = threadIdx.x; q < nqt; q += blockDim.x) {
        double f = 1.0;
        if (pt.field == 0) f = p.V[oq + q];
        else if (pt.field == 2) f = p.G[oq * GD + (long long)nqt * (p.D * pt.i + pt.j) + q];
        A[q] = f;
      }
      if (threadIdx.x < p.D) {
        const int l = threadIdx.x;
        const int set = (l == pt.i) ? pt.pi : ((l == pt.j) ? pt.pj : 0);
        it.mo[l][M_GB] = diag_off[(l * p.Lp1 + p.terms[term].l[l]) * 5 + set];
      }
      __syncthreads();
      const double* yb = transform(p, it, false, A, Bf);
      for (int e = threadIdx.x; e < nbt; e += blockDim.x) acc[e] = fma(pt.coef, yb[e], acc[e]);
      __syncthreads();
    }
    store_contrib(p, it, acc);
  }
}

}  // namespace evr

extern "C" int evr_sg4_diagonal(evr_sg4_ctx* c, double* diag, void* stream) {
  if (!c || !diag) return set_error(EVR_ERR_ARG, "diagonal: NULL argument");
  if (!c->have_op) return set_error(EVR_ERR_STATE, "diagonal: set_operator was not called");
  if (c->nb0 > 1 || c->streamed || c->d_Jac || c->d_sqRho || c->n_t1 > 0)
    return evr_sg4_diagonal_by_apply(c, diag, stream);
  cudaStream_t s = (cudaStream_t)stream;
  const int D = c->D;
  std::vector<DiagPat> pats;
  if (c->d_V) pats.push_back(DiagPat{0, -1, -1, 0, 0, 1.0});
  if (c->type == 1) {
    for (int i = 0; i < D; ++i)
      if (c->F2[i * D + i] != 0.0) pats.push_back(DiagPat{1, i, -1, 4, 0, c->F2[i * D + i]});
    for (int i = 0; i < D; ++i)
      for (int j = i + 1; j < D; ++j)
        if (c->F2[i * D + j] != 0.0) pats.push_back(DiagPat{1, i, j, 1, 1, c->F2[i * D + j]});
    for (int i = 0; i < D; ++i)
      if (c->F1[i] != 0.0) pats.push_back(DiagPat{1, i, -1, 1, 0, c->F1[i]});
  } else if (c->type == 10) {
    for (int i = 0; i < D; ++i)
      for (int j = 0; j < D; ++j) {
        if (!c->d_G && i != j) continue;
        pats.push_back(DiagPat{c->d_G ? 2 : 1, i, j, i == j ? 3 : 1, 2, -0.5});
      }
  }
  if (pats.empty()) {  // the zero operator
    CUDA_TRY(cudaMemsetAsync(diag, 0, (size_t)c->N * 8, s));
    return EVR_OK;
  }
  // terms by decreasing grid size (the persistent CTAs then end balanced)
  std::vector<int> order(c->nb_SG);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return c->terms[a].nq > c->terms[b].nq; });
  // 45 KB of dynamic shared memory per CTA: with the kernel's static block it
  // stays within the 48 KB a launch may take without an attribute
  const int smem_doubles = 5760;
  const int grid = 4 * c->num_sms;  // four resident per SM (registers)
  const long long per_cta = 3LL * c->z.max_nq > smem_doubles ? 3LL * c->z.max_nq : 0;
  std::vector<TermInfo> terms = c->terms;
  for (TermInfo& T : terms) T.r = 1;
  double *d_contrib = nullptr, *d_part = nullptr, *d_scratch = nullptr;
  DiagPat* d_pats = nullptr;
  int* d_order = nullptr;
  TermInfo* d_terms = nullptr;
  unsigned int* d_counter = nullptr;
  auto cleanup = [&]() {
    void* ptrs[] = {d_contrib, d_part, d_scratch, d_pats, d_order, d_terms, d_counter};
    for (void* q : ptrs)
      if (q) cudaFree(q);
  };
  if (cudaMalloc(&d_contrib, (size_t)c->z.sum_nb * 8) != cudaSuccess ||
      cudaMalloc(&d_part, (size_t)c->n_chunks * 16) != cudaSuccess ||
      (per_cta && cudaMalloc(&d_scratch, (size_t)per_cta * grid * 8) != cudaSuccess) ||
      cudaMalloc(&d_pats, pats.size() * sizeof(DiagPat)) != cudaSuccess ||
      cudaMalloc(&d_order, order.size() * sizeof(int)) != cudaSuccess ||
      cudaMalloc(&d_terms, terms.size() * sizeof(TermInfo)) != cudaSuccess ||
      cudaMalloc(&d_counter, sizeof(unsigned int)) != cudaSuccess) {
    cudaGetLastError();
    cleanup();
    return set_error(EVR_ERR_ALLOC, "diagonal: device allocation failed");
  }
  cudaMemcpyAsync(d_pats, pats.data(), pats.size() * sizeof(DiagPat), cudaMemcpyHostToDevice, s);
  cudaMemcpyAsync(d_order, order.data(), order.size() * sizeof(int), cudaMemcpyHostToDevice, s);
  cudaMemcpyAsync(d_terms, terms.data(), terms.size() * sizeof(TermInfo), cudaMemcpyHostToDevice, s);
  cudaMemsetAsync(d_counter, 0, sizeof(unsigned int), s);
  KParams p = make_params(c, 1, 0, diag, c->N, diag, c->N, 1.0);
  p.terms = d_terms;
  p.smem_doubles = smem_doubles;
  p.gscratch = d_scratch;
  p.scratch_per_cta = per_cta;
  p.contrib = d_contrib;
  p.split = 0;
  diag_kernel<<<grid, 128, (size_t)smem_doubles * 8, s>>>(p, c->d_diag_off, d_pats, (int)pats.size(), d_order,
                                                          (int)c->nb_SG, d_counter);
  cudaError_t e = cudaGetLastError();
  int rc = e == cudaSuccess ? launch_reduce(c, d_contrib, (double2*)d_part, 1, 0, diag, c->N, diag, c->N, 0.0, 1.0, s)
                            : set_error(EVR_ERR_CUDA, "diagonal: %s", cudaGetErrorString(e));
  if (!rc && cudaStreamSynchronize(s) != cudaSuccess) rc = set_error(EVR_ERR_CUDA, "diagonal: kernel failed");
  cleanup();
  return rc;
}

// ------------------------------------------------------------------------
// Plan knobs and the autotuner (the counterpart of Tune_SG4threads_HPsi,
// SRC/sub_main/vib.f90:2013-2123, which times H.psi for each OpenMP thread
// count and keeps the fastest).  The knobs of a work plan are the launch
// geometry (wide, narrow, mid: CTAs per SM against shared memory and
// registers per item), the most right-hand sides one work item carries
// (reuse of the 1-D matrices and operator fields against the number and
// balance of items) and the thread mapping of the mode passes (one thread
// per fibre, per output element, or chosen per pass).  None of them changes
// the arithmetic of a term and right-hand side, so results are the same bits
// for every setting.  The tuner times H.psi for each candidate on the
// caller's block size and keeps the fastest, and records it in a JSON file
// keyed by the shape of the workload, so later runs apply it without timing.
// ------------------------------------------------------------------------
extern "C" int evr_sg4_set_plan(evr_sg4_ctx* c, int geo, int rmax, int split) {
  if (!c) return set_error(EVR_ERR_ARG, "set_plan: NULL context");
  if (geo < -1 || geo > 2) return set_error(EVR_ERR_ARG, "set_plan: geometry %d not in {-1, 0, 1, 2}", geo);
  if (geo == 1 && c->D > EVR_NARROW_FMAX)
    return set_error(EVR_ERR_ARG, "set_plan: the narrow geometry takes D <= %d (D = %d)", EVR_NARROW_FMAX, c->D);
  if (rmax == 0) rmax = EVR_AUTO_RMAX;
  if (split == -1) split = EVR_AUTO_SPLIT;
  if (rmax < 1 || rmax > 32) return set_error(EVR_ERR_ARG, "set_plan: rmax %d not in [1, 32]", rmax);
  if (split < 0 || split > 2) return set_error(EVR_ERR_ARG, "set_plan: split %d not in {0, 1, 2}", split);
  c->geo_override = geo;
  c->rmax = rmax;
  c->split = split;
  c->items_nrhs = -1;
  return EVR_OK;
}

extern "C" int evr_sg4_get_plan(const evr_sg4_ctx* c, int* geo, int* rmax, int* split) {
  if (!c || !geo || !rmax || !split) return set_error(EVR_ERR_ARG, "get_plan: NULL argument");
  *geo = c->geo_override;
  *rmax = c->rmax;
  *split = c->split;
  return EVR_OK;
}

namespace evr {

// cache key of a workload shape
static std::string tune_key(const evr_sg4_ctx* c, int nrhs, int flags) {
  char k[160];
  snprintf(k, sizeof(k), "D%d_L%d_LB%d_T%d_NB0%d_N%lld_R%d_C%d_G%d", c->D, c->L, c->LB, c->type, c->nb0, c->N, nrhs,
           (flags & EVR_APPLY_COMPLEX) ? 1 : 0, c->d_G ? 1 : 0);
  return k;
}

struct TuneEntry {
  int geo = -1, rmax = EVR_AUTO_RMAX, split = EVR_AUTO_SPLIT;
  double ms = 0.0, default_ms = 0.0;
};

// The cache: one JSON object, one entry per line,
//   "key": {"geo": g, "rmax": r, "split": s, "ms": t, "default_ms": t0},
static void tune_cache_read(const char* path, std::vector<std::pair<std::string, TuneEntry>>& out) {
  out.clear();
  FILE* f = fopen(path, "r");
  if (!f) return;
  char line[512];
  while (fgets(line, sizeof(line), f)) {
    char key[200];
    TuneEntry e;
    if (sscanf(line, " \"%199[^\"]\": {\"geo\": %d, \"rmax\": %d, \"split\": %d, \"ms\": %lf, \"default_ms\": %lf", key,
               &e.geo, &e.rmax, &e.split, &e.ms, &e.default_ms) == 6)
      out.emplace_back(key, e);
  }
  fclose(f);
}

static int tune_cache_write(const char* path, const std::vector<std::pair<std::string, TuneEntry>>& in) {
  const std::string tmp = std::string(path) + ".tmp";
  FILE* f = fopen(tmp.c_str(), "w");
  if (!f) return set_error(EVR_ERR_ARG, "tune: cannot write the cache %s", path);
  fprintf(f, "{\n");
  for (size_t k = 0; k < in.size(); ++k) {
    const TuneEntry& e = in[k].second;
    fprintf(f, "  \"%s\": {\"geo\": %d, \"rmax\": %d, \"split\": %d, \"ms\": %.6f, \"default_ms\": %.6f}%s\n",
            in[k].first.c_str(), e.geo, e.rmax, e.split, e.ms, e.default_ms, k + 1 < in.size() ? "," : "");
  }
  fprintf(f, "}\n");
  fclose(f);
  if (rename(tmp.c_str(), path) != 0) return set_error(EVR_ERR_ARG, "tune: cannot replace the cache %s", path);
  return EVR_OK;
}

}  // namespace evr

// the geometry the automatic plan picks for this block (geo_override = -1)
static int auto_geo_of(evr_sg4_ctx* c, int nrhs, int flags) {
  const int keep = c->geo_override;
  c->geo_override = -1;
  std::vector<TermInfo> terms;
  std::vector<Item> items, sorted;
  long long need = 0;
  int geo = 0;
  plan_sorted(c, (nrhs * c->nb0) << ((flags & EVR_APPLY_COMPLEX) ? 1 : 0), terms, items, sorted, need, geo);
  c->geo_override = keep;
  return geo;
}

extern "C" int evr_sg4_tune_plan(evr_sg4_ctx* c, int nrhs, int flags, const char* cache_path, evr_tune_result* res) {
  if (!c || nrhs < 1) return set_error(EVR_ERR_ARG, "tune: NULL context or nrhs < 1");
  if (!c->have_op) return set_error(EVR_ERR_STATE, "tune: set_operator was not called");
  if (flags & ~EVR_APPLY_COMPLEX) return set_error(EVR_ERR_ARG, "tune: flags may only hold EVR_APPLY_COMPLEX");
  const std::string key = tune_key(c, nrhs, flags);
  std::vector<std::pair<std::string, TuneEntry>> cache;
  if (cache_path) {
    tune_cache_read(cache_path, cache);
    for (const auto& kv : cache)
      if (kv.first == key) {
        int rc = evr_sg4_set_plan(c, kv.second.geo, kv.second.rmax, kv.second.split);
        if (rc) return rc;
        if (res) *res = evr_tune_result{kv.second.geo, kv.second.rmax, kv.second.split, kv.second.ms,
                                        kv.second.default_ms, 1};
        return EVR_OK;
      }
  }
  const size_t n = (size_t)c->nvec * nrhs * ((flags & EVR_APPLY_COMPLEX) ? 2 : 1);
  double *psi = nullptr, *out = nullptr;
  void* flush = nullptr;  // written before every timed call: each H.psi starts from a cold L2, as in use
  const size_t flush_bytes = (size_t)256 << 20;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  const int keep_geo = c->geo_override, keep_rmax = c->rmax, keep_split = c->split;
  auto cleanup = [&]() {
    if (psi) cudaFree(psi);
    if (out) cudaFree(out);
    if (flush) cudaFree(flush);
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
  };
  if (cudaMalloc(&psi, n * 8) != cudaSuccess || cudaMalloc(&out, n * 8) != cudaSuccess ||
      cudaMalloc(&flush, flush_bytes) != cudaSuccess ||
      cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) {
    cudaGetLastError();
    cleanup();
    return set_error(EVR_ERR_CUDA, "tune: allocation failed");
  }
  {  // deterministic test vectors: a linear congruential sequence in [-1, 1)
    std::vector<double> h(n);
    unsigned long long st = 0x9E3779B97F4A7C15ull;
    for (size_t k = 0; k < n; ++k) {
      st = st * 6364136223846793005ull + 1442695040888963407ull;
      h[k] = (double)(st >> 11) * (2.0 / 9007199254740992.0) - 1.0;
    }
    if (cudaMemcpy(psi, h.data(), n * 8, cudaMemcpyHostToDevice) != cudaSuccess) {
      cleanup();
      return set_error(EVR_ERR_CUDA, "tune: upload failed");
    }
  }
  // time one plan: one untimed H.psi (plans the items), then the best of three
  auto time_plan = [&](int geo, int rmax, int split, double* ms_out) -> int {
    int rc = evr_sg4_set_plan(c, geo, rmax, split);
    if (!rc) rc = evr_sg4_apply(c, flags, nrhs, psi, c->nvec, out, c->nvec, 0.0, 1.0, nullptr);
    double best = 1e300;
    for (int rep = 0; rep < 3 && !rc; ++rep) {
      float ms = 0.f;
      cudaMemsetAsync(flush, rep, flush_bytes, 0);
      cudaEventRecord(e0, 0);
      rc = evr_sg4_apply(c, flags, nrhs, psi, c->nvec, out, c->nvec, 0.0, 1.0, nullptr);
      cudaEventRecord(e1, 0);
      if (!rc && (cudaEventSynchronize(e1) != cudaSuccess || cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess))
        rc = set_error(EVR_ERR_CUDA, "tune: timing failed");
      best = std::min(best, (double)ms);
    }
    *ms_out = best;
    return rc;
  };
  TuneEntry best;
  int rc = time_plan(-1, EVR_AUTO_RMAX, EVR_AUTO_SPLIT, &best.default_ms);  // the automatic plan first
  if (!rc) {
    best.ms = best.default_ms;
    best.geo = auto_geo_of(c, nrhs, flags);
    std::vector<int> geos = {0, 2};
    if (c->D <= EVR_NARROW_FMAX) geos.push_back(1);
    for (int geo : geos)
      for (int rmax : {4, 8, 16, 32})
        for (int split : {0, 1, 2}) {
          double ms = 0.0;
          if ((rc = time_plan(geo, rmax, split, &ms))) break;
          if (ms < 0.99 * best.ms) {  // a candidate must beat the best so far by more than timing noise
            best.ms = ms;
            best.geo = geo;
            best.rmax = rmax;
            best.split = split;
          }
        }
  }
  // confirmation: the minimum over many candidates favours a lucky timing, so
  // the winner and the automatic plan are timed again, alternately, five
  // times each; the winner stays only if its median is more than 1 % faster
  if (!rc && !(best.geo == -1 || (best.rmax == EVR_AUTO_RMAX && best.split == EVR_AUTO_SPLIT &&
                                   best.geo == auto_geo_of(c, nrhs, flags)))) {
    std::vector<double> ta, tb;
    for (int k = 0; k < 5 && !rc; ++k) {
      double ms = 0.0;
      if (!(rc = time_plan(-1, EVR_AUTO_RMAX, EVR_AUTO_SPLIT, &ms))) ta.push_back(ms);
      if (!rc && !(rc = time_plan(best.geo, best.rmax, best.split, &ms))) tb.push_back(ms);
    }
    if (!rc) {
      std::sort(ta.begin(), ta.end());
      std::sort(tb.begin(), tb.end());
      if (!(tb[2] < 0.99 * ta[2])) {
        best.geo = auto_geo_of(c, nrhs, flags);
        best.rmax = EVR_AUTO_RMAX;
        best.split = EVR_AUTO_SPLIT;
        best.ms = ta[2];
      } else {
        best.ms = tb[2];
      }
      best.default_ms = ta[2];
    }
  }
  cleanup();
  if (rc) {
    evr_sg4_set_plan(c, keep_geo, keep_rmax, keep_split);
    return rc;
  }
  if ((rc = evr_sg4_set_plan(c, best.geo, best.rmax, best.split))) return rc;
  if (cache_path) {
    cache.emplace_back(key, best);
    if ((rc = tune_cache_write(cache_path, cache))) return rc;
  }
  if (res) *res = evr_tune_result{best.geo, best.rmax, best.split, best.ms, best.default_ms, 0};
  return EVR_OK;
}

extern "C" int evr_sg4_tune(evr_sg4_ctx* c, int nrhs, int flags, int* best_rmax, double* best_ms) {
  evr_tune_result r;
  int rc = evr_sg4_tune_plan(c, nrhs, flags, nullptr, &r);
  if (rc) return rc;
  if (best_rmax) *best_rmax = r.rmax;
  if (best_ms) *best_ms = r.ms;
  return EVR_OK;
}
