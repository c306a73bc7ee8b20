// sg4_solvers.cu -- the callers of the SG4 H.psi on the device: block
// Davidson (sub_propagation_Davidson, SRC/sub_propagation/
// sub_module_Davidson.f90:59-767) with the exact diagonal as preconditioner,
// Chebyshev propagation (march_cheby; single context, replayed from a CUDA
// graph at fixed order, and many contexts in lock-step), and field-driven
// RK4 with the adjoint optimal-control gradient (march_RK4_field, fcn_field,
// build_field).  Host C++ drives the iterations; every vector operation and
// every H.psi stays on the GPU (cuBLAS DGEMM for the small dense products of
// the Davidson subspace), only m x m projected matrices and scalars go to
// the host.
#include <cublas_v2.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "evr_sg4.h"
#include "sg4_internal.h"
#include "sg4_reduce.cuh"

namespace evr {

#define CUDA_TRY_S(call)                                                                        \
  do {                                                                                          \
    cudaError_t e_ = (call);                                                                    \
    if (e_ != cudaSuccess)                                                                      \
      return set_error(EVR_ERR_CUDA, "%s:%d %s: %s", __FILE__, __LINE__, #call, cudaGetErrorString(e_)); \
  } while (0)
#define CUBLAS_TRY(call)                                                                        \
  do {                                                                                          \
    cublasStatus_t s_ = (call);                                                                 \
    if (s_ != CUBLAS_STATUS_SUCCESS)                                                            \
      return set_error(EVR_ERR_CUDA, "%s:%d %s: cuBLAS status %d", __FILE__, __LINE__, #call, (int)s_); \
  } while (0)

// e_{n0 + j} in column j (N x nb, ld N)
__global__ void unit_block_kernel(double* X, long long N, int nb, long long n0) {
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < N * nb;
       e += (long long)gridDim.x * blockDim.x) {
    const long long j = e / N, n = e - j * N;
    X[e] = (n == n0 + j) ? 1.0 : 0.0;
  }
}

__global__ void take_diag_kernel(const double* HX, long long N, int nb, long long n0, double* diag) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j < nb) diag[n0 + j] = HX[(long long)j * N + n0 + j];
}

// Y = 0.5 * (A + B)
__global__ void average_kernel(double* Y, const double* A, const double* B, long long n) {
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x)
    Y[e] = 0.5 * (A[e] + B[e]);
}

// R(:,k) -= theta_k X(:,k);  then the Davidson correction
// T(:,k) = R(:,k) / (theta_k - diag) (or R when no diagonal is given)
__global__ void residual_kernel(double* R, const double* X, const double* theta, long long N, int nev) {
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < N * nev;
       e += (long long)gridDim.x * blockDim.x) {
    const int k = (int)(e / N);
    R[e] = fma(-theta[k], X[e], R[e]);
  }
}

__global__ void precond_kernel(double* T, const double* R, const double* diag, const double* theta,
                               const int* cols, long long N, int nnew) {
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < N * nnew;
       e += (long long)gridDim.x * blockDim.x) {
    const int j = (int)(e / N);
    const long long n = e - (long long)j * N;
    const int k = cols[j];
    double r = R[(long long)k * N + n];
    if (diag) {
      double den = theta[k] - diag[n];
      if (fabs(den) < 1e-8) den = den < 0 ? -1e-8 : 1e-8;
      r = r / den;
    }
    T[e] = r;
  }
}

// Jacobi eigen-decomposition of a small symmetric matrix (row-major, n x n):
// eigenvalues ascending in w, eigenvectors as columns of Z (row-major).
static void jacobi_eigen(int n, std::vector<double> A, std::vector<double>& w, std::vector<double>& Z) {
  Z.assign((size_t)n * n, 0.0);
  for (int i = 0; i < n; ++i) Z[(size_t)i * n + i] = 1.0;
  for (int sweep = 0; sweep < 100; ++sweep) {
    double off = 0.0, tot = 0.0;
    for (int i = 0; i < n; ++i)
      for (int j = 0; j < n; ++j) {
        double a = A[(size_t)i * n + j] * A[(size_t)i * n + j];
        tot += a;
        if (i != j) off += a;
      }
    if (off <= 1e-32 * tot || off == 0.0) break;
    for (int p = 0; p < n - 1; ++p)
      for (int q = p + 1; q < n; ++q) {
        const double apq = A[(size_t)p * n + q];
        if (apq == 0.0) continue;
        const double app = A[(size_t)p * n + p], aqq = A[(size_t)q * n + q];
        const double theta = (aqq - app) / (2.0 * apq);
        const double t = (theta >= 0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
        const double c = 1.0 / std::sqrt(t * t + 1.0), s = t * c;
        for (int k = 0; k < n; ++k) {  // A <- J^T A J
          const double akp = A[(size_t)k * n + p], akq = A[(size_t)k * n + q];
          A[(size_t)k * n + p] = c * akp - s * akq;
          A[(size_t)k * n + q] = s * akp + c * akq;
        }
        for (int k = 0; k < n; ++k) {
          const double apk = A[(size_t)p * n + k], aqk = A[(size_t)q * n + k];
          A[(size_t)p * n + k] = c * apk - s * aqk;
          A[(size_t)q * n + k] = s * apk + c * aqk;
        }
        for (int k = 0; k < n; ++k) {
          const double zkp = Z[(size_t)k * n + p], zkq = Z[(size_t)k * n + q];
          Z[(size_t)k * n + p] = c * zkp - s * zkq;
          Z[(size_t)k * n + q] = s * zkp + c * zkq;
        }
      }
  }
  std::vector<int> idx(n);
  for (int i = 0; i < n; ++i) idx[i] = i;
  std::sort(idx.begin(), idx.end(), [&](int a, int b) { return A[(size_t)a * n + a] < A[(size_t)b * n + b]; });
  std::vector<double> Zs((size_t)n * n);
  w.resize(n);
  for (int k = 0; k < n; ++k) {
    w[k] = A[(size_t)idx[k] * n + idx[k]];
    for (int i = 0; i < n; ++i) Zs[(size_t)i * n + k] = Z[(size_t)i * n + idx[k]];
  }
  Z.swap(Zs);
}

struct DevBuf {
  double* p = nullptr;
  ~DevBuf() {
    if (p) cudaFree(p);
  }
};

// HX = H_s X for a block (H_s = H, or (H + H^T)/2 when symmetrize)
static int apply_hs(evr_sg4_ctx* c, long long N, int nb, const double* X, double* HX, double* tmp, bool symmetrize,
                    cudaStream_t s) {
  int rc = evr_sg4_apply(c, 0, nb, X, N, HX, N, 0.0, 1.0, s);
  if (rc) return rc;
  if (symmetrize) {
    rc = evr_sg4_apply(c, EVR_APPLY_TRANSPOSE, nb, X, N, tmp, N, 0.0, 1.0, s);
    if (rc) return rc;
    average_kernel<<<256, 256, 0, s>>>(HX, HX, tmp, N * nb);
    CUDA_TRY_S(cudaGetLastError());
  }
  return EVR_OK;
}

}  // namespace evr

using namespace evr;

extern "C" int evr_sg4_diagonal_by_apply(evr_sg4_ctx* c, double* diag, void* stream) {
  if (!c || !diag) return set_error(EVR_ERR_ARG, "diagonal: NULL argument");
  long long sz[8];
  evr_sg4_ctx_sizes(c, sz);
  const long long N = sz[0];
  const int nb = 64;
  cudaStream_t s = (cudaStream_t)stream;
  DevBuf X, HX;
  CUDA_TRY_S(cudaMalloc(&X.p, (size_t)N * nb * 8));
  CUDA_TRY_S(cudaMalloc(&HX.p, (size_t)N * nb * 8));
  for (long long n0 = 0; n0 < N; n0 += nb) {
    const int m = (int)std::min<long long>(nb, N - n0);
    unit_block_kernel<<<256, 256, 0, s>>>(X.p, N, m, n0);
    int rc = evr_sg4_apply(c, 0, m, X.p, N, HX.p, N, 0.0, 1.0, s);
    if (rc) return rc;
    take_diag_kernel<<<1, 64, 0, s>>>(HX.p, N, m, n0, diag);
  }
  CUDA_TRY_S(cudaGetLastError());
  CUDA_TRY_S(cudaStreamSynchronize(s));
  return EVR_OK;
}

// w *= 1/nrm when nrm > tol (the new direction survives), else w = 0 (it is
// dropped; the Davidson basis keeps a zero column in that slot)
__global__ void dav_scale_or_drop_kernel(double* w, long long N, const double* nrm, double tol, int* alive) {
  const double r = *nrm;
  const bool keep = r > tol;
  const double f = keep ? 1.0 / r : 0.0;
  if (blockIdx.x == 0 && threadIdx.x == 0) *alive = keep ? 1 : 0;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < N; e += (long long)gridDim.x * blockDim.x)
    w[e] *= f;
}

// dst(:, m + j) = src(:, j), j < ncols, with m read from the device
__global__ void dav_place_kernel(const double* src, double* dst, long long N, int ncols, const int* m_dev) {
  const long long off = (long long)(*m_dev) * N;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < N * ncols;
       e += (long long)gridDim.x * blockDim.x)
    dst[off + e] = src[e];
}

namespace evr {

// Parameters of one Davidson phase, written by the host into pinned memory
// before the phase runs and copied to the device as the phase's first step
// (a node of its graph): the Ritz coefficients Y (mmax x nev, zero rows for
// unused slots), the Ritz values, the slot where new directions go and the
// residual columns to expand.
struct DavParams {
  int m;
  int ncols;
  int pad[2];
  // followed by: int cols[blk] (padded to 8 bytes), double theta[nev], double Y[mmax*nev]
};

struct DavState {
  evr_sg4_ctx* c = nullptr;
  cublasHandle_t h = nullptr;
  cudaStream_t s = nullptr;
  long long N = 0;
  int nev = 0, blk = 0, mmax = 0;
  bool sym = false;
  const double* diag = nullptr;
  double *V = nullptr, *HV = nullptr, *X = nullptr, *R = nullptr, *W = nullptr, *HW = nullptr, *tmp = nullptr;
  double *Tt = nullptr, *T = nullptr, *cv = nullptr, *nrm = nullptr;
  unsigned char* dparams = nullptr;  // device copy of the parameter block
  unsigned char* hparams = nullptr;  // pinned
  size_t params_bytes = 0;
  double* h_T = nullptr;             // pinned: mmax x mmax
  double* h_nrm = nullptr;           // pinned: nev residual norms, then blk norms of new directions
  int* d_alive = nullptr;
  int* h_alive = nullptr;            // pinned: blk
  int* dm() const { return (int*)dparams; }
  int* dcols() const { return (int*)(dparams + sizeof(DavParams)); }
  size_t cols_bytes() const { return ((size_t)blk * sizeof(int) + 7) / 8 * 8; }
  double* dtheta() const { return (double*)(dparams + sizeof(DavParams) + cols_bytes()); }
  double* dY() const { return dtheta() + nev; }
  int* hcols() const { return (int*)(hparams + sizeof(DavParams)); }
  double* htheta() const { return (double*)(hparams + sizeof(DavParams) + cols_bytes()); }
  double* hY() const { return htheta() + nev; }
};

static int ew_blocks(long long n) { return (int)std::max<long long>(1, std::min<long long>((n + 255) / 256, 1024)); }

// Ritz vectors X = V Y, R = HV Y - X theta and the residual norms (into pinned
// memory).  Fixed sizes (all mmax slots; unused slots are zero columns with
// zero rows of Y), so one recorded graph serves every iteration.
static int dav_phase_ritz(DavState& d, cudaStream_t s) {
  const double one = 1.0, zero = 0.0;
  const int N = (int)d.N;
  CUBLAS_TRY(cublasSetStream(d.h, s));
  CUDA_TRY_S(cudaMemcpyAsync(d.dparams, d.hparams, d.params_bytes, cudaMemcpyHostToDevice, s));
  CUBLAS_TRY(cublasDgemm(d.h, CUBLAS_OP_N, CUBLAS_OP_N, N, d.nev, d.mmax, &one, d.V, N, d.dY(), d.mmax, &zero, d.X, N));
  CUBLAS_TRY(cublasDgemm(d.h, CUBLAS_OP_N, CUBLAS_OP_N, N, d.nev, d.mmax, &one, d.HV, N, d.dY(), d.mmax, &zero, d.R, N));
  residual_kernel<<<256, 256, 0, s>>>(d.R, d.X, d.dtheta(), d.N, d.nev);
  CUDA_TRY_S(cudaGetLastError());
  CUBLAS_TRY(cublasSetPointerMode(d.h, CUBLAS_POINTER_MODE_DEVICE));
  for (int j = 0; j < d.nev; ++j) {
    cublasStatus_t st = cublasDnrm2(d.h, N, d.R + (size_t)j * N, 1, d.nrm + j);
    if (st != CUBLAS_STATUS_SUCCESS) {
      cublasSetPointerMode(d.h, CUBLAS_POINTER_MODE_HOST);
      return set_error(EVR_ERR_CUDA, "davidson: cublasDnrm2 status %d", (int)st);
    }
  }
  CUBLAS_TRY(cublasSetPointerMode(d.h, CUBLAS_POINTER_MODE_HOST));
  CUDA_TRY_S(cudaMemcpyAsync(d.h_nrm, d.nrm, (size_t)d.nev * 8, cudaMemcpyDeviceToHost, s));
  return EVR_OK;
}

// Expansion by nw new directions W: the Davidson correction of the residual
// columns `cols` (precond) or the caller's block as given, orthonormalised
// against V (classical Gram-Schmidt, twice) and among themselves (modified
// Gram-Schmidt, two passes per column; a direction whose norm falls below
// 1e-10 is dropped, left as a zero column), placed in slots m..m+nw-1, H_s
// applied, and the projected matrix T = V^T HV (all mmax slots) copied to
// pinned memory with the survivor flags.  Every size is fixed for a given nw.
template <class A>
static int dav_phase_expand(DavState& d, int nw, bool precond, cudaStream_t s, A&& apply) {
  const double one = 1.0, zero = 0.0, mone = -1.0;
  const int N = (int)d.N;
  CUBLAS_TRY(cublasSetStream(d.h, s));
  CUDA_TRY_S(cudaMemcpyAsync(d.dparams, d.hparams, d.params_bytes, cudaMemcpyHostToDevice, s));
  if (precond) {
    precond_kernel<<<256, 256, 0, s>>>(d.W, d.R, d.diag, d.dtheta(), d.dcols(), d.N, nw);
    CUDA_TRY_S(cudaGetLastError());
  }
  for (int pass = 0; pass < 2; ++pass) {  // against V (unused slots are zero)
    CUBLAS_TRY(cublasDgemm(d.h, CUBLAS_OP_T, CUBLAS_OP_N, d.mmax, nw, N, &one, d.V, N, d.W, N, &zero, d.Tt, d.mmax));
    CUBLAS_TRY(cublasDgemm(d.h, CUBLAS_OP_N, CUBLAS_OP_N, N, nw, d.mmax, &mone, d.V, N, d.Tt, d.mmax, &one, d.W, N));
  }
  for (int j = 0; j < nw; ++j) {
    double* wj = d.W + (size_t)j * N;
    for (int pass = 0; pass < 2 && j > 0; ++pass) {
      CUBLAS_TRY(cublasDgemv(d.h, CUBLAS_OP_T, N, j, &one, d.W, N, wj, 1, &zero, d.cv, 1));
      CUBLAS_TRY(cublasDgemv(d.h, CUBLAS_OP_N, N, j, &mone, d.W, N, d.cv, 1, &one, wj, 1));
    }
    CUBLAS_TRY(cublasSetPointerMode(d.h, CUBLAS_POINTER_MODE_DEVICE));
    cublasStatus_t st = cublasDnrm2(d.h, N, wj, 1, d.nrm + d.nev + j);
    CUBLAS_TRY(cublasSetPointerMode(d.h, CUBLAS_POINTER_MODE_HOST));
    if (st != CUBLAS_STATUS_SUCCESS) return set_error(EVR_ERR_CUDA, "davidson: cublasDnrm2 status %d", (int)st);
    dav_scale_or_drop_kernel<<<ew_blocks(d.N), 256, 0, s>>>(wj, d.N, d.nrm + d.nev + j, 1e-10, d.d_alive + j);
  }
  dav_place_kernel<<<ew_blocks(d.N * nw), 256, 0, s>>>(d.W, d.V, d.N, nw, d.dm());
  CUDA_TRY_S(cudaGetLastError());
  int rc = apply(nw, s);
  if (rc) return rc;
  dav_place_kernel<<<ew_blocks(d.N * nw), 256, 0, s>>>(d.HW, d.HV, d.N, nw, d.dm());
  CUDA_TRY_S(cudaGetLastError());
  CUBLAS_TRY(cublasDgemm(d.h, CUBLAS_OP_T, CUBLAS_OP_N, d.mmax, d.mmax, N, &one, d.V, N, d.HV, N, &zero, d.T, d.mmax));
  CUDA_TRY_S(cudaMemcpyAsync(d.h_T, d.T, (size_t)d.mmax * d.mmax * 8, cudaMemcpyDeviceToHost, s));
  CUDA_TRY_S(cudaMemcpyAsync(d.h_alive, d.d_alive, (size_t)nw * sizeof(int), cudaMemcpyDeviceToHost, s));
  return EVR_OK;
}

// A phase run eagerly, or recorded once as a CUDA graph (keyed by its shape)
// and replayed.  The first run of each shape is eager: it also sizes the
// H.psi plan for that block, which allocates, and allocation cannot be
// recorded.
struct DavGraphs {
  std::vector<cudaGraphExec_t> exec;  // [0]: Ritz phase; [1 + nw]: expansion by nw
  std::vector<char> seen;
  cudaStream_t cs = nullptr;
  ~DavGraphs() {
    for (cudaGraphExec_t e : exec)
      if (e) cudaGraphExecDestroy(e);
    if (cs) cudaStreamDestroy(cs);
  }
};

template <class F>
static int dav_run(DavGraphs& g, int key, bool graph, cudaStream_t s, F&& enqueue) {
  if (!graph || !g.seen[key]) {
    g.seen[key] = 1;
    return enqueue(s);
  }
  if (!g.exec[key]) {
    if (!g.cs) CUDA_TRY_S(cudaStreamCreateWithFlags(&g.cs, cudaStreamNonBlocking));
    CUDA_TRY_S(cudaStreamSynchronize(s));
    cudaGraph_t gr = nullptr;
    CUDA_TRY_S(cudaStreamBeginCapture(g.cs, cudaStreamCaptureModeThreadLocal));
    int rc = enqueue(g.cs);
    cudaError_t ec = cudaStreamEndCapture(g.cs, &gr);
    if (rc) {
      if (gr) cudaGraphDestroy(gr);
      return rc;
    }
    if (ec != cudaSuccess) return set_error(EVR_ERR_CUDA, "davidson: graph capture: %s", cudaGetErrorString(ec));
    ec = cudaGraphInstantiate(&g.exec[key], gr, 0);
    cudaGraphDestroy(gr);
    if (ec != cudaSuccess) {
      g.exec[key] = nullptr;
      return set_error(EVR_ERR_CUDA, "davidson: graph instantiate: %s", cudaGetErrorString(ec));
    }
  }
  CUDA_TRY_S(cudaGraphLaunch(g.exec[key], s));
  return EVR_OK;
}

}  // namespace evr

extern "C" int evr_sg4_davidson(evr_sg4_ctx* c, const evr_davidson_opts* o, const double* guess, int nguess,
                                const double* diag, double* evals, double* evecs, double* resid, int* iterations,
                                void* stream) {
  if (!c || !o || !evals) return set_error(EVR_ERR_ARG, "davidson: NULL argument");
  long long sz[8];
  int rc = evr_sg4_ctx_sizes(c, sz);
  if (rc) return rc;
  const long long N = sz[0];
  const int nev = o->nev;
  const int blk = o->block > 0 ? o->block : nev;
  const int mmax = o->max_subspace > 0 ? o->max_subspace : std::max(3 * nev, nev + 2 * blk);
  if (nev < 1 || nev > N || blk < 1 || mmax < nev + blk || mmax > N || o->max_it < 1 || !(o->conv_resi > 0))
    return set_error(EVR_ERR_ARG, "davidson: need 1 <= nev, block >= 1, nev+block <= max_subspace <= N, conv_resi > 0");
  if (N > 2147483647LL) return set_error(EVR_ERR_ARG, "davidson: N exceeds the int range of cuBLAS");
  cudaStream_t s = (cudaStream_t)stream;
  DavState d;
  d.c = c;
  d.s = s;
  d.N = N;
  d.nev = nev;
  d.blk = blk;
  d.mmax = mmax;
  d.sym = o->symmetrize != 0;
  d.diag = diag;
  CUBLAS_TRY(cublasCreate(&d.h));
  struct Guard {
    DavState& d;
    std::vector<void*> dev, host;
    ~Guard() {
      if (d.h) cublasDestroy(d.h);
      for (void* p : dev) cudaFree(p);
      for (void* p : host) cudaFreeHost(p);
    }
  } guard{d, {}, {}};
  auto dalloc = [&](double** p, size_t n) -> int {
    CUDA_TRY_S(cudaMalloc(p, std::max<size_t>(n, 1) * 8));
    guard.dev.push_back(*p);
    return EVR_OK;
  };
  const int n0 = nguess > 0 && guess ? std::min(nguess, mmax - blk) : nev;
  const int wcols = std::max(blk, n0);
  if ((rc = dalloc(&d.V, (size_t)N * mmax)) || (rc = dalloc(&d.HV, (size_t)N * mmax)) ||
      (rc = dalloc(&d.X, (size_t)N * nev)) || (rc = dalloc(&d.R, (size_t)N * nev)) ||
      (rc = dalloc(&d.W, (size_t)N * wcols)) || (rc = dalloc(&d.HW, (size_t)N * wcols)) ||
      (rc = dalloc(&d.tmp, (size_t)N * std::max(wcols, nev))) || (rc = dalloc(&d.Tt, (size_t)mmax * wcols)) ||
      (rc = dalloc(&d.T, (size_t)mmax * mmax)) || (rc = dalloc(&d.cv, (size_t)wcols)) ||
      (rc = dalloc(&d.nrm, (size_t)nev + wcols)))
    return rc;
  double* ws = nullptr;  // cuBLAS workspace: no allocation while a graph is recorded
  if ((rc = dalloc(&ws, (size_t)4 << 20))) return rc;
  CUBLAS_TRY(cublasSetWorkspace(d.h, ws, (size_t)32 << 20));
  d.params_bytes = sizeof(DavParams) + d.cols_bytes() + (size_t)(nev + (size_t)mmax * nev) * 8;
  {
    void* p = nullptr;
    CUDA_TRY_S(cudaMalloc(&p, d.params_bytes));
    guard.dev.push_back(p);
    d.dparams = (unsigned char*)p;
    CUDA_TRY_S(cudaMalloc(&p, (size_t)wcols * sizeof(int)));
    guard.dev.push_back(p);
    d.d_alive = (int*)p;
    CUDA_TRY_S(cudaMallocHost(&p, d.params_bytes));
    guard.host.push_back(p);
    d.hparams = (unsigned char*)p;
    memset(p, 0, d.params_bytes);
    CUDA_TRY_S(cudaMallocHost(&p, (size_t)mmax * mmax * 8));
    guard.host.push_back(p);
    d.h_T = (double*)p;
    CUDA_TRY_S(cudaMallocHost(&p, (size_t)(nev + wcols) * 8));
    guard.host.push_back(p);
    d.h_nrm = (double*)p;
    CUDA_TRY_S(cudaMallocHost(&p, (size_t)wcols * sizeof(int)));
    guard.host.push_back(p);
    d.h_alive = (int*)p;
  }
  CUDA_TRY_S(cudaMemsetAsync(d.V, 0, (size_t)N * mmax * 8, s));
  CUDA_TRY_S(cudaMemsetAsync(d.HV, 0, (size_t)N * mmax * 8, s));
  // one fixed H.psi (and H^T.psi) per block width W -> HW (-> tmp), recordable
  struct Bound {
    BoundApply *H = nullptr, *HT = nullptr;
  };
  std::vector<Bound> bound(wcols + 1);
  struct BGuard {
    std::vector<Bound>& b;
    ~BGuard() {
      for (Bound& x : b) {
        bound_apply_destroy(x.H);
        bound_apply_destroy(x.HT);
      }
    }
  } bguard{bound};
  long long nslices = 0;
  if ((rc = evr_sg4_field_slices(c, &nslices))) return rc;
  const bool graph = !o->no_graph && nslices == 0;  // streamed fields: eager launches
  auto apply_block = [&](int nw, cudaStream_t st) -> int {
    if (!graph) return apply_hs(c, N, nw, d.W, d.HW, d.tmp, d.sym, st);
    Bound& b = bound[nw];
    int r = EVR_OK;
    if (!b.H && (r = bound_apply_create(c, nw, 0, d.W, d.HW, &b.H))) return r;
    if (d.sym && !b.HT && (r = bound_apply_create(c, nw, 1, d.W, d.tmp, &b.HT))) return r;
    if ((r = bound_apply_launch(b.H, st))) return r;
    if (d.sym) {
      if ((r = bound_apply_launch(b.HT, st))) return r;
      average_kernel<<<256, 256, 0, st>>>(d.HW, d.HW, d.tmp, N * nw);
      CUDA_TRY_S(cudaGetLastError());
    }
    return EVR_OK;
  };
  // the apply inside the expansion goes through apply_block
  DavGraphs gr;
  gr.exec.assign(2 + wcols, nullptr);
  gr.seen.assign(2 + wcols, 0);
  auto expand = [&](int nw, bool precond) -> int {
    auto enq = [&](cudaStream_t st) -> int { return dav_phase_expand(d, nw, precond, st, apply_block); };
    // the initial block is never recorded (its width may differ from blk and it runs once)
    int r = precond ? dav_run(gr, 1 + nw, graph, s, enq) : enq(s);
    if (r) return r;
    CUDA_TRY_S(cudaStreamSynchronize(s));
    return EVR_OK;
  };

  // initial block: the caller's guess, or the first packed functions (lowest L)
  if (guess && nguess > 0) {
    CUDA_TRY_S(cudaMemcpyAsync(d.W, guess, (size_t)N * n0 * 8, cudaMemcpyDeviceToDevice, s));
  } else {
    unit_block_kernel<<<256, 256, 0, s>>>(d.W, N, n0, 0);
  }
  DavParams* hp = (DavParams*)d.hparams;
  hp->m = 0;
  if ((rc = expand(n0, false))) return rc;
  std::vector<char> live(mmax, 0);  // slot holds a (non-zero) basis vector
  int m = 0;
  for (int j = 0; j < n0; ++j)
    if (d.h_alive[j]) live[m++] = 1;
  if (m == 0) return set_error(EVR_ERR_NUMERIC, "davidson: the initial block is rank deficient");

  std::vector<double> w, Z, theta(nev), rn(nev);
  int it = 0, k = 0;
  bool converged = false;
  for (it = 0; it < o->max_it; ++it) {
    // projected matrix (live slots), symmetrised on the host (sub_hermitic_H)
    std::vector<int> slot;
    for (int i = 0; i < m; ++i)
      if (live[i]) slot.push_back(i);
    const int ml = (int)slot.size();
    std::vector<double> A((size_t)ml * ml);
    for (int i = 0; i < ml; ++i)
      for (int j = 0; j < ml; ++j)
        A[(size_t)i * ml + j] = 0.5 * (d.h_T[slot[i] + (size_t)mmax * slot[j]] + d.h_T[slot[j] + (size_t)mmax * slot[i]]);
    jacobi_eigen(ml, A, w, Z);
    k = std::min(nev, ml);
    double* Y = d.hY();
    memset(Y, 0, (size_t)mmax * nev * 8);
    for (int j = 0; j < k; ++j)
      for (int i = 0; i < ml; ++i) Y[slot[i] + (size_t)mmax * j] = Z[(size_t)i * ml + j];
    for (int j = 0; j < nev; ++j) d.htheta()[j] = j < k ? w[j] : 0.0;
    for (int j = 0; j < k; ++j) theta[j] = w[j];
    // Ritz vectors, residuals and their norms
    if ((rc = dav_run(gr, 0, graph, s, [&](cudaStream_t st) { return dav_phase_ritz(d, st); }))) return rc;
    CUDA_TRY_S(cudaStreamSynchronize(s));
    std::vector<int> todo;
    for (int j = 0; j < k; ++j) {
      rn[j] = d.h_nrm[j];
      if (!std::isfinite(rn[j])) return set_error(EVR_ERR_NUMERIC, "davidson: non-finite residual");
      if (!(rn[j] < o->conv_resi)) todo.push_back(j);
    }
    if (k == nev && todo.empty()) {
      converged = true;
      break;
    }
    // restart (keep the Ritz vectors) when the new block does not fit
    const int nnew = std::min((int)todo.size(), blk);
    if (m + nnew > mmax) {
      const double one = 1.0, zero = 0.0;
      CUBLAS_TRY(cublasSetStream(d.h, s));
      CUBLAS_TRY(cublasDgemm(d.h, CUBLAS_OP_N, CUBLAS_OP_N, (int)N, k, mmax, &one, d.HV, (int)N, d.dY(), mmax, &zero,
                             d.tmp, (int)N));
      CUDA_TRY_S(cudaMemsetAsync(d.V, 0, (size_t)N * mmax * 8, s));
      CUDA_TRY_S(cudaMemsetAsync(d.HV, 0, (size_t)N * mmax * 8, s));
      CUDA_TRY_S(cudaMemcpyAsync(d.V, d.X, (size_t)N * k * 8, cudaMemcpyDeviceToDevice, s));
      CUDA_TRY_S(cudaMemcpyAsync(d.HV, d.tmp, (size_t)N * k * 8, cudaMemcpyDeviceToDevice, s));
      std::fill(live.begin(), live.end(), 0);
      for (int j = 0; j < k; ++j) live[j] = 1;
      m = k;
    }
    hp->m = m;
    hp->ncols = nnew;
    for (int j = 0; j < nnew; ++j) d.hcols()[j] = todo[j];
    if ((rc = expand(nnew, true))) return rc;
    int added = 0;
    for (int j = 0; j < nnew; ++j) {
      live[m + j] = d.h_alive[j] ? 1 : 0;
      added += d.h_alive[j] ? 1 : 0;
    }
    if (added == 0) return set_error(EVR_ERR_NUMERIC, "davidson: no new direction survived orthogonalisation");
    m += nnew;
  }
  for (int j = 0; j < nev; ++j) evals[j] = theta[j];
  if (resid)
    for (int j = 0; j < nev; ++j) resid[j] = rn[j];
  if (evecs) CUDA_TRY_S(cudaMemcpyAsync(evecs, d.X, (size_t)N * nev * 8, cudaMemcpyDeviceToDevice, s));
  CUDA_TRY_S(cudaStreamSynchronize(s));
  if (iterations) *iterations = it + 1;
  if (!converged) return set_error(EVR_ERR_NUMERIC, "davidson: not converged after %d iterations", o->max_it);
  return EVR_OK;
}

// ------------------------------------------------------------------------
// Chebyshev propagation (march_cheby, SRC/sub_propagation/
// sub_module_propa_march.f90:4145-4437).  Complex psi, interleaved
// complex128, N x nrhs.  Per step:
//   dE = Hmax - Hmin, E0 = Hmin + dE/2, Esc = dE/2, r = dE dt / 2,
//   c_1 = J_0(r), c_k = 2 J_{k-1}(r)  (cof, :5739, via Bessel J_n),
//   w1 = psi, out = c_1 w1, w2 = -i Hs w1, out += c_2 w2,
//   w3 = w1 - 2i Hs w2, w1 <- w2, w2 <- w3, out += c_k w2   (k = 3..npoly)
//   with Hs = (H - E0)/Esc fused into the H.psi launch (sub_scaledOpPsi),
//   stopping early once |c_k| |w2|^2 < poly_tol; a step whose terms blow up
//   (> 1e15) is redone with Hmax raised by dE/10, up to 10 times; finally
//   psi = out exp(-i E0 dt).
// ------------------------------------------------------------------------

// Bessel J_0..J_{n-1}(r) by Miller's backward recurrence in long double,
// normalised with J_0 + 2 sum_k J_2k = 1.
static void bessel_j(double r, int n, std::vector<double>& J) {
  J.assign(n, 0.0);
  if (r == 0.0) {
    J[0] = 1.0;
    return;
  }
  const int start = 2 * ((std::max(n, (int)r) + 20 + (int)(2.0 * std::sqrt(40.0 * (r + 1.0)))) / 2);
  std::vector<long double> b(start + 2, 0.0L);
  b[start + 1] = 0.0L;
  b[start] = 1e-300L;
  for (int k = start; k >= 1; --k) {
    b[k - 1] = (2.0L * k / (long double)r) * b[k] - b[k + 1];
    if (std::fabs((double)b[k - 1]) > 1e250) {  // rescale to avoid overflow
      for (int q = k - 1; q <= start + 1; ++q) b[q] *= 1e-250L;
    }
  }
  long double norm = b[0];
  for (int k = 2; k <= start; k += 2) norm += 2.0L * b[k];
  for (int k = 0; k < n; ++k) J[k] = (double)(b[k] / norm);
}

// w (complex) = a*w + (b0 + i b1) * h ; out += c * w ; nrm += |w|^2
__global__ void cheby_update_kernel(double2* w, const double2* h, double2* out, long long n, double a, double b0,
                                    double b1, double c, double* nrm) {
  double acc = 0.0;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
    double2 x = w[e], y = h[e];
    double2 r;
    r.x = a * x.x + (b0 * y.x - b1 * y.y);
    r.y = a * x.y + (b0 * y.y + b1 * y.x);
    w[e] = r;
    double2 o = out[e];
    o.x = fma(c, r.x, o.x);
    o.y = fma(c, r.y, o.y);
    out[e] = o;
    acc = fma(r.x, r.x, fma(r.y, r.y, acc));
  }
  for (int off = 16; off > 0; off >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, off);
  if ((threadIdx.x & 31) == 0 && nrm) atomicAdd(nrm, acc);
}

__global__ void cscale_kernel(double2* out, const double2* in, long long n, double cr, double ci) {
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
    double2 x = in[e];
    out[e] = make_double2(cr * x.x - ci * x.y, cr * x.y + ci * x.x);
  }
}

// ac[v] = <a(:,v) | b(:,v)>  (one block per column, complex)
__global__ void cdot_cols_kernel(const double2* a, const double2* b, long long N, long long ld, double2* ac) {
  const int v = blockIdx.x;
  double sr = 0.0, si = 0.0;
  for (long long n = threadIdx.x; n < N; n += blockDim.x) {
    double2 x = a[v * ld + n], y = b[v * ld + n];
    sr = fma(x.x, y.x, fma(x.y, y.y, sr));   // conj(x) y
    si = fma(x.x, y.y, fma(-x.y, y.x, si));
  }
  __shared__ double rs[32], is[32];
  for (int off = 16; off > 0; off >>= 1) {
    sr += __shfl_down_sync(0xffffffffu, sr, off);
    si += __shfl_down_sync(0xffffffffu, si, off);
  }
  if ((threadIdx.x & 31) == 0) {
    rs[threadIdx.x >> 5] = sr;
    is[threadIdx.x >> 5] = si;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double r = 0.0, i = 0.0;
    for (int k = 0; k < (int)(blockDim.x >> 5); ++k) {
      r += rs[k];
      i += is[k];
    }
    ac[v] = make_double2(r, i);
  }
}

// Element-wise kernels on complex vectors: 64-thread blocks, enough of them
// to cover n once (up to 32 per SM of a 152-SM GB300), so short vectors
// spread their FP64 work over many SMs.
static inline int ew_grid(long long n) { return (int)std::max<long long>(1, std::min<long long>((n + 63) / 64, 32 * 152)); }
#define EW_THREADS 64

// One fixed-order step, enqueued on s (recorded once as a CUDA graph and
// replayed): save <- psi, the recurrence of order npoly on w1/w2, |w|^2 of
// the last term into hb[0] (pinned), psi = out e^{-i E0 dt}, and the
// autocorrelation <psi0|psi> into hb[1..].
namespace evr {
struct ChebyStep {
  evr_sg4_ctx* c;
  int nrhs;
  long long N, n;
  double *w1, *w2, *h, *out, *save, *nrm, *acb, *psi;
  const double* P0;
  double* hb;
  bool autocorr;
};
}  // namespace evr

static int enqueue_cheby_step(const ChebyStep& st, const std::vector<double>& cf, double E0, double Esc, double ph,
                              cudaStream_t s) {
  const long long n = st.n;
  const int G = ew_grid(n), B = EW_THREADS;
  double *a = st.w1, *b = st.w2;
  CUDA_TRY_S(cudaMemcpyAsync(st.save, st.psi, (size_t)n * 16, cudaMemcpyDeviceToDevice, s));
  CUDA_TRY_S(cudaMemcpyAsync(a, st.save, (size_t)n * 16, cudaMemcpyDeviceToDevice, s));
  cscale_kernel<<<G, B, 0, s>>>((double2*)st.out, (const double2*)a, n, cf[0], 0.0);
  int rc = evr_sg4_apply(st.c, EVR_APPLY_COMPLEX, st.nrhs, a, st.N, st.h, st.N, E0, Esc, s);
  if (rc) return rc;
  CUDA_TRY_S(cudaMemsetAsync(b, 0, (size_t)n * 16, s));
  cheby_update_kernel<<<G, B, 0, s>>>((double2*)b, (const double2*)st.h, (double2*)st.out, n, 0.0, 0.0, -1.0, cf[1],
                                      nullptr);
  const int npoly = (int)cf.size();
  for (int k = 3; k <= npoly; ++k) {
    if ((rc = evr_sg4_apply(st.c, EVR_APPLY_COMPLEX, st.nrhs, b, st.N, st.h, st.N, E0, Esc, s))) return rc;
    const bool last = k == npoly;
    if (last) CUDA_TRY_S(cudaMemsetAsync(st.nrm, 0, 8, s));
    cheby_update_kernel<<<G, B, 0, s>>>((double2*)a, (const double2*)st.h, (double2*)st.out, n, 1.0, 0.0, -2.0,
                                        cf[k - 1], last ? st.nrm : nullptr);
    std::swap(a, b);
  }
  if (npoly >= 3) CUDA_TRY_S(cudaMemcpyAsync(st.hb, st.nrm, 8, cudaMemcpyDeviceToHost, s));
  cscale_kernel<<<G, B, 0, s>>>((double2*)st.psi, (const double2*)st.out, n, std::cos(ph), std::sin(ph));
  if (st.autocorr) {
    cdot_cols_kernel<<<st.nrhs, 256, 0, s>>>((const double2*)st.P0, (const double2*)st.psi, st.N, st.N,
                                             (double2*)st.acb);
    CUDA_TRY_S(cudaMemcpyAsync(st.hb + 1, st.acb, (size_t)st.nrhs * 16, cudaMemcpyDeviceToHost, s));
  }
  CUDA_TRY_S(cudaGetLastError());
  return EVR_OK;
}

namespace evr {
struct GraphGuard {
  cudaGraphExec_t exec = nullptr;
  cudaStream_t cs = nullptr;
  double* hb = nullptr;
  void reset() {
    if (exec) cudaGraphExecDestroy(exec);
    exec = nullptr;
  }
  ~GraphGuard() {
    reset();
    if (cs) cudaStreamDestroy(cs);
    if (hb) cudaFreeHost(hb);
  }
};
}  // namespace evr

extern "C" int evr_sg4_cheby_propagate(evr_sg4_ctx* c, const evr_cheby_opts* o, int nrhs, double* psi,
                                       const double* psi0, double* autocorr, int* npoly_used, void* stream) {
  if (!c || !o || !psi || nrhs < 1) return set_error(EVR_ERR_ARG, "cheby: NULL argument or nrhs < 1");
  if (!(o->Hmax > o->Hmin) || !(o->dt > 0) || o->npoly < 2 || o->nsteps < 0)
    return set_error(EVR_ERR_ARG, "cheby: need Hmax > Hmin, dt > 0, npoly >= 2");
  long long sz[8];
  int rc = evr_sg4_ctx_sizes(c, sz);
  if (rc) return rc;
  const long long N = sz[0], n = N * nrhs;
  cudaStream_t s = (cudaStream_t)stream;
  DevBuf w1, w2, h, out, save, nrm, acb;
  CUDA_TRY_S(cudaMalloc(&w1.p, (size_t)n * 16));
  CUDA_TRY_S(cudaMalloc(&w2.p, (size_t)n * 16));
  CUDA_TRY_S(cudaMalloc(&h.p, (size_t)n * 16));
  CUDA_TRY_S(cudaMalloc(&out.p, (size_t)n * 16));
  CUDA_TRY_S(cudaMalloc(&save.p, (size_t)n * 16));
  CUDA_TRY_S(cudaMalloc(&nrm.p, 8));
  CUDA_TRY_S(cudaMalloc(&acb.p, (size_t)nrhs * 16));
  double2* P = (double2*)psi;
  const double2* P0 = (const double2*)(psi0 ? psi0 : nullptr);
  if (!P0) {  // the autocorrelation reference is the initial packet
    CUDA_TRY_S(cudaMemcpyAsync(save.p, psi, (size_t)n * 16, cudaMemcpyDeviceToDevice, s));
  }
  DevBuf p0copy;
  if (!P0) {
    CUDA_TRY_S(cudaMalloc(&p0copy.p, (size_t)n * 16));
    CUDA_TRY_S(cudaMemcpyAsync(p0copy.p, psi, (size_t)n * 16, cudaMemcpyDeviceToDevice, s));
    P0 = (const double2*)p0copy.p;
  }
  const int G = ew_grid(n), B = EW_THREADS;
  double Hmin = o->Hmin, Hmax = o->Hmax;
  int used = 0;
  std::vector<double> J;
  auto autocorr_at = [&](int step) -> int {
    if (!autocorr) return EVR_OK;
    cdot_cols_kernel<<<nrhs, 256, 0, s>>>(P0, P, N, N, (double2*)acb.p);
    CUDA_TRY_S(cudaGetLastError());
    CUDA_TRY_S(cudaMemcpyAsync(autocorr + (size_t)2 * nrhs * step, acb.p, (size_t)nrhs * 16, cudaMemcpyDeviceToHost, s));
    return EVR_OK;
  };
  if ((rc = autocorr_at(0))) return rc;
  // fixed order: once a step has run eagerly, the step is recorded as a CUDA
  // graph and replayed; a replayed step that diverges is undone from `save`
  // and redone eagerly (with Hmax raised), after which the graph is recorded again
  const bool use_graph = o->poly_tol <= 0.0 && !o->no_graph;
  GraphGuard gg;
  std::vector<double> gcf;
  if (use_graph) {
    CUDA_TRY_S(cudaStreamCreateWithFlags(&gg.cs, cudaStreamNonBlocking));
    CUDA_TRY_S(cudaMallocHost(&gg.hb, (size_t)(1 + 2 * nrhs) * 8));
  }
  const ChebyStep cst{c, nrhs, N, n, w1.p, w2.p, h.p, out.p, save.p, nrm.p, acb.p, psi, (const double*)P0,
                      gg.hb, autocorr != nullptr};
  for (int step = 0; step < o->nsteps; ++step) {
    if (gg.exec) {
      CUDA_TRY_S(cudaGraphLaunch(gg.exec, s));
      CUDA_TRY_S(cudaStreamSynchronize(s));
      const double norm_exit = o->npoly >= 3 ? std::fabs(gg.hb[0] * gcf[o->npoly - 1]) : 0.0;
      if (norm_exit <= 1e15) {
        if (autocorr) memcpy(autocorr + (size_t)2 * nrhs * (step + 1), gg.hb + 1, (size_t)nrhs * 16);
        used = std::max(used, o->npoly);
        continue;
      }
      CUDA_TRY_S(cudaMemcpyAsync(psi, save.p, (size_t)n * 16, cudaMemcpyDeviceToDevice, s));  // undo
      gg.reset();
    }
    CUDA_TRY_S(cudaMemcpyAsync(save.p, psi, (size_t)n * 16, cudaMemcpyDeviceToDevice, s));
    bool ok = false;
    for (int attempt = 0; attempt < 10 && !ok; ++attempt) {
      const double dE = Hmax - Hmin, E0 = Hmin + 0.5 * dE, Esc = 0.5 * dE, r = 0.5 * dE * o->dt;
      bessel_j(r, o->npoly, J);
      std::vector<double> cf(o->npoly);
      cf[0] = J[0];
      for (int k = 1; k < o->npoly; ++k) cf[k] = 2.0 * J[k];
      // w1 = psi, out = c_1 psi
      CUDA_TRY_S(cudaMemcpyAsync(w1.p, save.p, (size_t)n * 16, cudaMemcpyDeviceToDevice, s));
      cscale_kernel<<<G, B, 0, s>>>((double2*)out.p, (const double2*)w1.p, n, cf[0], 0.0);
      // w2 = -i Hs w1 ; out += c_2 w2
      if ((rc = evr_sg4_apply(c, EVR_APPLY_COMPLEX, nrhs, w1.p, N, h.p, N, E0, Esc, s))) return rc;
      CUDA_TRY_S(cudaMemsetAsync(w2.p, 0, (size_t)n * 16, s));
      cheby_update_kernel<<<G, B, 0, s>>>((double2*)w2.p, (const double2*)h.p, (double2*)out.p, n, 0.0, 0.0, -1.0,
                                          cf[1], nullptr);
      double norm_exit = 0.0;
      int k_end = 2;
      bool blown = false;
      for (int k = 3; k <= o->npoly; ++k) {
        if ((rc = evr_sg4_apply(c, EVR_APPLY_COMPLEX, nrhs, w2.p, N, h.p, N, E0, Esc, s))) return rc;
        const bool check = o->poly_tol > 0.0 || k == o->npoly;
        if (check) CUDA_TRY_S(cudaMemsetAsync(nrm.p, 0, 8, s));
        // w3 = w1 - 2i h, written over w1; then w1 <-> w2
        cheby_update_kernel<<<G, B, 0, s>>>((double2*)w1.p, (const double2*)h.p, (double2*)out.p, n, 1.0, 0.0,
                                            -2.0, cf[k - 1], check ? nrm.p : nullptr);
        std::swap(w1.p, w2.p);
        k_end = k;
        if (check) {
          double nr = 0.0;
          CUDA_TRY_S(cudaMemcpyAsync(&nr, nrm.p, 8, cudaMemcpyDeviceToHost, s));
          CUDA_TRY_S(cudaStreamSynchronize(s));
          norm_exit = std::fabs(nr * cf[k - 1]);
          if (!(norm_exit <= 1e15)) {
            blown = true;
            break;
          }
          if (o->poly_tol > 0.0 && norm_exit < o->poly_tol) break;
        }
      }
      used = std::max(used, k_end);
      if (blown || (o->poly_tol > 0.0 && !(norm_exit < o->poly_tol))) {
        Hmax += 0.1 * dE;  // :4362
        continue;
      }
      const double ph = -E0 * o->dt;  // psi = out exp(-i E0 dt)
      cscale_kernel<<<G, B, 0, s>>>(P, (const double2*)out.p, n, std::cos(ph), std::sin(ph));
      CUDA_TRY_S(cudaGetLastError());
      ok = true;
    }
    if (!ok) return set_error(EVR_ERR_NUMERIC, "cheby: step %d did not converge after 10 Hmax increases", step);
    if ((rc = autocorr_at(step + 1))) return rc;
    if (use_graph && step + 1 < o->nsteps) {  // record the step with the bounds that worked
      const double dE = Hmax - Hmin, gE0 = Hmin + 0.5 * dE;
      bessel_j(0.5 * dE * o->dt, o->npoly, J);
      gcf.assign(o->npoly, 0.0);
      gcf[0] = J[0];
      for (int k = 1; k < o->npoly; ++k) gcf[k] = 2.0 * J[k];
      CUDA_TRY_S(cudaStreamSynchronize(s));
      cudaGraph_t graph = nullptr;
      CUDA_TRY_S(cudaStreamBeginCapture(gg.cs, cudaStreamCaptureModeRelaxed));
      rc = enqueue_cheby_step(cst, gcf, gE0, 0.5 * dE, -gE0 * o->dt, gg.cs);
      cudaError_t ec = cudaStreamEndCapture(gg.cs, &graph);
      if (rc) {
        if (graph) cudaGraphDestroy(graph);
        return rc;
      }
      if (ec != cudaSuccess) return set_error(EVR_ERR_CUDA, "cheby: graph capture: %s", cudaGetErrorString(ec));
      ec = cudaGraphInstantiate(&gg.exec, graph, 0);
      cudaGraphDestroy(graph);
      if (ec != cudaSuccess) {
        gg.exec = nullptr;
        return set_error(EVR_ERR_CUDA, "cheby: graph instantiate: %s", cudaGetErrorString(ec));
      }
    }
  }
  CUDA_TRY_S(cudaStreamSynchronize(s));
  if (npoly_used) *npoly_used = used;
  return EVR_OK;
}

// ------------------------------------------------------------------------
// Field-driven RK4 (march_RK4_field, SRC/sub_propagation/
// sub_module_propa_march.f90:397-548, with fcn_field :1439-1520):
//   dpsi/dt = -i (H0 - E(t) mu) psi,  E held at E[k] over step k ('grid'
//   field, :483-510), classic RK4 stages on (H0 - E0) with the phase
//   exp(-i E0 dt) restored after each step, as fcn_field does with
//   para_H%E0 (E0 near the middle of the spectrum keeps RK4 stable).  H0 and
//   mu are two contexts on the same basis (mu a type-0 operator).  Several
//   packets can be propagated together, each with its own field (packet b
//   sees E[k*nb + b]).  The optimal-control gradient is the exact adjoint of
//   those discrete steps: with S = <target|psi_N>,
//   J = |S|^2,  lambda_N = S target,  and for each step the stage costates
//   kb4 = h/6 l, kb3 = h/3 l + h sb4, kb2 = h/3 l + h/2 sb3, kb1 = h/6 l + h/2 sb2,
//   sb_i = A^dagger kb_i = i (H0^T - E mu^T) kb_i,  lambda_{k-1} = l + sum sb_i,
//   dJ/dE_k = sum_i 2 Re(kb_i^dagger (i mu s_i)),
// s_i the stage inputs of step k.  psi is checkpointed every `checkpoint`
// field intervals and each segment is recomputed (keeping its stage inputs)
// before its backward sweep.  Each field interval dt is integrated with nsub
// RK4 steps of dt/nsub (E held over the interval), which keeps fixed-step
// RK4 accurate when dt times the spectral range is too large for one step.
// The reference's control update (build_field, SRC/sub_propagation/
// sub_control.f90:907-1010) uses the continuous-time form of the same
// derivative, -2 Im(S* <chi(t)|mu|psi(t)>).
//
// Every kernel of a field interval takes the interval index from a device
// counter (SweepCtl) instead of a launch argument, so one field interval --
// nsub steps x 4 stages x (H0/mu launch, chunk sums, stage update), then the
// counter update -- is recorded once as a CUDA graph and replayed for every
// interval; the eager path launches the same kernels in the same order.
// ------------------------------------------------------------------------

// Device-side position of a sweep: the current field interval and which
// interval's stage inputs are recorded (-1: none, -2: every interval, else
// the intervals of checkpoint segment rec_seg).
struct SweepCtl {
  int k;
  int rec_seg;
};

// The two operators of a stage (H0 and mu, or both transposed) run in one
// persistent launch (field_pair_apply); the kernels below join their chunk
// partials in the same order as evr_sg4_hpsi and fuse the stage arithmetic.
struct StageIn {
  const double2* part;         // [2][n_chunks][nrhs_v] (s, c) partials, H0 first
  const long long* fun_chunk;  // [N+1]
  long long nch2;              // n_chunks * nrhs_v: offset of mu's partials
  long long N;
  int nb, nrhs_v;              // packets, 2 nb virtual columns
  double2* x;                  // stage input [nb][N], overwritten by the next stage's input
  const double* E;             // field samples [nsteps][nb] (device)
  const SweepCtl* ctl;         // current interval
  double E0, h;
  int C, nsub;                 // checkpoint spacing, RK4 steps per interval
  double2* rec;                // stage-input records: two alternating segment buffers, or NULL
  long long seg_rec;           // complex elements per segment buffer
};

// stage inputs of step u of interval k, stage `stage`, when interval k is recorded
__device__ __forceinline__ double2* rec_at(const StageIn& a, int k, int u, int stage) {
  if (!a.rec) return nullptr;
  const int seg = k / a.C;
  if (a.ctl->rec_seg != -2 && a.ctl->rec_seg != seg) return nullptr;
  return a.rec + (size_t)(seg & 1) * a.seg_rec + (((size_t)(k - seg * a.C) * a.nsub + u) * 4 + (stage - 1)) * a.N * a.nb;
}

// The four ordered sums of element (n, packet b) -- H0 re, H0 im, mu re,
// mu im -- are joined by four lanes of a warp, one sum each, and gathered
// with shuffles: GB300's FP64 pipe does about two operations per clock per
// SM, so these joins must be spread over many SMs (a block of 32 threads
// handles 8 elements); with one thread per element and 256-thread blocks the
// stage kernels of a small operator ran on two SMs and took longer than its
// H.psi launch.  Each sum is the join of evr_sg4_hpsi in its order.  Call
// from every lane of a warp with the same e0 (the first element of the
// warp's eight); lane q of group g handles element e0 + g.
__device__ __forceinline__ bool stage_sums4(const StageIn& a, long long e0, long long& e, int& b, double2& xv,
                                            double& E, double& re, double& im, double& mr, double& mi) {
  const int lane = threadIdx.x & 31, g = lane >> 2, q = lane & 3;
  e = e0 + g;
  const long long ne = a.N * a.nb;
  double v = 0.0;
  b = 0;
  long long n = 0;
  if (e < ne) {
    b = (int)(e / a.N);
    n = e - (long long)b * a.N;
    const long long c0 = a.fun_chunk[n], c1 = a.fun_chunk[n + 1];
    v = join_chunks(a.part + (q >> 1) * a.nch2, c0, c1, a.nrhs_v, 2 * b + (q & 1));
  }
  const double hr0 = __shfl_sync(0xffffffffu, v, lane & ~3), hi0 = __shfl_sync(0xffffffffu, v, (lane & ~3) | 1);
  mr = __shfl_sync(0xffffffffu, v, (lane & ~3) | 2);
  mi = __shfl_sync(0xffffffffu, v, (lane & ~3) | 3);
  if (q != 0 || e >= ne) return false;
  xv = a.x[e];
  E = a.E[(long long)a.ctl->k * a.nb + b];
  double hr = hr0, hi = hi0;
  if (a.E0 != 0.0) {  // (H0 - E0) x, as the scaled H.psi writes it
    hr = hr - a.E0 * xv.x;
    hi = hi - a.E0 * xv.y;
  }
  re = hr - E * mr;
  im = hi - E * mi;
  return true;
}

__device__ __forceinline__ double2 cmul(double2 t, double cr, double ci) {
  return make_double2(cr * t.x - ci * t.y, cr * t.y + ci * t.x);
}

// first element of this warp's eight, and the element stride of the grid
__device__ __forceinline__ long long warp_elem0() {
  return ((long long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5)) * 8;
}
__device__ __forceinline__ long long grid_elem_stride() { return (long long)gridDim.x * (blockDim.x >> 5) * 8; }

// forward stage i of RK4 step u of the current interval, y -> y (h = step):
//   k = -i ((H0 - E0) x - E mu x);  [rec = x]
//   i=1: acc = y + h/6 k, x = y + h/2 k     i=2: acc += h/3 k, x = y + h/2 k
//   i=3: acc += h/3 k,    x = y + h k       i=4: y = (acc + h/6 k) e^{-i E0 h}, x = y
__global__ void __launch_bounds__(256) rk_stage_kernel(StageIn a, int u, int stage, double2* y, double2* acc,
                                                       double cr, double ci) {
  const long long ne = a.N * a.nb;
  double2* rec = rec_at(a, a.ctl->k, u, stage);
  for (long long e0 = warp_elem0(); e0 < ne; e0 += grid_elem_stride()) {
    long long e;
    int b;
    double2 xv;
    double E, re, im, mr, mi;
    if (!stage_sums4(a, e0, e, b, xv, E, re, im, mr, mi)) continue;
    const double2 k = make_double2(im, -re);  // -i (re + i im)
    if (rec) rec[e] = xv;
    const double2 yv = y[e];
    const double h = a.h;
    if (stage == 1) {
      acc[e] = make_double2(fma(h / 6.0, k.x, yv.x), fma(h / 6.0, k.y, yv.y));
      a.x[e] = make_double2(fma(0.5 * h, k.x, yv.x), fma(0.5 * h, k.y, yv.y));
    } else if (stage < 4) {
      const double2 ac = acc[e];
      acc[e] = make_double2(fma(h / 3.0, k.x, ac.x), fma(h / 3.0, k.y, ac.y));
      const double c = stage == 2 ? 0.5 * h : h;
      a.x[e] = make_double2(fma(c, k.x, yv.x), fma(c, k.y, yv.y));
    } else {
      const double2 ac = acc[e];
      double2 t = make_double2(fma(h / 6.0, k.x, ac.x), fma(h / 6.0, k.y, ac.y));
      if (a.E0 != 0.0) t = cmul(t, cr, ci);
      y[e] = t;
      a.x[e] = t;
    }
  }
}

// adjoint stage i (taken 4, 3, 2, 1) of RK4 step u of the current interval,
// costate l (phased); kb = x, s_i = the recorded stage input:
//   sb = +i ((H0^T - E0) kb - E mu^T kb);
//   gpart[...] = -2 Im((mu^T kb)^dagger s_i) = -2 Im(kb^dagger mu s_i), one per block;
//   i=4: yb = l + sb, x = h/3 l + h sb       i=3: yb += sb, x = h/3 l + h/2 sb
//   i=2: yb += sb, x = h/6 l + h/2 sb        i=1: l = (yb + sb) e^{+i E0 h}, x = h/6 l
// (the last form also prepares the previous step's stage 4).  The block
// partials of interval k, step u (taken nsub-1 .. 0), stage i go to
// gpart[((k nsub + nsub-1-u) 4 + 4-i) nblk + block].
__global__ void __launch_bounds__(256) rk_adjoint_stage_kernel(StageIn a, int u, int stage, double2* l, double2* yb,
                                                               double* gpart, double cr, double ci) {
  const int k = a.ctl->k;
  const int seg = k / a.C;
  const double2* s = a.rec + (size_t)(seg & 1) * a.seg_rec +
                     (((size_t)(k - seg * a.C) * a.nsub + u) * 4 + (stage - 1)) * a.N * a.nb;
  const long long ne = a.N * a.nb;
  double g = 0.0;
  for (long long e0 = warp_elem0(); e0 < ne; e0 += grid_elem_stride()) {
    long long e;
    int b;
    double2 xv;
    double E, re, im, mr, mi;
    if (!stage_sums4(a, e0, e, b, xv, E, re, im, mr, mi)) continue;
    const double2 sb = make_double2(-im, re);  // +i (re + i im)
    const double2 sv = s[e];
    g = fma(mr, sv.y, fma(-mi, sv.x, g));
    const double2 lv = l[e];
    const double h = a.h;
    if (stage == 4) {
      yb[e] = make_double2(fma(1.0, sb.x, lv.x), fma(1.0, sb.y, lv.y));
      a.x[e] = make_double2(fma(h, sb.x, (h / 3.0) * lv.x), fma(h, sb.y, (h / 3.0) * lv.y));
    } else if (stage > 1) {
      const double2 bb = yb[e];
      yb[e] = make_double2(fma(1.0, sb.x, bb.x), fma(1.0, sb.y, bb.y));
      const double c = stage == 3 ? h / 3.0 : h / 6.0;
      a.x[e] = make_double2(fma(0.5 * h, sb.x, c * lv.x), fma(0.5 * h, sb.y, c * lv.y));
    } else {
      const double2 bb = yb[e];
      double2 t = make_double2(fma(1.0, sb.x, bb.x), fma(1.0, sb.y, bb.y));
      if (a.E0 != 0.0) t = cmul(t, cr, ci);
      l[e] = t;
      a.x[e] = make_double2((h / 6.0) * t.x, (h / 6.0) * t.y);
    }
  }
  __shared__ double sh[32];
  for (int off = 16; off > 0; off >>= 1) g += __shfl_down_sync(0xffffffffu, g, off);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = g;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int q = 0; q < (int)(blockDim.x >> 5); ++q) t += sh[q];
    gpart[(((size_t)k * a.nsub + (a.nsub - 1 - u)) * 4 + (4 - stage)) * gridDim.x + blockIdx.x] = -2.0 * t;
  }
}

// sweep counter updates (one thread): the next interval, or the previous one
__global__ void sweep_step_kernel(SweepCtl* ctl, int delta) { ctl->k += delta; }

// checkpoint of the forward sweep: ck[k / C] = y at the start of every C-th interval
__global__ void checkpoint_kernel(const SweepCtl* ctl, int C, const double2* y, double2* ck, long long n) {
  const int k = ctl->k;
  if (k % C) return;
  double2* dst = ck + (size_t)(k / C) * n;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x)
    dst[e] = y[e];
}

// l = lambda e^{+i E0 h}, x = h/6 l: the start of the backward sweep
__global__ void rk_adjoint_start_kernel(double2* l, const double2* lam, double2* x, long long N, double h, double cr,
                                        double ci, int phase) {
  for (long long n = blockIdx.x * (long long)blockDim.x + threadIdx.x; n < N; n += (long long)gridDim.x * blockDim.x) {
    double2 t = lam[n];
    if (phase) t = cmul(t, cr, ci);
    l[n] = t;
    x[n] = make_double2((h / 6.0) * t.x, (h / 6.0) * t.y);
  }
}

// g[k] = sum of the stage partials of field interval k: nsub steps x 4 stages x nblk blocks, in that order
__global__ void rk_grad_sum_kernel(const double* gpart, int nsteps, int nsub, int nblk, double* g) {
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < nsteps; k += gridDim.x * blockDim.x) {
    double t = 0.0;
    const double* q = gpart + (size_t)k * nsub * 4 * nblk;
    for (int e = 0; e < nsub * 4 * nblk; ++e) t += q[e];
    g[k] = t;
  }
}

__global__ void ctl_set_kernel(SweepCtl* ctl, int k, int rec_seg) {
  ctl->k = k;
  ctl->rec_seg = rec_seg;
}

namespace evr {

// Stage-kernel geometry: four lanes per element (eight elements per warp),
// one-warp blocks for small blocks of vectors so the joins spread over many SMs.
static int stage_threads(long long ne) { return ne <= 32768 ? 32 : 256; }
static int join_blocks(long long ne) {
  const long long per = stage_threads(ne) / 4;
  return (int)std::max<long long>(1, std::min<long long>((ne + per - 1) / per, 4096));
}

// The kernels of one field interval of a forward or adjoint sweep, launched
// eagerly or recorded once as a CUDA graph and replayed.
struct Sweep {
  FieldPair* fp = nullptr;
  StageIn a{};
  double2* y = nullptr;     // forward: the state; adjoint: the costate l
  double2* acc = nullptr;   // forward: the RK4 accumulator; adjoint: yb
  double* gpart = nullptr;  // adjoint: gradient partials
  double2* ck = nullptr;    // forward: checkpoints (NULL: none)
  bool adjoint = false;
  double cr = 1.0, ci = 0.0;
  int nblk = 1, nthr = 32;
  cudaStream_t cs = nullptr;  // capture stream
  cudaGraphExec_t exec = nullptr;
  ~Sweep() {
    if (exec) cudaGraphExecDestroy(exec);
    if (cs) cudaStreamDestroy(cs);
  }
};

static void sweep_init(Sweep& w, FieldPair* fp, SweepCtl* ctl, const double* Edev, int nb, const evr_rk4_opts* o,
                       bool adjoint) {
  const FieldPairView v = field_pair_view(fp);
  w.fp = fp;
  w.adjoint = adjoint;
  const double h = o->dt / o->nsub;
  w.a = StageIn{(const double2*)v.part, v.fun_chunk, v.n_chunks * 2 * nb, v.N, nb, 2 * nb, (double2*)v.x,
                Edev, ctl, o->E0, h, o->checkpoint, o->nsub, nullptr, 0};
  w.cr = std::cos(o->E0 * h);
  w.ci = adjoint ? std::sin(o->E0 * h) : -std::sin(o->E0 * h);  // e^{+i E0 h} backward, e^{-i E0 h} forward
  w.nblk = join_blocks(v.N * nb);
  w.nthr = stage_threads(v.N * nb);
}

static int enqueue_interval(Sweep& w, cudaStream_t s) {
  const long long ne = w.a.N * w.a.nb;
  const int nsub = w.a.nsub;
  int rc;
  if (!w.adjoint) {
    if (w.ck)
      checkpoint_kernel<<<(unsigned)std::max<long long>(1, std::min<long long>((ne + 255) / 256, 1024)), 256, 0, s>>>(
          w.a.ctl, w.a.C, w.y, w.ck, ne);
    for (int u = 0; u < nsub; ++u)
      for (int stage = 1; stage <= 4; ++stage) {
        if ((rc = field_pair_apply(w.fp, s))) return rc;
        rk_stage_kernel<<<w.nblk, w.nthr, 0, s>>>(w.a, u, stage, w.y, w.acc, w.cr, w.ci);
      }
    sweep_step_kernel<<<1, 1, 0, s>>>(const_cast<SweepCtl*>(w.a.ctl), 1);
  } else {
    sweep_step_kernel<<<1, 1, 0, s>>>(const_cast<SweepCtl*>(w.a.ctl), -1);
    for (int u = nsub - 1; u >= 0; --u)
      for (int stage = 4; stage >= 1; --stage) {
        if ((rc = field_pair_apply(w.fp, s))) return rc;
        rk_adjoint_stage_kernel<<<w.nblk, w.nthr, 0, s>>>(w.a, u, stage, w.y, w.acc, w.gpart, w.cr, w.ci);
      }
  }
  CUDA_TRY_S(cudaGetLastError());
  return EVR_OK;
}

// one field interval on s: eager launches, or the recorded graph (recorded on first use)
static int run_interval(Sweep& w, bool graph, cudaStream_t s) {
  if (!graph) return enqueue_interval(w, s);
  if (!w.exec) {
    if (!w.cs) CUDA_TRY_S(cudaStreamCreateWithFlags(&w.cs, cudaStreamNonBlocking));
    cudaGraph_t g = nullptr;
    CUDA_TRY_S(cudaStreamBeginCapture(w.cs, cudaStreamCaptureModeThreadLocal));
    int rc = enqueue_interval(w, w.cs);
    cudaError_t ec = cudaStreamEndCapture(w.cs, &g);
    if (rc) {
      if (g) cudaGraphDestroy(g);
      return rc;
    }
    if (ec != cudaSuccess) return set_error(EVR_ERR_CUDA, "rk4: graph capture: %s", cudaGetErrorString(ec));
    ec = cudaGraphInstantiate(&w.exec, g, 0);
    cudaGraphDestroy(g);
    if (ec != cudaSuccess) {
      w.exec = nullptr;
      return set_error(EVR_ERR_CUDA, "rk4: graph instantiate: %s", cudaGetErrorString(ec));
    }
  }
  CUDA_TRY_S(cudaGraphLaunch(w.exec, s));
  return EVR_OK;
}

struct PairGuard {
  FieldPair* p = nullptr;
  ~PairGuard() { field_pair_destroy(p); }
};
struct StreamGuard {
  cudaStream_t s = nullptr;
  cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
  ~StreamGuard() {
    for (cudaEvent_t e : ev)
      if (e) cudaEventDestroy(e);
    if (s) cudaStreamDestroy(s);
  }
};

}  // namespace evr

static int check_field_args(evr_sg4_ctx* H0, evr_sg4_ctx* mu, const evr_rk4_opts* o, int nb, const double* E,
                            long long* N) {
  if (!H0 || !mu || !o || !E) return set_error(EVR_ERR_ARG, "rk4: NULL argument");
  long long a[8], b[8];
  int rc = evr_sg4_ctx_sizes(H0, a);
  if (!rc) rc = evr_sg4_ctx_sizes(mu, b);
  if (rc) return rc;
  if (a[0] != b[0] || a[1] != b[1] || a[3] != b[3]) return set_error(EVR_ERR_ARG, "rk4: H0 and mu are on different bases");
  if (o->nsteps < 1 || !(o->dt > 0) || o->checkpoint < 1 || o->nsub < 1 || nb < 1)
    return set_error(EVR_ERR_ARG, "rk4: need nsteps >= 1, dt > 0, checkpoint >= 1, nsub >= 1, packets >= 1");
  for (long long k = 0; k < (long long)o->nsteps * nb; ++k)
    if (!std::isfinite(E[k])) return set_error(EVR_ERR_NUMERIC, "rk4: field sample %lld is not finite", k);
  *N = a[0];
  return EVR_OK;
}

extern "C" int evr_sg4_rk4_field_batch(evr_sg4_ctx* H0, evr_sg4_ctx* mu, const evr_rk4_opts* o, int nb,
                                       const double* E, double* psi, void* stream) {
  long long N = 0;
  int rc = check_field_args(H0, mu, o, nb, E, &N);
  if (rc) return rc;
  if (!psi) return set_error(EVR_ERR_ARG, "rk4: psi is NULL");
  cudaStream_t s = (cudaStream_t)stream;
  PairGuard fp;
  if ((rc = field_pair_create(H0, mu, 0, nb, &fp.p))) return rc;
  const size_t vb = (size_t)N * nb * 16;
  DevBuf acc, Ed, ctl;
  CUDA_TRY_S(cudaMalloc(&acc.p, vb));
  CUDA_TRY_S(cudaMalloc(&Ed.p, (size_t)o->nsteps * nb * 8));
  CUDA_TRY_S(cudaMalloc(&ctl.p, sizeof(SweepCtl)));
  CUDA_TRY_S(cudaMemcpyAsync(Ed.p, E, (size_t)o->nsteps * nb * 8, cudaMemcpyHostToDevice, s));
  ctl_set_kernel<<<1, 1, 0, s>>>((SweepCtl*)ctl.p, 0, -1);
  Sweep w;
  sweep_init(w, fp.p, (SweepCtl*)ctl.p, Ed.p, nb, o, false);
  w.y = (double2*)psi;
  w.acc = (double2*)acc.p;
  CUDA_TRY_S(cudaMemcpyAsync(w.a.x, psi, vb, cudaMemcpyDeviceToDevice, s));
  const bool graph = !o->no_graph;
  for (int k = 0; k < o->nsteps; ++k)
    if ((rc = run_interval(w, graph, s))) return rc;
  CUDA_TRY_S(cudaStreamSynchronize(s));
  return EVR_OK;
}

extern "C" int evr_sg4_rk4_field(evr_sg4_ctx* H0, evr_sg4_ctx* mu, const evr_rk4_opts* o, const double* E, double* psi,
                                 void* stream) {
  return evr_sg4_rk4_field_batch(H0, mu, o, 1, E, psi, stream);
}

// Optimal-control gradient.  Stream A runs the forward sweep (checkpoints
// every C field intervals, the stage inputs of the last segment kept), then
// the backward sweep segment by segment; stream B recomputes segment k-1 from
// its checkpoint (keeping its stage inputs) while stream A runs the adjoint
// of segment k, with two stage buffers alternating between them.  Both
// streams' launches are small, so they share the SMs.  Each sweep replays
// the CUDA graph of one field interval (or launches the same kernels).
extern "C" int evr_sg4_oc_gradient(evr_sg4_ctx* H0, evr_sg4_ctx* mu, const evr_rk4_opts* o, const double* E,
                                   const double* psi0, const double* target, double* J, double* grad, void* stream) {
  long long N = 0;
  int rc = check_field_args(H0, mu, o, 1, E, &N);
  if (rc) return rc;
  if (!psi0 || !target || !J || !grad) return set_error(EVR_ERR_ARG, "oc_gradient: NULL argument");
  cudaStream_t sA = (cudaStream_t)stream;
  StreamGuard sg;
  CUDA_TRY_S(cudaStreamCreateWithFlags(&sg.s, cudaStreamNonBlocking));
  for (cudaEvent_t& e : sg.ev) CUDA_TRY_S(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
  cudaStream_t sB = sg.s;
  const int C = o->checkpoint, ns = o->nsteps, nseg = (ns + C - 1) / C, nsub = o->nsub;
  const double hs = o->dt / nsub;
  const size_t vb = (size_t)N * 16;
  const bool graph = !o->no_graph;
  PairGuard fwd, adj;
  if ((rc = field_pair_create(H0, mu, 0, 1, &fwd.p)) || (rc = field_pair_create(H0, mu, 1, 1, &adj.p))) return rc;
  DevBuf y, acc, ck, rec, lam, l, yb, gpart, g, ov, Ed, ctl;
  for (DevBuf* b : {&y, &acc, &lam, &l, &yb}) CUDA_TRY_S(cudaMalloc(&b->p, vb));
  CUDA_TRY_S(cudaMalloc(&ck.p, vb * nseg));                                 // checkpoints
  const size_t seg_rec = (size_t)C * nsub * 4 * N;                         // complex: stage inputs of a segment
  CUDA_TRY_S(cudaMalloc(&rec.p, seg_rec * 2 * 16));                         // two alternating segment buffers
  CUDA_TRY_S(cudaMalloc(&g.p, (size_t)ns * 8));
  CUDA_TRY_S(cudaMalloc(&ov.p, 16));
  CUDA_TRY_S(cudaMalloc(&Ed.p, (size_t)ns * 8));
  CUDA_TRY_S(cudaMalloc(&ctl.p, 3 * sizeof(SweepCtl)));                    // forward (A), recompute (B), adjoint (A)
  SweepCtl* cF = (SweepCtl*)ctl.p;
  SweepCtl* cB = cF + 1;
  SweepCtl* cA = cF + 2;
  CUDA_TRY_S(cudaMemcpyAsync(Ed.p, E, (size_t)ns * 8, cudaMemcpyHostToDevice, sA));
  Sweep wf, wb, wa;
  sweep_init(wf, fwd.p, cF, Ed.p, 1, o, false);
  sweep_init(wb, fwd.p, cB, Ed.p, 1, o, false);
  sweep_init(wa, adj.p, cA, Ed.p, 1, o, true);
  CUDA_TRY_S(cudaMalloc(&gpart.p, (size_t)ns * nsub * 4 * wa.nblk * 8));
  for (Sweep* w : {&wf, &wb}) {
    w->y = (double2*)y.p;
    w->acc = (double2*)acc.p;
    w->a.rec = (double2*)rec.p;
    w->a.seg_rec = (long long)seg_rec;
  }
  wf.ck = (double2*)ck.p;
  wa.y = (double2*)l.p;
  wa.acc = (double2*)yb.p;
  wa.gpart = gpart.p;
  wa.a.rec = (double2*)rec.p;
  wa.a.seg_rec = (long long)seg_rec;
  // forward sweep (stream A): checkpoints, the stage inputs of the last segment kept
  ctl_set_kernel<<<1, 1, 0, sA>>>(cF, 0, nseg - 1);
  CUDA_TRY_S(cudaMemcpyAsync(y.p, psi0, vb, cudaMemcpyDeviceToDevice, sA));
  CUDA_TRY_S(cudaMemcpyAsync(wf.a.x, psi0, vb, cudaMemcpyDeviceToDevice, sA));
  for (int stp = 0; stp < ns; ++stp)
    if ((rc = run_interval(wf, graph, sA))) return rc;
  // S = <target|psi_N>, J = |S|^2, lambda_N = S target
  cdot_cols_kernel<<<1, 256, 0, sA>>>((const double2*)target, (const double2*)y.p, N, N, (double2*)ov.p);
  double2 S;
  CUDA_TRY_S(cudaMemcpyAsync(&S, ov.p, 16, cudaMemcpyDeviceToHost, sA));
  CUDA_TRY_S(cudaStreamSynchronize(sA));  // also: the forward pair and its buffers are free for stream B
  *J = S.x * S.x + S.y * S.y;
  cscale_kernel<<<64, 256, 0, sA>>>((double2*)lam.p, (const double2*)target, N, S.x, S.y);
  rk_adjoint_start_kernel<<<64, 256, 0, sA>>>((double2*)l.p, (const double2*)lam.p, wa.a.x, N, hs, wa.cr, wa.ci,
                                             o->E0 != 0.0);
  ctl_set_kernel<<<1, 1, 0, sA>>>(cA, ns, -1);
  CUDA_TRY_S(cudaGetLastError());
  cudaEvent_t ready[2] = {sg.ev[0], sg.ev[1]}, freed[2] = {sg.ev[2], sg.ev[3]};
  for (int seg = nseg - 1; seg >= 0; --seg) {
    if (seg > 0) {  // stream B: recompute segment seg-1 into the other buffer
      const int ps = seg - 1;
      if (seg + 1 < nseg) CUDA_TRY_S(cudaStreamWaitEvent(sB, freed[ps & 1], 0));
      ctl_set_kernel<<<1, 1, 0, sB>>>(cB, ps * C, -2);
      CUDA_TRY_S(cudaMemcpyAsync(y.p, ck.p + (size_t)ps * 2 * N, vb, cudaMemcpyDeviceToDevice, sB));
      CUDA_TRY_S(cudaMemcpyAsync(wb.a.x, y.p, vb, cudaMemcpyDeviceToDevice, sB));
      for (int stp = ps * C; stp < std::min(ns, (ps + 1) * C); ++stp)
        if ((rc = run_interval(wb, graph, sB))) return rc;
      CUDA_TRY_S(cudaEventRecord(ready[ps & 1], sB));
    }
    if (seg < nseg - 1) CUDA_TRY_S(cudaStreamWaitEvent(sA, ready[seg & 1], 0));
    const int a0 = seg * C, b0 = std::min(ns, a0 + C);
    for (int stp = b0 - 1; stp >= a0; --stp)  // stream A: adjoint of segment seg
      if ((rc = run_interval(wa, graph, sA))) return rc;
    CUDA_TRY_S(cudaEventRecord(freed[seg & 1], sA));
  }
  rk_grad_sum_kernel<<<(ns + 255) / 256, 256, 0, sA>>>(gpart.p, ns, nsub, wa.nblk, g.p);
  CUDA_TRY_S(cudaMemcpyAsync(grad, g.p, (size_t)ns * 8, cudaMemcpyDeviceToHost, sA));
  CUDA_TRY_S(cudaStreamSynchronize(sA));
  CUDA_TRY_S(cudaStreamSynchronize(sB));
  return EVR_OK;
}

// ------------------------------------------------------------------------
// Chebyshev propagation of every context of a complex multi-context plan in
// lock-step (the uneven-instance workload): each expansion order is
// ONE evr_sg4_multi_hpsi over all contexts still in their step, with each
// context's own (E0, Esc) fused, followed by the per-context recurrence
// update.  Per context the arithmetic is that of evr_sg4_cheby_propagate
// with a fixed order (march_cheby, sub_module_propa_march.f90:4145-4437); a
// context whose step diverges (> 1e15) redoes the step with its Hmax raised
// by (Hmax-Hmin)/10 (:4362), alone with the other diverged contexts.
// ------------------------------------------------------------------------
extern "C" int evr_sg4_multi_cheby_propagate(evr_sg4_multi* m, const evr_cheby_opts* o, double* const* psi,
                                             double* const* autocorr, int* npoly_used, void* stream) {
  if (!m || !o || !psi) return set_error(EVR_ERR_ARG, "multi_cheby: NULL argument");
  std::vector<evr_sg4_ctx*> ctxs;
  std::vector<int> nv;
  int cshift = 0, transpose = 0;
  multi_shape(m, &ctxs, &nv, &cshift, &transpose);
  const int n = (int)ctxs.size();
  if (!cshift || transpose) return set_error(EVR_ERR_ARG, "multi_cheby: the plan must be complex, not transposed");
  const double dt = o[0].dt;
  const int npoly = o[0].npoly, nsteps = o[0].nsteps;
  for (int k = 0; k < n; ++k) {
    if (!psi[k]) return set_error(EVR_ERR_ARG, "multi_cheby: psi[%d] is NULL", k);
    if (!(o[k].Hmax > o[k].Hmin) || !(o[k].dt > 0) || o[k].npoly < 2 || o[k].nsteps < 0)
      return set_error(EVR_ERR_ARG, "multi_cheby: context %d needs Hmax > Hmin, dt > 0, npoly >= 2", k);
    if (o[k].dt != dt || o[k].npoly != npoly || o[k].nsteps != nsteps || o[k].poly_tol > 0.0)
      return set_error(EVR_ERR_ARG, "multi_cheby: dt, npoly, nsteps must agree and poly_tol be <= 0 (fixed order)");
  }
  cudaStream_t s = (cudaStream_t)stream;
  std::vector<long long> N(n), len(n), off(n + 1, 0);
  for (int k = 0; k < n; ++k) {
    long long sz[8];
    int rc = evr_sg4_ctx_sizes(ctxs[k], sz);
    if (rc) return rc;
    N[k] = sz[0];
    len[k] = N[k] * nv[k];  // complex elements
    off[k + 1] = off[k] + len[k];
  }
  // per context: w1, w2, h, out, psi0 (complex), carved from one pool
  DevBuf pool, nrm, acb;
  const long long tot = off[n];
  CUDA_TRY_S(cudaMalloc(&pool.p, (size_t)tot * 5 * 16));
  CUDA_TRY_S(cudaMalloc(&nrm.p, (size_t)n * 8));
  const int max_nrhs = *std::max_element(nv.begin(), nv.end());
  CUDA_TRY_S(cudaMalloc(&acb.p, (size_t)max_nrhs * 16));
  auto buf = [&](int which, int k) { return (double2*)pool.p + which * tot + off[k]; };
  std::vector<double2*> w1(n), w2(n);
  for (int k = 0; k < n; ++k) {
    w1[k] = buf(0, k);
    w2[k] = buf(1, k);
    CUDA_TRY_S(cudaMemcpyAsync(buf(4, k), psi[k], (size_t)len[k] * 16, cudaMemcpyDeviceToDevice, s));
  }
  const int B = EW_THREADS;
  auto autocorr_at = [&](int step) -> int {
    if (!autocorr) return EVR_OK;
    for (int k = 0; k < n; ++k) {
      if (!autocorr[k]) continue;
      const int nr = nv[k];
      cdot_cols_kernel<<<nr, 256, 0, s>>>(buf(4, k), (const double2*)psi[k], N[k], N[k], (double2*)acb.p);
      CUDA_TRY_S(cudaGetLastError());
      CUDA_TRY_S(cudaMemcpyAsync(autocorr[k] + (size_t)2 * nr * step, acb.p, (size_t)nr * 16, cudaMemcpyDeviceToHost,
                                 s));
      CUDA_TRY_S(cudaStreamSynchronize(s));  // acb is reused by the next context
    }
    return EVR_OK;
  };
  int rc = autocorr_at(0);
  if (rc) return rc;
  std::vector<double> Hmin(n), Hmax(n), E0(n), Esc(n), hnrm(n);
  for (int k = 0; k < n; ++k) {
    Hmin[k] = o[k].Hmin;
    Hmax[k] = o[k].Hmax;
  }
  std::vector<std::vector<double>> cf(n);
  std::vector<double> J;
  std::vector<const double*> src(n);
  std::vector<double*> dst(n);
  std::vector<long long> ld(N.begin(), N.end());
  std::vector<char> pending(n);
  // Recorded steps: with every context in its step and its (E0, Esc, c_k)
  // unchanged since the recording, one whole step -- the start of every
  // context's recurrence, each order's merged H.psi (bound parameter blocks:
  // the source vector alternates between two buffers, so two blocks) with the
  // contexts' ordered accumulations and recurrence updates, and the norms of
  // the last terms into pinned memory -- replays as one CUDA graph.  A context
  // whose step diverges is then redone eagerly, alone with the other diverged
  // ones; the same kernels run either way, so the bits are those of the eager
  // path.
  const bool use_graph = !o[0].no_graph;
  struct StepGraph {
    cudaGraphExec_t exec = nullptr;
    cudaStream_t cs = nullptr;
    double* hnrm = nullptr;
    ~StepGraph() {
      if (exec) cudaGraphExecDestroy(exec);
      if (cs) cudaStreamDestroy(cs);
      if (hnrm) cudaFreeHost(hnrm);
    }
  } sgr;
  std::vector<double> rec_E0(n, 0.0), rec_Esc(n, 0.0);
  std::vector<const double*> src0(n), src1(n);
  std::vector<double*> dstb(n);
  if (use_graph) {
    for (int k = 0; k < n; ++k) {
      src0[k] = (const double*)buf(0, k);
      src1[k] = (const double*)buf(1, k);
      dstb[k] = (double*)buf(2, k);
    }
    if ((rc = multi_bind(m, 0, src0.data(), dstb.data())) || (rc = multi_bind(m, 1, src1.data(), dstb.data())))
      return rc;
    CUDA_TRY_S(cudaStreamCreateWithFlags(&sgr.cs, cudaStreamNonBlocking));
    CUDA_TRY_S(cudaMallocHost(&sgr.hnrm, (size_t)n * 8));
  }
  auto enqueue_step = [&](cudaStream_t st) -> int {  // every context, fixed (E0, Esc, c_k)
    for (int k = 0; k < n; ++k) {
      CUDA_TRY_S(cudaMemcpyAsync(buf(0, k), psi[k], (size_t)len[k] * 16, cudaMemcpyDeviceToDevice, st));
      cscale_kernel<<<ew_grid(len[k]), B, 0, st>>>(buf(3, k), buf(0, k), len[k], cf[k][0], 0.0);
      CUDA_TRY_S(cudaMemsetAsync(buf(1, k), 0, (size_t)len[k] * 16, st));
    }
    for (int ord = 2; ord <= npoly; ++ord) {
      const bool odd = ord & 1;
      int r = multi_launch_bound(m, (ord == 2 || !odd) ? 0 : 1, (ord == 2 || !odd) ? src0.data() : src1.data(),
                                 dstb.data(), E0.data(), Esc.data(), st);
      if (r) return r;
      const bool last = ord == npoly;
      if (last) CUDA_TRY_S(cudaMemsetAsync(nrm.p, 0, (size_t)n * 8, st));
      for (int k = 0; k < n; ++k) {
        if (ord == 2) {
          cheby_update_kernel<<<ew_grid(len[k]), B, 0, st>>>(buf(1, k), buf(2, k), buf(3, k), len[k], 0.0, 0.0, -1.0,
                                                             cf[k][1], last ? nrm.p + k : nullptr);
        } else {
          cheby_update_kernel<<<ew_grid(len[k]), B, 0, st>>>(odd ? buf(0, k) : buf(1, k), buf(2, k), buf(3, k),
                                                             len[k], 1.0, 0.0, -2.0, cf[k][ord - 1],
                                                             last ? nrm.p + k : nullptr);
        }
      }
      CUDA_TRY_S(cudaGetLastError());
    }
    CUDA_TRY_S(cudaMemcpyAsync(sgr.hnrm, nrm.p, (size_t)n * 8, cudaMemcpyDeviceToHost, st));
    return EVR_OK;
  };
  for (int step = 0; step < nsteps; ++step) {
    std::fill(pending.begin(), pending.end(), 1);
    for (int attempt = 0; attempt < 10; ++attempt) {
      if (use_graph && attempt == 0) {  // every context pending: the recorded step
        bool same = sgr.exec != nullptr;
        for (int k = 0; k < n; ++k) {
          const double dE = Hmax[k] - Hmin[k], r0 = 0.5 * dE * dt;
          E0[k] = Hmin[k] + 0.5 * dE;
          Esc[k] = 0.5 * dE;
          if (E0[k] != rec_E0[k] || Esc[k] != rec_Esc[k]) same = false;
          bessel_j(r0, npoly, J);
          cf[k].assign(npoly, 0.0);
          cf[k][0] = J[0];
          for (int q = 1; q < npoly; ++q) cf[k][q] = 2.0 * J[q];
        }
        if (!same) {
          if (sgr.exec) cudaGraphExecDestroy(sgr.exec);
          sgr.exec = nullptr;
          CUDA_TRY_S(cudaStreamSynchronize(s));
          cudaGraph_t gr = nullptr;
          CUDA_TRY_S(cudaStreamBeginCapture(sgr.cs, cudaStreamCaptureModeThreadLocal));
          rc = enqueue_step(sgr.cs);
          cudaError_t ec = cudaStreamEndCapture(sgr.cs, &gr);
          if (rc) {
            if (gr) cudaGraphDestroy(gr);
            return rc;
          }
          if (ec != cudaSuccess) return set_error(EVR_ERR_CUDA, "multi_cheby: graph capture: %s", cudaGetErrorString(ec));
          ec = cudaGraphInstantiate(&sgr.exec, gr, 0);
          cudaGraphDestroy(gr);
          if (ec != cudaSuccess) {
            sgr.exec = nullptr;
            return set_error(EVR_ERR_CUDA, "multi_cheby: graph instantiate: %s", cudaGetErrorString(ec));
          }
          rec_E0 = E0;
          rec_Esc = Esc;
        }
        CUDA_TRY_S(cudaGraphLaunch(sgr.exec, s));
        CUDA_TRY_S(cudaStreamSynchronize(s));
        bool any = false;
        for (int k = 0; k < n; ++k) {
          const double norm_exit = std::fabs(sgr.hnrm[k] * cf[k][npoly - 1]);
          if (!(norm_exit <= 1e15)) {
            Hmax[k] += 0.1 * (Hmax[k] - Hmin[k]);
            any = true;
            continue;
          }
          const double ph = -E0[k] * dt;  // psi = out exp(-i E0 dt)
          cscale_kernel<<<ew_grid(len[k]), B, 0, s>>>((double2*)psi[k], buf(3, k), len[k], std::cos(ph),
                                                      std::sin(ph));
          pending[k] = 0;
        }
        CUDA_TRY_S(cudaGetLastError());
        if (!any) break;
        continue;
      }
      for (int k = 0; k < n; ++k) {
        src[k] = nullptr;
        if (!pending[k]) continue;
        const double dE = Hmax[k] - Hmin[k], r = 0.5 * dE * dt;
        E0[k] = Hmin[k] + 0.5 * dE;
        Esc[k] = 0.5 * dE;
        bessel_j(r, npoly, J);
        cf[k].assign(npoly, 0.0);
        cf[k][0] = J[0];
        for (int q = 1; q < npoly; ++q) cf[k][q] = 2.0 * J[q];
        w1[k] = buf(0, k);
        w2[k] = buf(1, k);
        CUDA_TRY_S(cudaMemcpyAsync(w1[k], psi[k], (size_t)len[k] * 16, cudaMemcpyDeviceToDevice, s));
        cscale_kernel<<<ew_grid(len[k]), B, 0, s>>>(buf(3, k), w1[k], len[k], cf[k][0], 0.0);
        CUDA_TRY_S(cudaMemsetAsync(w2[k], 0, (size_t)len[k] * 16, s));
      }
      // w2 = -i Hs w1, out += c_2 w2 ; then w3 = w1 - 2i Hs w2, out += c_k w3
      for (int ord = 2; ord <= npoly; ++ord) {
        for (int k = 0; k < n; ++k) {
          src[k] = pending[k] ? (const double*)(ord == 2 ? w1[k] : w2[k]) : nullptr;
          dst[k] = (double*)buf(2, k);
        }
        if ((rc = evr_sg4_multi_hpsi(m, src.data(), ld.data(), dst.data(), ld.data(), E0.data(), Esc.data(), s)))
          return rc;
        const bool last = ord == npoly;
        if (last) CUDA_TRY_S(cudaMemsetAsync(nrm.p, 0, (size_t)n * 8, s));
        for (int k = 0; k < n; ++k) {
          if (!pending[k]) continue;
          if (ord == 2) {
            cheby_update_kernel<<<ew_grid(len[k]), B, 0, s>>>(w2[k], buf(2, k), buf(3, k), len[k], 0.0, 0.0, -1.0, cf[k][1],
                                                last ? nrm.p + k : nullptr);
          } else {
            cheby_update_kernel<<<ew_grid(len[k]), B, 0, s>>>(w1[k], buf(2, k), buf(3, k), len[k], 1.0, 0.0, -2.0,
                                                cf[k][ord - 1], last ? nrm.p + k : nullptr);
            std::swap(w1[k], w2[k]);
          }
        }
        CUDA_TRY_S(cudaGetLastError());
      }
      CUDA_TRY_S(cudaMemcpyAsync(hnrm.data(), nrm.p, (size_t)n * 8, cudaMemcpyDeviceToHost, s));
      CUDA_TRY_S(cudaStreamSynchronize(s));
      bool any = false;
      for (int k = 0; k < n; ++k) {
        if (!pending[k]) continue;
        const double norm_exit = std::fabs(hnrm[k] * cf[k][npoly - 1]);
        if (!(norm_exit <= 1e15)) {
          Hmax[k] += 0.1 * (Hmax[k] - Hmin[k]);
          any = true;
          continue;
        }
        const double ph = -E0[k] * dt;  // psi = out exp(-i E0 dt)
        cscale_kernel<<<ew_grid(len[k]), B, 0, s>>>((double2*)psi[k], buf(3, k), len[k], std::cos(ph), std::sin(ph));
        pending[k] = 0;
      }
      CUDA_TRY_S(cudaGetLastError());
      if (!any) break;
    }
    for (int k = 0; k < n; ++k)
      if (pending[k])
        return set_error(EVR_ERR_NUMERIC, "multi_cheby: context %d, step %d did not converge after 10 Hmax increases",
                         k, step);
    if ((rc = autocorr_at(step + 1))) return rc;
  }
  CUDA_TRY_S(cudaStreamSynchronize(s));
  if (npoly_used) *npoly_used = npoly;
  return EVR_OK;
}
