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

extern "C" int evr_sg4_diagonal(evr_sg4_ctx* c, double* diag, void* stream) {
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
  const bool sym = o->symmetrize != 0;
  cudaStream_t s = (cudaStream_t)stream;
  cublasHandle_t h = nullptr;
  CUBLAS_TRY(cublasCreate(&h));
  struct HGuard {
    cublasHandle_t h;
    ~HGuard() { cublasDestroy(h); }
  } hg{h};
  CUBLAS_TRY(cublasSetStream(h, s));
  DevBuf V, HV, X, R, T, W, tmp, Y, th, colsb;
  CUDA_TRY_S(cudaMalloc(&V.p, (size_t)N * mmax * 8));
  CUDA_TRY_S(cudaMalloc(&HV.p, (size_t)N * mmax * 8));
  CUDA_TRY_S(cudaMalloc(&X.p, (size_t)N * nev * 8));
  CUDA_TRY_S(cudaMalloc(&R.p, (size_t)N * nev * 8));
  CUDA_TRY_S(cudaMalloc(&W.p, (size_t)N * std::max(nev, blk) * 8));
  CUDA_TRY_S(cudaMalloc(&tmp.p, (size_t)N * mmax * 8));
  CUDA_TRY_S(cudaMalloc(&T.p, (size_t)mmax * mmax * 8));
  CUDA_TRY_S(cudaMalloc(&Y.p, (size_t)mmax * nev * 8));
  CUDA_TRY_S(cudaMalloc(&th.p, (size_t)nev * 8));
  CUDA_TRY_S(cudaMalloc(&colsb.p, (size_t)blk * 8));
  int* cols = (int*)colsb.p;
  const double one = 1.0, zero = 0.0, mone = -1.0;

  // orthonormalise the nw columns of W against V(:, :m) and among themselves
  // (classical Gram-Schmidt twice, then modified Gram-Schmidt in the block);
  // appends the surviving columns to V and returns how many survived.
  auto add_block = [&](int m, int nw, int& added) -> int {
    added = 0;
    for (int pass = 0; pass < 2 && m > 0; ++pass) {
      CUBLAS_TRY(cublasDgemm(h, CUBLAS_OP_T, CUBLAS_OP_N, m, nw, (int)N, &one, V.p, (int)N, W.p, (int)N, &zero,
                             T.p, mmax));
      CUBLAS_TRY(cublasDgemm(h, CUBLAS_OP_N, CUBLAS_OP_N, (int)N, nw, m, &mone, V.p, (int)N, T.p, mmax, &one,
                             W.p, (int)N));
    }
    for (int j = 0; j < nw; ++j) {
      double* wj = W.p + (size_t)j * N;
      for (int pass = 0; pass < 2; ++pass)
        for (int i = 0; i < added; ++i) {
          double d = 0.0;
          CUBLAS_TRY(cublasDdot(h, (int)N, V.p + (size_t)(m + i) * N, 1, wj, 1, &d));
          const double md = -d;
          CUBLAS_TRY(cublasDaxpy(h, (int)N, &md, V.p + (size_t)(m + i) * N, 1, wj, 1));
        }
      double nrm = 0.0;
      CUBLAS_TRY(cublasDnrm2(h, (int)N, wj, 1, &nrm));
      if (!(nrm > 1e-10) || m + added >= mmax) continue;
      const double inv = 1.0 / nrm;
      CUBLAS_TRY(cublasDscal(h, (int)N, &inv, wj, 1));
      CUDA_TRY_S(cudaMemcpyAsync(V.p + (size_t)(m + added) * N, wj, (size_t)N * 8, cudaMemcpyDeviceToDevice, s));
      ++added;
    }
    return EVR_OK;
  };

  // initial block: the caller's guess, or the first packed functions (lowest L)
  int m = 0, added = 0;
  const int n0 = nguess > 0 && guess ? std::min(nguess, mmax - blk) : nev;
  if (guess && nguess > 0) {
    CUDA_TRY_S(cudaMemcpyAsync(W.p, guess, (size_t)N * std::min(n0, std::max(nev, blk)) * 8,
                               cudaMemcpyDeviceToDevice, s));
  } else {
    unit_block_kernel<<<256, 256, 0, s>>>(W.p, N, n0, 0);
  }
  if ((rc = add_block(0, std::min(n0, std::max(nev, blk)), added))) return rc;
  if ((rc = apply_hs(c, N, added, V.p, HV.p, tmp.p, sym, s))) return rc;
  m = added;

  std::vector<double> Th, w, Z, theta(nev), rn(nev);
  int it = 0;
  bool converged = false;
  for (it = 0; it < o->max_it; ++it) {
    // projected matrix T = V^T HV, symmetrised on the host (sub_hermitic_H)
    CUBLAS_TRY(cublasDgemm(h, CUBLAS_OP_T, CUBLAS_OP_N, m, m, (int)N, &one, V.p, (int)N, HV.p, (int)N, &zero, T.p, m));
    Th.resize((size_t)m * m);
    CUDA_TRY_S(cudaMemcpyAsync(Th.data(), T.p, (size_t)m * m * 8, cudaMemcpyDeviceToHost, s));
    CUDA_TRY_S(cudaStreamSynchronize(s));
    std::vector<double> A((size_t)m * m);
    for (int i = 0; i < m; ++i)
      for (int j = 0; j < m; ++j) A[(size_t)i * m + j] = 0.5 * (Th[i + (size_t)m * j] + Th[j + (size_t)m * i]);
    jacobi_eigen(m, A, w, Z);
    const int k = std::min(nev, m);
    std::vector<double> Yh((size_t)m * k);
    for (int j = 0; j < k; ++j)
      for (int i = 0; i < m; ++i) Yh[i + (size_t)m * j] = Z[(size_t)i * m + j];
    for (int j = 0; j < k; ++j) theta[j] = w[j];
    CUDA_TRY_S(cudaMemcpyAsync(Y.p, Yh.data(), Yh.size() * 8, cudaMemcpyHostToDevice, s));
    CUDA_TRY_S(cudaMemcpyAsync(th.p, theta.data(), (size_t)k * 8, cudaMemcpyHostToDevice, s));
    // Ritz vectors and residuals
    CUBLAS_TRY(cublasDgemm(h, CUBLAS_OP_N, CUBLAS_OP_N, (int)N, k, m, &one, V.p, (int)N, Y.p, m, &zero, X.p, (int)N));
    CUBLAS_TRY(cublasDgemm(h, CUBLAS_OP_N, CUBLAS_OP_N, (int)N, k, m, &one, HV.p, (int)N, Y.p, m, &zero, R.p, (int)N));
    residual_kernel<<<256, 256, 0, s>>>(R.p, X.p, th.p, N, k);
    CUDA_TRY_S(cudaGetLastError());
    for (int j = 0; j < k; ++j) CUBLAS_TRY(cublasDnrm2(h, (int)N, R.p + (size_t)j * N, 1, &rn[j]));
    CUDA_TRY_S(cudaStreamSynchronize(s));
    std::vector<int> todo;
    for (int j = 0; j < k; ++j)
      if (!(rn[j] < o->conv_resi)) todo.push_back(j);
    if (k == nev && todo.empty()) {
      converged = true;
      break;
    }
    for (int j = 0; j < k; ++j)
      if (!std::isfinite(rn[j])) return set_error(EVR_ERR_NUMERIC, "davidson: non-finite residual");
    // restart (keep the Ritz vectors) when the new block does not fit
    const int nnew = std::min((int)todo.size(), blk);
    if (m + nnew > mmax) {
      CUDA_TRY_S(cudaMemcpyAsync(V.p, X.p, (size_t)N * k * 8, cudaMemcpyDeviceToDevice, s));
      CUBLAS_TRY(cublasDgemm(h, CUBLAS_OP_N, CUBLAS_OP_N, (int)N, k, m, &one, HV.p, (int)N, Y.p, m, &zero, tmp.p,
                             (int)N));
      CUDA_TRY_S(cudaMemcpyAsync(HV.p, tmp.p, (size_t)N * k * 8, cudaMemcpyDeviceToDevice, s));
      m = k;
    }
    CUDA_TRY_S(cudaMemcpyAsync(cols, todo.data(), (size_t)nnew * sizeof(int), cudaMemcpyHostToDevice, s));
    precond_kernel<<<256, 256, 0, s>>>(W.p, R.p, diag, th.p, cols, N, nnew);
    CUDA_TRY_S(cudaGetLastError());
    if ((rc = add_block(m, nnew, added))) return rc;
    if (added == 0) return set_error(EVR_ERR_NUMERIC, "davidson: no new direction survived orthogonalisation");
    if ((rc = apply_hs(c, N, added, V.p + (size_t)m * N, HV.p + (size_t)m * N, tmp.p, sym, s))) return rc;
    m += added;
  }
  for (int j = 0; j < nev; ++j) evals[j] = theta[j];
  if (resid)
    for (int j = 0; j < nev; ++j) resid[j] = rn[j];
  if (evecs) CUDA_TRY_S(cudaMemcpyAsync(evecs, X.p, (size_t)N * nev * 8, cudaMemcpyDeviceToDevice, s));
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
  const int G = 2 * 152, B = 256;
  const long long n = st.n;
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
  const int G = 2 * 152, B = 256;
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
//   para_H%E0 (E0 near the middle of the spectrum keeps RK4 stable).  H0 and mu are two contexts on the
// same basis (mu a type-0 operator).  The optimal-control gradient is the
// exact adjoint of those discrete steps: with S = <target|psi_N>,
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
// ------------------------------------------------------------------------

// The two operators of a stage (H0 and mu, or both transposed) run in one
// persistent launch (field_pair_apply); the kernels below join their chunk
// partials in the same order as evr_sg4_hpsi and fuse the stage arithmetic.
struct StageIn {
  const double2* part;         // [2][n_chunks][2] (s, c) partials, H0 first
  const long long* fun_chunk;  // [N+1]
  long long nch2;              // 2 n_chunks: offset of mu's partials
  long long N;
  double2* x;                  // stage input, overwritten by the next stage's input
  double E, E0, h;
};

__device__ __forceinline__ void stage_sums(const StageIn& a, long long n, double2 xv, double& re, double& im,
                                           double& mr, double& mi) {
  const long long c0 = a.fun_chunk[n], c1 = a.fun_chunk[n + 1];
  double hr = join_chunks(a.part, c0, c1, 2, 0), hi = join_chunks(a.part, c0, c1, 2, 1);
  mr = join_chunks(a.part + a.nch2, c0, c1, 2, 0);
  mi = join_chunks(a.part + a.nch2, c0, c1, 2, 1);
  if (a.E0 != 0.0) {  // (H0 - E0) x, as the scaled H.psi writes it
    hr = hr - a.E0 * xv.x;
    hi = hi - a.E0 * xv.y;
  }
  re = hr - a.E * mr;
  im = hi - a.E * mi;
}

__device__ __forceinline__ double2 cmul(double2 t, double cr, double ci) {
  return make_double2(cr * t.x - ci * t.y, cr * t.y + ci * t.x);
}

// forward stage i of an RK4 step y -> y (h = step):
//   k = -i ((H0 - E0) x - E mu x);  [rec = x]
//   i=1: acc = y + h/6 k, x = y + h/2 k     i=2: acc += h/3 k, x = y + h/2 k
//   i=3: acc += h/3 k,    x = y + h k       i=4: y = (acc + h/6 k) e^{-i E0 h}, x = y
__global__ void __launch_bounds__(256) rk_stage_kernel(StageIn a, int stage, double2* y, double2* acc, double2* rec,
                                                       double cr, double ci) {
  for (long long n = blockIdx.x * (long long)blockDim.x + threadIdx.x; n < a.N; n += (long long)gridDim.x * blockDim.x) {
    const double2 xv = a.x[n];
    double re, im, mr, mi;
    stage_sums(a, n, xv, re, im, mr, mi);
    const double2 k = make_double2(im, -re);  // -i (re + i im)
    if (rec) rec[n] = xv;
    const double2 yv = y[n];
    const double h = a.h;
    if (stage == 1) {
      acc[n] = make_double2(fma(h / 6.0, k.x, yv.x), fma(h / 6.0, k.y, yv.y));
      a.x[n] = make_double2(fma(0.5 * h, k.x, yv.x), fma(0.5 * h, k.y, yv.y));
    } else if (stage < 4) {
      const double2 ac = acc[n];
      acc[n] = make_double2(fma(h / 3.0, k.x, ac.x), fma(h / 3.0, k.y, ac.y));
      const double c = stage == 2 ? 0.5 * h : h;
      a.x[n] = make_double2(fma(c, k.x, yv.x), fma(c, k.y, yv.y));
    } else {
      const double2 ac = acc[n];
      double2 t = make_double2(fma(h / 6.0, k.x, ac.x), fma(h / 6.0, k.y, ac.y));
      if (a.E0 != 0.0) t = cmul(t, cr, ci);
      y[n] = t;
      a.x[n] = t;
    }
  }
}

// adjoint stage i (taken 4, 3, 2, 1) of one RK4 step, costate l (phased):
//   sb = +i ((H0^T - E0) kb - E mu^T kb),  kb = x;
//   gpart[block] = -2 Im((mu^T kb)^dagger s_i) = -2 Im(kb^dagger mu s_i), s_i the stage input;
//   i=4: yb = l + sb, x = h/3 l + h sb       i=3: yb += sb, x = h/3 l + h/2 sb
//   i=2: yb += sb, x = h/6 l + h/2 sb        i=1: l = (yb + sb) e^{+i E0 h}, x = h/6 l
// (the last form also prepares the previous step's stage 4)
__global__ void __launch_bounds__(256) rk_adjoint_stage_kernel(StageIn a, int stage, double2* l, double2* yb,
                                                               const double2* s, double* gpart, double cr,
                                                               double ci) {
  double g = 0.0;
  for (long long n = blockIdx.x * (long long)blockDim.x + threadIdx.x; n < a.N; n += (long long)gridDim.x * blockDim.x) {
    const double2 xv = a.x[n];
    double re, im, mr, mi;
    stage_sums(a, n, xv, re, im, mr, mi);
    const double2 sb = make_double2(-im, re);  // +i (re + i im)
    const double2 sv = s[n];
    g = fma(mr, sv.y, fma(-mi, sv.x, g));
    const double2 lv = l[n];
    const double h = a.h;
    if (stage == 4) {
      yb[n] = make_double2(fma(1.0, sb.x, lv.x), fma(1.0, sb.y, lv.y));
      a.x[n] = make_double2(fma(h, sb.x, (h / 3.0) * lv.x), fma(h, sb.y, (h / 3.0) * lv.y));
    } else if (stage > 1) {
      const double2 b = yb[n];
      yb[n] = make_double2(fma(1.0, sb.x, b.x), fma(1.0, sb.y, b.y));
      const double c = stage == 3 ? h / 3.0 : h / 6.0;
      a.x[n] = make_double2(fma(0.5 * h, sb.x, c * lv.x), fma(0.5 * h, sb.y, c * lv.y));
    } else {
      const double2 b = yb[n];
      double2 t = make_double2(fma(1.0, sb.x, b.x), fma(1.0, sb.y, b.y));
      if (a.E0 != 0.0) t = cmul(t, cr, ci);
      l[n] = t;
      a.x[n] = make_double2((h / 6.0) * t.x, (h / 6.0) * t.y);
    }
  }
  __shared__ double sh[32];
  for (int off = 16; off > 0; off >>= 1) g += __shfl_down_sync(0xffffffffu, g, off);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = g;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int k = 0; k < (int)(blockDim.x >> 5); ++k) t += sh[k];
    gpart[blockIdx.x] = -2.0 * t;
  }
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

namespace evr {

// RK4 steps driven by a FieldPair (forward operators), fused per stage
struct FwdSweep {
  FieldPair* fp;
  FieldPairView v;
  double* y;    // device complex N
  double* acc;
  int nblk;
};

static int rk4_step_fused(FwdSweep& w, double E, double E0, double h, double* rec, cudaStream_t s) {
  StageIn a{(const double2*)w.v.part, w.v.fun_chunk, 2 * w.v.n_chunks, w.v.N, (double2*)w.v.x, E, E0, h};
  const double cr = std::cos(E0 * h), ci = -std::sin(E0 * h);
  for (int stage = 1; stage <= 4; ++stage) {
    int rc = field_pair_apply(w.fp, s);
    if (rc) return rc;
    rk_stage_kernel<<<w.nblk, 256, 0, s>>>(a, stage, (double2*)w.y, (double2*)w.acc,
                                           rec ? (double2*)rec + (size_t)(stage - 1) * w.v.N : nullptr, cr, ci);
  }
  CUDA_TRY_S(cudaGetLastError());
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

static int check_field_args(evr_sg4_ctx* H0, evr_sg4_ctx* mu, const evr_rk4_opts* o, const double* E, long long* N) {
  if (!H0 || !mu || !o || !E) return set_error(EVR_ERR_ARG, "rk4: NULL argument");
  long long a[8], b[8];
  int rc = evr_sg4_ctx_sizes(H0, a);
  if (!rc) rc = evr_sg4_ctx_sizes(mu, b);
  if (rc) return rc;
  if (a[0] != b[0] || a[1] != b[1] || a[3] != b[3]) return set_error(EVR_ERR_ARG, "rk4: H0 and mu are on different bases");
  if (o->nsteps < 1 || !(o->dt > 0) || o->checkpoint < 1 || o->nsub < 1)
    return set_error(EVR_ERR_ARG, "rk4: need nsteps >= 1, dt > 0, checkpoint >= 1, nsub >= 1");
  for (int k = 0; k < o->nsteps; ++k)
    if (!std::isfinite(E[k])) return set_error(EVR_ERR_NUMERIC, "rk4: field sample %d is not finite", k);
  *N = a[0];
  return EVR_OK;
}

static int join_blocks(long long N) { return (int)std::max<long long>(1, std::min<long long>((N + 255) / 256, 1024)); }

extern "C" int evr_sg4_rk4_field(evr_sg4_ctx* H0, evr_sg4_ctx* mu, const evr_rk4_opts* o, const double* E, double* psi,
                                 void* stream) {
  long long N = 0;
  int rc = check_field_args(H0, mu, o, E, &N);
  if (rc) return rc;
  if (!psi) return set_error(EVR_ERR_ARG, "rk4: psi is NULL");
  cudaStream_t s = (cudaStream_t)stream;
  PairGuard fp;
  if ((rc = field_pair_create(H0, mu, 0, &fp.p))) return rc;
  DevBuf acc;
  CUDA_TRY_S(cudaMalloc(&acc.p, (size_t)N * 16));
  FwdSweep w{fp.p, field_pair_view(fp.p), psi, acc.p, join_blocks(N)};
  CUDA_TRY_S(cudaMemcpyAsync(w.v.x, psi, (size_t)N * 16, cudaMemcpyDeviceToDevice, s));
  const double hs = o->dt / o->nsub;
  for (int st = 0; st < o->nsteps; ++st)
    for (int u = 0; u < o->nsub; ++u)
      if ((rc = rk4_step_fused(w, E[st], o->E0, hs, nullptr, s))) return rc;
  CUDA_TRY_S(cudaStreamSynchronize(s));
  return EVR_OK;
}

// Optimal-control gradient.  Stream A runs the forward sweep (checkpoints
// every C field intervals, the stages of the last segment kept), then the
// backward sweep segment by segment; stream B recomputes segment k-1 from
// its checkpoint (keeping its stage inputs) while stream A runs the adjoint
// of segment k, with two stage buffers alternating between them.  Both
// streams' launches are small, so they share the SMs.
extern "C" int evr_sg4_oc_gradient(evr_sg4_ctx* H0, evr_sg4_ctx* mu, const evr_rk4_opts* o, const double* E,
                                   const double* psi0, const double* target, double* J, double* grad, void* stream) {
  long long N = 0;
  int rc = check_field_args(H0, mu, o, E, &N);
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
  const int nblk = join_blocks(N);
  PairGuard fwd, adj;
  if ((rc = field_pair_create(H0, mu, 0, &fwd.p)) || (rc = field_pair_create(H0, mu, 1, &adj.p))) return rc;
  DevBuf y, acc, ck, rec, lam, l, yb, gpart, g, ov;
  for (DevBuf* b : {&y, &acc, &lam, &l, &yb}) CUDA_TRY_S(cudaMalloc(&b->p, vb));
  CUDA_TRY_S(cudaMalloc(&ck.p, vb * nseg));                                // checkpoints
  const size_t seg_rec = (size_t)C * nsub * 4 * 2 * N;                    // doubles: stage inputs of a segment
  CUDA_TRY_S(cudaMalloc(&rec.p, seg_rec * 2 * 8));                         // two alternating segment buffers
  CUDA_TRY_S(cudaMalloc(&gpart.p, (size_t)ns * nsub * 4 * nblk * 8));
  CUDA_TRY_S(cudaMalloc(&g.p, (size_t)ns * 8));
  CUDA_TRY_S(cudaMalloc(&ov.p, 16));
  FwdSweep w{fwd.p, field_pair_view(fwd.p), y.p, acc.p, nblk};
  auto rec_of = [&](int seg, int stp, int u) {
    return rec.p + (size_t)(seg & 1) * seg_rec + ((size_t)(stp - seg * C) * nsub + u) * 4 * 2 * N;
  };
  // forward sweep (stream A)
  CUDA_TRY_S(cudaMemcpyAsync(y.p, psi0, vb, cudaMemcpyDeviceToDevice, sA));
  CUDA_TRY_S(cudaMemcpyAsync(w.v.x, psi0, vb, cudaMemcpyDeviceToDevice, sA));
  for (int stp = 0; stp < ns; ++stp) {
    const int seg = stp / C;
    if (stp % C == 0) CUDA_TRY_S(cudaMemcpyAsync(ck.p + (size_t)seg * 2 * N, y.p, vb, cudaMemcpyDeviceToDevice, sA));
    for (int u = 0; u < nsub; ++u)
      if ((rc = rk4_step_fused(w, E[stp], o->E0, hs, seg == nseg - 1 ? rec_of(seg, stp, u) : nullptr, sA))) return rc;
  }
  // S = <target|psi_N>, J = |S|^2, lambda_N = S target
  cdot_cols_kernel<<<1, 256, 0, sA>>>((const double2*)target, (const double2*)y.p, N, N, (double2*)ov.p);
  double2 S;
  CUDA_TRY_S(cudaMemcpyAsync(&S, ov.p, 16, cudaMemcpyDeviceToHost, sA));
  CUDA_TRY_S(cudaStreamSynchronize(sA));  // also: the forward pair and its buffers are free for stream B
  *J = S.x * S.x + S.y * S.y;
  cscale_kernel<<<64, 256, 0, sA>>>((double2*)lam.p, (const double2*)target, N, S.x, S.y);
  const FieldPairView av = field_pair_view(adj.p);
  const double cr = std::cos(o->E0 * hs), ci = std::sin(o->E0 * hs);  // e^{+i E0 h}
  rk_adjoint_start_kernel<<<nblk, 256, 0, sA>>>((double2*)l.p, (const double2*)lam.p, (double2*)av.x, N, hs, cr, ci,
                                                o->E0 != 0.0);
  CUDA_TRY_S(cudaGetLastError());
  cudaEvent_t ready[2] = {sg.ev[0], sg.ev[1]}, freed[2] = {sg.ev[2], sg.ev[3]};
  StageIn a{(const double2*)av.part, av.fun_chunk, 2 * av.n_chunks, N, (double2*)av.x, 0.0, o->E0, hs};
  for (int seg = nseg - 1; seg >= 0; --seg) {
    if (seg > 0) {  // stream B: recompute segment seg-1 into the other buffer
      const int ps = seg - 1;
      if (seg + 1 < nseg) CUDA_TRY_S(cudaStreamWaitEvent(sB, freed[ps & 1], 0));
      CUDA_TRY_S(cudaMemcpyAsync(y.p, ck.p + (size_t)ps * 2 * N, vb, cudaMemcpyDeviceToDevice, sB));
      CUDA_TRY_S(cudaMemcpyAsync(w.v.x, y.p, vb, cudaMemcpyDeviceToDevice, sB));
      for (int stp = ps * C; stp < std::min(ns, (ps + 1) * C); ++stp)
        for (int u = 0; u < nsub; ++u)
          if ((rc = rk4_step_fused(w, E[stp], o->E0, hs, rec_of(ps, stp, u), sB))) return rc;
      CUDA_TRY_S(cudaEventRecord(ready[ps & 1], sB));
    }
    if (seg < nseg - 1) CUDA_TRY_S(cudaStreamWaitEvent(sA, ready[seg & 1], 0));
    const int a0 = seg * C, b0 = std::min(ns, a0 + C);
    for (int stp = b0 - 1; stp >= a0; --stp) {  // stream A: adjoint of segment seg
      a.E = E[stp];
      for (int u = nsub - 1; u >= 0; --u) {
        const double2* st = (const double2*)rec_of(seg, stp, u);
        double* gp = gpart.p + ((size_t)stp * nsub + (nsub - 1 - u)) * 4 * nblk;
        for (int stage = 4; stage >= 1; --stage) {
          if ((rc = field_pair_apply(adj.p, sA))) return rc;
          rk_adjoint_stage_kernel<<<nblk, 256, 0, sA>>>(a, stage, (double2*)l.p, (double2*)yb.p,
                                                        st + (size_t)(stage - 1) * N, gp + (4 - stage) * nblk, cr,
                                                        ci);
        }
      }
    }
    CUDA_TRY_S(cudaGetLastError());
    CUDA_TRY_S(cudaEventRecord(freed[seg & 1], sA));
  }
  rk_grad_sum_kernel<<<(ns + 255) / 256, 256, 0, sA>>>(gpart.p, ns, nsub, nblk, g.p);
  CUDA_TRY_S(cudaMemcpyAsync(grad, g.p, (size_t)ns * 8, cudaMemcpyDeviceToHost, sA));
  CUDA_TRY_S(cudaStreamSynchronize(sA));
  CUDA_TRY_S(cudaStreamSynchronize(sB));
  return EVR_OK;
}

// ------------------------------------------------------------------------
// Chebyshev propagation of every context of a complex multi-context plan in
// lock-step (the batched uneven-instance workload): each expansion order is
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
  const int G = 2 * 152, B = 256;
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
  for (int step = 0; step < nsteps; ++step) {
    std::fill(pending.begin(), pending.end(), 1);
    for (int attempt = 0; attempt < 10; ++attempt) {
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
        cscale_kernel<<<G, B, 0, s>>>(buf(3, k), w1[k], len[k], cf[k][0], 0.0);
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
            cheby_update_kernel<<<G, B, 0, s>>>(w2[k], buf(2, k), buf(3, k), len[k], 0.0, 0.0, -1.0, cf[k][1],
                                                last ? nrm.p + k : nullptr);
          } else {
            cheby_update_kernel<<<G, B, 0, s>>>(w1[k], buf(2, k), buf(3, k), len[k], 1.0, 0.0, -2.0,
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
        cscale_kernel<<<G, B, 0, s>>>((double2*)psi[k], buf(3, k), len[k], std::cos(ph), std::sin(ph));
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
