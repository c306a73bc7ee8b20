// sg4_solvers.cu -- the callers of the SG4 H.psi on the device: block
// Davidson (sub_propagation_Davidson, SRC/sub_propagation/
// sub_module_Davidson.f90:59-767) and the exact diagonal used as its
// preconditioner.  Host C++ drives the iteration; every vector operation and
// every H.psi stays on the GPU (cuBLAS DGEMM for the small dense products of
// the subspace), only the m x m projected matrix goes to the host.
#include <cublas_v2.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "evr_sg4.h"
#include "sg4_internal.h"

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
  for (int step = 0; step < o->nsteps; ++step) {
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
// field intervals and each segment is recomputed (keeping its stages and
// mu s_i) before its backward sweep, so the gradient costs about three
// forward propagations.  Each field interval dt is integrated with nsub RK4
// steps of dt/nsub (E held over the interval), which keeps fixed-step RK4
// accurate when dt times the spectral range is too large for one step.
// The reference's control update (build_field, SRC/sub_propagation/
// sub_control.f90:907-1010) uses the continuous-time form of the same
// derivative, -2 Im(S* <chi(t)|mu|psi(t)>).
// ------------------------------------------------------------------------

// k = -i (h1 - E h2)  [sign = -1]   or   k = +i (h1 - E h2)  [sign = +1]
__global__ void field_f_kernel(double2* k, const double2* h1, const double2* h2, long long n, double E, double sign) {
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
    const double2 a = h1[e], b = h2[e];
    const double re = a.x - E * b.x, im = a.y - E * b.y;
    k[e] = make_double2(-sign * im, sign * re);  // sign * i * (re + i im)
  }
}

// out = x + a y   (complex vectors, real a)
__global__ void zaxpy_kernel(double2* out, const double2* x, double a, const double2* y, long long n) {
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
    const double2 u = x[e], v = y[e];
    out[e] = make_double2(fma(a, v.x, u.x), fma(a, v.y, u.y));
  }
}

// acc[0] += -2 Im(a^dagger b) = -2 sum (a.x b.y - a.y b.x)  (one block, deterministic)
__global__ void grad_term_kernel(const double2* a, const double2* b, long long n, double* acc) {
  double s = 0.0;
  for (long long e = threadIdx.x; e < n; e += blockDim.x) {
    const double2 x = a[e], y = b[e];
    s = fma(x.x, y.y, fma(-x.y, y.x, s));
  }
  __shared__ double sh[32];
  for (int off = 16; off > 0; off >>= 1) s += __shfl_down_sync(0xffffffffu, s, off);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int k = 0; k < (int)(blockDim.x >> 5); ++k) t += sh[k];
    acc[0] += -2.0 * t;
  }
}

namespace evr {

struct FieldOps {
  evr_sg4_ctx* H0;
  evr_sg4_ctx* mu;
  double E0;   // energy shift of fcn_field's sub_scaledOpPsi(WP, dWP, para_H%E0, ONE)
  long long N;
  cudaStream_t s;
  double* h1;  // scratch N complex
  double* h2;
};

// k = -i (H0 x - E mu x); optionally keeps mu x in mux
static int field_f(FieldOps& f, const double* x, double* k, double E, double* mux) {
  double* m = mux ? mux : f.h2;
  int rc = evr_sg4_apply(f.H0, EVR_APPLY_COMPLEX, 1, x, f.N, f.h1, f.N, f.E0, 1.0, f.s);
  if (rc) return rc;
  if ((rc = evr_sg4_apply(f.mu, EVR_APPLY_COMPLEX, 1, x, f.N, m, f.N, 0.0, 1.0, f.s))) return rc;
  field_f_kernel<<<64, 256, 0, f.s>>>((double2*)k, (const double2*)f.h1, (const double2*)m, f.N, E, -1.0);
  CUDA_TRY_S(cudaGetLastError());
  return EVR_OK;
}

// sb = i (H0^T kb - E mu^T kb)
static int field_fadj(FieldOps& f, const double* kb, double* sb, double E) {
  int rc = evr_sg4_apply(f.H0, EVR_APPLY_COMPLEX | EVR_APPLY_TRANSPOSE, 1, kb, f.N, f.h1, f.N, f.E0, 1.0, f.s);
  if (rc) return rc;
  if ((rc = evr_sg4_apply(f.mu, EVR_APPLY_COMPLEX | EVR_APPLY_TRANSPOSE, 1, kb, f.N, f.h2, f.N, 0.0, 1.0, f.s)))
    return rc;
  field_f_kernel<<<64, 256, 0, f.s>>>((double2*)sb, (const double2*)f.h1, (const double2*)f.h2, f.N, E, +1.0);
  CUDA_TRY_S(cudaGetLastError());
  return EVR_OK;
}

// one RK4 step y -> y (in place); st (if given) receives s1..s4 then mu s1..mu s4
static int rk4_step(FieldOps& f, double* y, double E, double dt, double* st, double* k, double* acc, double* sbuf) {
  const long long n = f.N;
  auto S = [&](int i) { return st ? st + (size_t)i * 2 * n : sbuf; };
  auto M = [&](int i) { return st ? st + (size_t)(4 + i) * 2 * n : nullptr; };
  // acc = y ; s1 = y
  CUDA_TRY_S(cudaMemcpyAsync(acc, y, (size_t)n * 16, cudaMemcpyDeviceToDevice, f.s));
  double* s1 = S(0);
  if (st) CUDA_TRY_S(cudaMemcpyAsync(s1, y, (size_t)n * 16, cudaMemcpyDeviceToDevice, f.s));
  int rc = field_f(f, st ? s1 : y, k, E, M(0));                          // k1
  if (rc) return rc;
  zaxpy_kernel<<<64, 256, 0, f.s>>>((double2*)acc, (const double2*)acc, dt / 6.0, (const double2*)k, n);
  double* s2 = S(1);
  zaxpy_kernel<<<64, 256, 0, f.s>>>((double2*)s2, (const double2*)y, 0.5 * dt, (const double2*)k, n);
  if ((rc = field_f(f, s2, k, E, M(1)))) return rc;                      // k2
  zaxpy_kernel<<<64, 256, 0, f.s>>>((double2*)acc, (const double2*)acc, dt / 3.0, (const double2*)k, n);
  double* s3 = st ? S(2) : s2;
  zaxpy_kernel<<<64, 256, 0, f.s>>>((double2*)s3, (const double2*)y, 0.5 * dt, (const double2*)k, n);
  if ((rc = field_f(f, s3, k, E, M(2)))) return rc;                      // k3
  zaxpy_kernel<<<64, 256, 0, f.s>>>((double2*)acc, (const double2*)acc, dt / 3.0, (const double2*)k, n);
  double* s4 = st ? S(3) : s3;
  zaxpy_kernel<<<64, 256, 0, f.s>>>((double2*)s4, (const double2*)y, dt, (const double2*)k, n);
  if ((rc = field_f(f, s4, k, E, M(3)))) return rc;                      // k4
  zaxpy_kernel<<<64, 256, 0, f.s>>>((double2*)y, (const double2*)acc, dt / 6.0, (const double2*)k, n);
  if (f.E0 != 0.0)  // WP = WP exp(-i E0 dt) (march_RK4_field :533-535)
    cscale_kernel<<<64, 256, 0, f.s>>>((double2*)y, (const double2*)y, n, std::cos(f.E0 * dt), -std::sin(f.E0 * dt));
  CUDA_TRY_S(cudaGetLastError());
  return EVR_OK;
}

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

extern "C" int evr_sg4_rk4_field(evr_sg4_ctx* H0, evr_sg4_ctx* mu, const evr_rk4_opts* o, const double* E, double* psi,
                                 void* stream) {
  long long N = 0;
  int rc = check_field_args(H0, mu, o, E, &N);
  if (rc) return rc;
  if (!psi) return set_error(EVR_ERR_ARG, "rk4: psi is NULL");
  cudaStream_t s = (cudaStream_t)stream;
  DevBuf h1, h2, k, acc, sb;
  for (DevBuf* b : {&h1, &h2, &k, &acc, &sb}) CUDA_TRY_S(cudaMalloc(&b->p, (size_t)N * 16));
  FieldOps f{H0, mu, o->E0, N, s, h1.p, h2.p};
  const int nsub = o->nsub;
  for (int st = 0; st < o->nsteps; ++st)
    for (int u = 0; u < nsub; ++u)
      if ((rc = rk4_step(f, psi, E[st], o->dt / nsub, nullptr, k.p, acc.p, sb.p))) return rc;
  CUDA_TRY_S(cudaStreamSynchronize(s));
  return EVR_OK;
}

extern "C" int evr_sg4_oc_gradient(evr_sg4_ctx* H0, evr_sg4_ctx* mu, const evr_rk4_opts* o, const double* E,
                                   const double* psi0, const double* target, double* J, double* grad, void* stream) {
  long long N = 0;
  int rc = check_field_args(H0, mu, o, E, &N);
  if (rc) return rc;
  if (!psi0 || !target || !J || !grad) return set_error(EVR_ERR_ARG, "oc_gradient: NULL argument");
  cudaStream_t s = (cudaStream_t)stream;
  const int C = o->checkpoint, ns = o->nsteps, nseg = (ns + C - 1) / C;
  const size_t vb = (size_t)N * 16;
  DevBuf h1, h2, k, acc, sb, y, ck, st, lam, yb, kb1, kb2, kb3, kb4, sv, g, ov;
  for (DevBuf* b : {&h1, &h2, &k, &acc, &sb, &y, &lam, &yb, &kb1, &kb2, &kb3, &kb4, &sv})
    CUDA_TRY_S(cudaMalloc(&b->p, vb));
  CUDA_TRY_S(cudaMalloc(&ck.p, vb * (nseg + 1)));            // checkpoints
  const int nsub = o->nsub;
  const double hs = o->dt / nsub;                            // RK4 step inside a field interval
  CUDA_TRY_S(cudaMalloc(&st.p, vb * 8 * (size_t)C * nsub));  // stages of one segment
  CUDA_TRY_S(cudaMalloc(&g.p, (size_t)ns * 8));
  CUDA_TRY_S(cudaMalloc(&ov.p, 16));
  CUDA_TRY_S(cudaMemsetAsync(g.p, 0, (size_t)ns * 8, s));
  FieldOps f{H0, mu, o->E0, N, s, h1.p, h2.p};
  // forward sweep, keeping psi at the start of every segment
  CUDA_TRY_S(cudaMemcpyAsync(y.p, psi0, vb, cudaMemcpyDeviceToDevice, s));
  for (int stp = 0; stp < ns; ++stp) {
    if (stp % C == 0) CUDA_TRY_S(cudaMemcpyAsync(ck.p + (size_t)(stp / C) * 2 * N, y.p, vb, cudaMemcpyDeviceToDevice, s));
    for (int u = 0; u < nsub; ++u)
      if ((rc = rk4_step(f, y.p, E[stp], hs, nullptr, k.p, acc.p, sb.p))) return rc;
  }
  // S = <target|psi_N>, J = |S|^2, lambda_N = S target
  cdot_cols_kernel<<<1, 256, 0, s>>>((const double2*)target, (const double2*)y.p, N, N, (double2*)ov.p);
  double2 S;
  CUDA_TRY_S(cudaMemcpyAsync(&S, ov.p, 16, cudaMemcpyDeviceToHost, s));
  CUDA_TRY_S(cudaStreamSynchronize(s));
  *J = S.x * S.x + S.y * S.y;
  cscale_kernel<<<64, 256, 0, s>>>((double2*)lam.p, (const double2*)target, N, S.x, S.y);
  // backward sweep, segment by segment
  for (int seg = nseg - 1; seg >= 0; --seg) {
    const int a = seg * C, b = std::min(ns, a + C);
    CUDA_TRY_S(cudaMemcpyAsync(y.p, ck.p + (size_t)seg * 2 * N, vb, cudaMemcpyDeviceToDevice, s));
    for (int stp = a; stp < b; ++stp)  // recompute, keeping s_i and mu s_i of every RK4 step
      for (int u = 0; u < nsub; ++u)
        if ((rc = rk4_step(f, y.p, E[stp], hs, st.p + ((size_t)(stp - a) * nsub + u) * 8 * 2 * N, k.p, acc.p,
                           sb.p)))
          return rc;
    for (int sub = (b - a) * nsub - 1; sub >= 0; --sub) {
      const int stp = a + sub / nsub;
      const double* sts = st.p + (size_t)sub * 8 * 2 * N;
      auto MU = [&](int i) { return (const double2*)(sts + (size_t)(4 + i) * 2 * N); };
      const double h = hs, Ek = E[stp];
      double* gk = g.p + stp;
      const double2* L = (const double2*)lam.p;
      // the step ends with the phase exp(-i E0 h): its adjoint multiplies l by exp(+i E0 h)
      if (o->E0 != 0.0)
        cscale_kernel<<<64, 256, 0, s>>>((double2*)lam.p, (const double2*)lam.p, N, std::cos(o->E0 * h),
                                         std::sin(o->E0 * h));
      // yb = l; kb4 = h/6 l
      CUDA_TRY_S(cudaMemcpyAsync(yb.p, lam.p, vb, cudaMemcpyDeviceToDevice, s));
      cscale_kernel<<<64, 256, 0, s>>>((double2*)kb4.p, L, N, h / 6.0, 0.0);
      if ((rc = field_fadj(f, kb4.p, sv.p, Ek))) return rc;  // sb4
      grad_term_kernel<<<1, 256, 0, s>>>((const double2*)kb4.p, MU(3), N, gk);
      zaxpy_kernel<<<64, 256, 0, s>>>((double2*)yb.p, (const double2*)yb.p, 1.0, (const double2*)sv.p, N);
      cscale_kernel<<<64, 256, 0, s>>>((double2*)kb3.p, L, N, h / 3.0, 0.0);
      zaxpy_kernel<<<64, 256, 0, s>>>((double2*)kb3.p, (const double2*)kb3.p, h, (const double2*)sv.p, N);
      if ((rc = field_fadj(f, kb3.p, sv.p, Ek))) return rc;  // sb3
      grad_term_kernel<<<1, 256, 0, s>>>((const double2*)kb3.p, MU(2), N, gk);
      zaxpy_kernel<<<64, 256, 0, s>>>((double2*)yb.p, (const double2*)yb.p, 1.0, (const double2*)sv.p, N);
      cscale_kernel<<<64, 256, 0, s>>>((double2*)kb2.p, L, N, h / 3.0, 0.0);
      zaxpy_kernel<<<64, 256, 0, s>>>((double2*)kb2.p, (const double2*)kb2.p, 0.5 * h, (const double2*)sv.p, N);
      if ((rc = field_fadj(f, kb2.p, sv.p, Ek))) return rc;  // sb2
      grad_term_kernel<<<1, 256, 0, s>>>((const double2*)kb2.p, MU(1), N, gk);
      zaxpy_kernel<<<64, 256, 0, s>>>((double2*)yb.p, (const double2*)yb.p, 1.0, (const double2*)sv.p, N);
      cscale_kernel<<<64, 256, 0, s>>>((double2*)kb1.p, L, N, h / 6.0, 0.0);
      zaxpy_kernel<<<64, 256, 0, s>>>((double2*)kb1.p, (const double2*)kb1.p, 0.5 * h, (const double2*)sv.p, N);
      if ((rc = field_fadj(f, kb1.p, sv.p, Ek))) return rc;  // sb1
      grad_term_kernel<<<1, 256, 0, s>>>((const double2*)kb1.p, MU(0), N, gk);
      zaxpy_kernel<<<64, 256, 0, s>>>((double2*)lam.p, (const double2*)yb.p, 1.0, (const double2*)sv.p, N);
      CUDA_TRY_S(cudaGetLastError());
    }
  }
  CUDA_TRY_S(cudaMemcpyAsync(grad, g.p, (size_t)ns * 8, cudaMemcpyDeviceToHost, s));
  CUDA_TRY_S(cudaStreamSynchronize(s));
  return EVR_OK;
}
