// FP64 spectral stage: generalized symmetric eigensolve of the pencil (S, M),
// the spectral objective and its matrix adjoints, and the FP64 maps between
// the hidden-layer pencil and the K x K pencil.
//
// All matrices are square and symmetric, so row- and column-major storage
// coincide; eigenvectors are returned with row k holding eigenvector k.
#include <cublas_v2.h>
#include <cusolverDn.h>
#include <cmath>
#include <vector>
#include "elementwise.cuh"

namespace neb {

namespace {
struct Handles {
  cusolverDnHandle_t solver = nullptr;
  cublasHandle_t blas = nullptr;
  ~Handles() {
    if (solver) cusolverDnDestroy(solver);
    if (blas) cublasDestroy(blas);
  }
};
thread_local Handles g_handles;

int handles(cudaStream_t stream, cusolverDnHandle_t* s, cublasHandle_t* b) {
  if (!g_handles.solver && cusolverDnCreate(&g_handles.solver) != CUSOLVER_STATUS_SUCCESS) {
    set_error("cusolverDnCreate failed");
    return NEB_ERR_CUDA;
  }
  if (!g_handles.blas && cublasCreate(&g_handles.blas) != CUBLAS_STATUS_SUCCESS) {
    set_error("cublasCreate failed");
    return NEB_ERR_CUDA;
  }
  cusolverDnSetStream(g_handles.solver, stream);
  cublasSetStream(g_handles.blas, stream);
  cublasSetPointerMode(g_handles.blas, CUBLAS_POINTER_MODE_HOST);
  if (s) *s = g_handles.solver;
  if (b) *b = g_handles.blas;
  return NEB_OK;
}

size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

// Row-major C[m][n] = alpha op(A) op(B) + beta C through column-major cuBLAS
// (C^T = op(B)^T op(A)^T).
int gemm_rm(cublasHandle_t h, bool ta, bool tb, int m, int n, int k, double alpha,
            const double* A, int lda, const double* B, int ldb, double beta, double* C, int ldc) {
  cublasStatus_t st = cublasDgemm(h, tb ? CUBLAS_OP_T : CUBLAS_OP_N, ta ? CUBLAS_OP_T : CUBLAS_OP_N,
                                  n, m, k, &alpha, B, ldb, A, lda, &beta, C, ldc);
  if (st != CUBLAS_STATUS_SUCCESS) {
    set_error("cublasDgemm failed (%d)", (int)st);
    return NEB_ERR_CUDA;
  }
  return NEB_OK;
}
}  // namespace

}  // namespace neb

using namespace neb;

extern "C" size_t neb_spectral_workspace_bytes(int m) {
  if (m <= 0) return 0;
  cusolverDnHandle_t s;
  if (handles(nullptr, &s, nullptr) != NEB_OK) return 0;
  int lwork = 0;
  if (cusolverDnDsygvd_bufferSize(s, CUSOLVER_EIG_TYPE_1, CUSOLVER_EIG_MODE_VECTOR,
                                  CUBLAS_FILL_MODE_LOWER, m, nullptr, m, nullptr, m, nullptr,
                                  &lwork) != CUSOLVER_STATUS_SUCCESS)
    return 0;
  size_t mm = (size_t)m * m * sizeof(double);
  return align256(mm) * 2 + align256((size_t)lwork * sizeof(double));
}

extern "C" int neb_spectral(int m, const double* M, const double* S, const double* c, double* lam,
                            double* V, double* G_M, double* G_S, double* loss, int* info,
                            void* workspace, size_t workspace_bytes, neb_stream_t stream_) {
  NEB_REQUIRE(m > 0, "neb_spectral: m must be positive");
  NEB_REQUIRE(M && S && c && lam && V && G_M && G_S && loss && info, "neb_spectral: null pointer");
  cudaStream_t stream = (cudaStream_t)stream_;
  cusolverDnHandle_t sol;
  cublasHandle_t blas;
  int st = handles(stream, &sol, &blas);
  if (st) return st;
  int lwork = 0;
  if (cusolverDnDsygvd_bufferSize(sol, CUSOLVER_EIG_TYPE_1, CUSOLVER_EIG_MODE_VECTOR,
                                  CUBLAS_FILL_MODE_LOWER, m, V, m, (double*)workspace, m, lam,
                                  &lwork) != CUSOLVER_STATUS_SUCCESS) {
    set_error("cusolverDnDsygvd_bufferSize failed");
    return NEB_ERR_CUDA;
  }
  size_t mm = (size_t)m * m * sizeof(double);
  size_t need = align256(mm) * 2 + align256((size_t)lwork * sizeof(double));
  if (workspace_bytes < need || workspace == nullptr) {
    set_error("neb_spectral: workspace %zu < %zu bytes", workspace_bytes, need);
    return NEB_ERR_WORKSPACE;
  }
  char* ws = (char*)workspace;
  double* Mw = (double*)ws;
  double* Tw = (double*)(ws + align256(mm));
  double* work = (double*)(ws + 2 * align256(mm));
  NEB_CUDA_CHECK(cudaMemcpyAsync(Mw, M, mm, cudaMemcpyDeviceToDevice, stream));
  NEB_CUDA_CHECK(cudaMemcpyAsync(V, S, mm, cudaMemcpyDeviceToDevice, stream));
  // S v = lam M v; on exit V (column-major) holds M-orthonormal eigenvectors
  cusolverStatus_t cs;
  {
  KernelScope ks("cusolver_dsygvd", stream, 9.0 * m * (double)m * m, 0);
  cs = cusolverDnDsygvd(sol, CUSOLVER_EIG_TYPE_1, CUSOLVER_EIG_MODE_VECTOR,
                                         CUBLAS_FILL_MODE_LOWER, m, V, m, Mw, m, lam, work, lwork,
                                         info);
  }
  if (cs != CUSOLVER_STATUS_SUCCESS) {
    set_error("cusolverDnDsygvd failed (%d)", (int)cs);
    return NEB_ERR_SOLVER;
  }
  int threads = 256;
  int blocks = (int)ceil_div((int64_t)m * m, threads);
  // G_S = V diag(c) V^T, G_M = -V diag(c lam) V^T (column-major V: column j =
  // eigenvector j; symmetric results)
  double one = 1.0, zero = 0.0, mone = -1.0;
  {
    KernelScope ks("scale_columns", stream, 0, 16.0 * m * m);
    scale_columns<<<blocks, threads, 0, stream>>>(V, c, nullptr, m, Tw);
    NEB_LAUNCH_CHECK();
  }
  {
    KernelScope ks("cublas_dgemm", stream, 2.0 * m * (double)m * m, 24.0 * m * m);
    if (cublasDgemm(blas, CUBLAS_OP_N, CUBLAS_OP_T, m, m, m, &one, Tw, m, V, m, &zero, G_S, m) !=
        CUBLAS_STATUS_SUCCESS) {
      set_error("cublasDgemm (G_S) failed");
      return NEB_ERR_CUDA;
    }
  }
  {
    KernelScope ks("scale_columns", stream, 0, 16.0 * m * m);
    scale_columns<<<blocks, threads, 0, stream>>>(V, c, lam, m, Tw);
    NEB_LAUNCH_CHECK();
  }
  {
    KernelScope ks("cublas_dgemm", stream, 2.0 * m * (double)m * m, 24.0 * m * m);
    if (cublasDgemm(blas, CUBLAS_OP_N, CUBLAS_OP_T, m, m, m, &mone, Tw, m, V, m, &zero, G_M, m) !=
        CUBLAS_STATUS_SUCCESS) {
      set_error("cublasDgemm (G_M) failed");
      return NEB_ERR_CUDA;
    }
  }
  {
    KernelScope ks("weighted_sum", stream, 0, 16.0 * m);
    weighted_sum<<<1, 256, 0, stream>>>(c, lam, m, loss, info);
    NEB_LAUNCH_CHECK();
  }
  return NEB_OK;
}

extern "C" size_t neb_pencil_workspace_bytes(int K, int H) {
  return align256((size_t)K * H * sizeof(double)) * 2;
}

extern "C" int neb_pencil_project(int K, int H, const double* W, const double* A_M,
                                  const double* A_S, double* M, double* S, void* workspace,
                                  size_t workspace_bytes, neb_stream_t stream_) {
  NEB_REQUIRE(K > 0 && H > 0 && W && A_M && A_S && M && S, "neb_pencil_project: bad arguments");
  if (workspace_bytes < neb_pencil_workspace_bytes(K, H) || !workspace) {
    set_error("neb_pencil_project: workspace too small");
    return NEB_ERR_WORKSPACE;
  }
  cublasHandle_t blas;
  int st = handles((cudaStream_t)stream_, nullptr, &blas);
  if (st) return st;
  double* T1 = (double*)workspace;
  if ((st = gemm_rm(blas, false, false, K, H, H, 1.0, W, H, A_M, H, 0.0, T1, H))) return st;
  if ((st = gemm_rm(blas, false, true, K, K, H, 1.0, T1, H, W, H, 0.0, M, K))) return st;
  if ((st = gemm_rm(blas, false, false, K, H, H, 1.0, W, H, A_S, H, 0.0, T1, H))) return st;
  if ((st = gemm_rm(blas, false, true, K, K, H, 1.0, T1, H, W, H, 0.0, S, K))) return st;
  return NEB_OK;
}

extern "C" int neb_pencil_pullback(int K, int H, const double* W, const double* A_M,
                                   const double* A_S, const double* G_M, const double* G_S,
                                   double* G_Mh, double* G_Sh, double* gW, void* workspace,
                                   size_t workspace_bytes, neb_stream_t stream_) {
  NEB_REQUIRE(K > 0 && H > 0 && W && A_M && A_S && G_M && G_S && G_Mh && G_Sh,
              "neb_pencil_pullback: bad arguments");
  if (workspace_bytes < neb_pencil_workspace_bytes(K, H) || !workspace) {
    set_error("neb_pencil_pullback: workspace too small");
    return NEB_ERR_WORKSPACE;
  }
  cublasHandle_t blas;
  int st = handles((cudaStream_t)stream_, nullptr, &blas);
  if (st) return st;
  double* T1 = (double*)workspace;
  double* T2 = (double*)((char*)workspace + align256((size_t)K * H * sizeof(double)));
  // G_h = W^T G W
  if ((st = gemm_rm(blas, false, false, K, H, K, 1.0, G_M, K, W, H, 0.0, T1, H))) return st;
  if ((st = gemm_rm(blas, true, false, H, H, K, 1.0, W, H, T1, H, 0.0, G_Mh, H))) return st;
  if ((st = gemm_rm(blas, false, false, K, H, K, 1.0, G_S, K, W, H, 0.0, T2, H))) return st;
  if ((st = gemm_rm(blas, true, false, H, H, K, 1.0, W, H, T2, H, 0.0, G_Sh, H))) return st;
  if (gW) {
    // gW = 2 (G_M W A_M + G_S W A_S) = 2 (T1 A_M + T2 A_S)
    if ((st = gemm_rm(blas, false, false, K, H, H, 2.0, T1, H, A_M, H, 0.0, gW, H))) return st;
    if ((st = gemm_rm(blas, false, false, K, H, H, 2.0, T2, H, A_S, H, 1.0, gW, H))) return st;
  }
  return NEB_OK;
}

// --------------------------------------------------- finite (range) pencil
// Rank-revealing FP64 route for pencils whose mass matrix may be singular:
// M = Q diag(e) Q^T (ascending e); the r eigenvalues above rank_rtol * e_max
// span range(M) (the eigenvalue-ratio rank test of paper_rollout.py:180-186);
// the finite pencil is C = Q_r^T S Q_r with Q_r = Q[:, m-r:] diag(e^-1/2),
// C = Y diag(lam) Y^T, V = Q_r Y (M-orthonormal), the objective and its
// adjoints over those r pairs.  When r = m this equals the sygvd route.
namespace neb {
namespace {
__global__ void range_basis(const double* __restrict__ Q, const double* __restrict__ e, int m,
                            int r, double* __restrict__ Qr) {
  int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (idx >= (int64_t)m * r) return;
  int j = (int)(idx / m);
  int col = m - r + j;
  Qr[idx] = Q[(int64_t)col * m + idx % m] / sqrt(e[col]);
}

// out[i + j rows] = V[i + j rows] * c_j (* lam_j)
__global__ void scale_cols(const double* __restrict__ V, int rows, int cols,
                           const double* __restrict__ c, const double* __restrict__ lam,
                           double* __restrict__ out) {
  int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (idx >= (int64_t)rows * cols) return;
  int j = (int)(idx / rows);
  out[idx] = V[idx] * c[j] * (lam ? lam[j] : 1.0);
}

int syevd_lwork(cusolverDnHandle_t s, int n, int* lwork) {
  if (cusolverDnDsyevd_bufferSize(s, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER, n, nullptr,
                                  n, nullptr, lwork) != CUSOLVER_STATUS_SUCCESS) {
    set_error("cusolverDnDsyevd_bufferSize failed");
    return NEB_ERR_CUDA;
  }
  return NEB_OK;
}
}  // namespace
}  // namespace neb

extern "C" size_t neb_spectral_range_workspace_bytes(int m) {
  if (m <= 0) return 0;
  cusolverDnHandle_t s;
  if (handles(nullptr, &s, nullptr) != NEB_OK) return 0;
  int lwork = 0;
  if (syevd_lwork(s, m, &lwork) != NEB_OK) return 0;
  size_t mm = align256((size_t)m * m * sizeof(double));
  return 4 * mm + align256((size_t)m * sizeof(double)) + 256 +
         align256((size_t)lwork * sizeof(double));
}

extern "C" int neb_spectral_range(int m, const double* M, const double* S, const double* c,
                                  double rank_rtol, double* lam, double* V, double* G_M,
                                  double* G_S, double* loss, int* rank, int* info,
                                  void* workspace, size_t workspace_bytes,
                                  neb_stream_t stream_) {
  NEB_REQUIRE(m > 0 && rank_rtol >= 0.0, "neb_spectral_range: bad arguments");
  NEB_REQUIRE(M && S && c && lam && V && G_M && G_S && loss && rank && info,
              "neb_spectral_range: null pointer");
  cudaStream_t stream = (cudaStream_t)stream_;
  cusolverDnHandle_t sol;
  cublasHandle_t blas;
  int st = handles(stream, &sol, &blas);
  if (st) return st;
  if (workspace_bytes < neb_spectral_range_workspace_bytes(m) || !workspace) {
    set_error("neb_spectral_range: workspace too small");
    return NEB_ERR_WORKSPACE;
  }
  int lwork = 0;
  if ((st = syevd_lwork(sol, m, &lwork))) return st;
  const size_t mm = align256((size_t)m * m * sizeof(double));
  char* ws = (char*)workspace;
  double* Q = (double*)ws;
  double* Qr = (double*)(ws + mm);
  double* T = (double*)(ws + 2 * mm);
  double* Cm = (double*)(ws + 3 * mm);
  double* e = (double*)(ws + 4 * mm);
  int* dinfo = (int*)(ws + 4 * mm + align256((size_t)m * sizeof(double)));
  double* work = (double*)(ws + 4 * mm + align256((size_t)m * sizeof(double)) + 256);
  NEB_CUDA_CHECK(cudaMemcpyAsync(Q, M, (size_t)m * m * sizeof(double), cudaMemcpyDeviceToDevice,
                                 stream));
  {
    KernelScope ks("cusolver_dsyevd", stream, 9.0 * m * (double)m * m, 0);
    if (cusolverDnDsyevd(sol, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER, m, Q, m, e, work,
                         lwork, dinfo) != CUSOLVER_STATUS_SUCCESS) {
      set_error("cusolverDnDsyevd (mass matrix) failed");
      return NEB_ERR_SOLVER;
    }
  }
  // the rank decides the size of the finite pencil: read e (m doubles) back
  std::vector<double> eh((size_t)m);
  int ih = 0;
  NEB_CUDA_CHECK(cudaMemcpyAsync(eh.data(), e, (size_t)m * sizeof(double), cudaMemcpyDeviceToHost,
                                 stream));
  NEB_CUDA_CHECK(cudaMemcpyAsync(&ih, dinfo, sizeof(int), cudaMemcpyDeviceToHost, stream));
  NEB_CUDA_CHECK(cudaStreamSynchronize(stream));
  if (ih != 0) {
    set_error("neb_spectral_range: eigensolve of the mass matrix failed (info %d)", ih);
    return NEB_ERR_SOLVER;
  }
  const double emax = eh[(size_t)m - 1];
  if (!std::isfinite(emax)) {
    set_error("neb_spectral_range: non-finite mass matrix");
    return NEB_ERR_NONFINITE;
  }
  int r = 0;
  for (int i = 0; i < m; ++i) r += eh[(size_t)i] > rank_rtol * emax ? 1 : 0;
  *rank = r;
  if (r == 0 || !(emax > 0.0)) {
    set_error("neb_spectral_range: the mass matrix has no positive eigenvalue");
    return NEB_ERR_NOT_PD;
  }
  int lwork_r = 0;
  if ((st = syevd_lwork(sol, r, &lwork_r))) return st;
  NEB_REQUIRE(lwork_r <= lwork, "neb_spectral_range: solver workspace for rank %d exceeds m", r);
  const int threads = 256;
  {
    KernelScope ks("range_basis", stream, 0, 16.0 * m * r);
    range_basis<<<(unsigned)ceil_div((int64_t)m * r, threads), threads, 0, stream>>>(Q, e, m, r,
                                                                                      Qr);
    NEB_LAUNCH_CHECK();
  }
  double one = 1.0, zero = 0.0, mone = -1.0;
  {
    KernelScope ks("cublas_dgemm", stream, 2.0 * m * (double)m * r + 2.0 * r * (double)r * m,
                   8.0 * (m * (double)m + 2.0 * m * r + r * (double)r), 2);
    // T = S Qr (m x r), C = Qr^T T (r x r)
    if (cublasDgemm(blas, CUBLAS_OP_N, CUBLAS_OP_N, m, r, m, &one, S, m, Qr, m, &zero, T, m) !=
            CUBLAS_STATUS_SUCCESS ||
        cublasDgemm(blas, CUBLAS_OP_T, CUBLAS_OP_N, r, r, m, &one, Qr, m, T, m, &zero, Cm, r) !=
            CUBLAS_STATUS_SUCCESS) {
      set_error("cublasDgemm (finite pencil) failed");
      return NEB_ERR_CUDA;
    }
  }
  {
    KernelScope ks("cusolver_dsyevd", stream, 9.0 * r * (double)r * r, 0);
    if (cusolverDnDsyevd(sol, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER, r, Cm, r, lam,
                         work, lwork, info) != CUSOLVER_STATUS_SUCCESS) {
      set_error("cusolverDnDsyevd (finite pencil) failed");
      return NEB_ERR_SOLVER;
    }
  }
  // V = Qr Y (m x r, column k = eigenvector k = row k of the row-major output)
  NEB_CUDA_CHECK(cudaMemsetAsync(V, 0, (size_t)m * m * sizeof(double), stream));
  {
    KernelScope ks("cublas_dgemm", stream, 2.0 * m * (double)r * r, 8.0 * (2.0 * m * r + r * r));
    if (cublasDgemm(blas, CUBLAS_OP_N, CUBLAS_OP_N, m, r, r, &one, Qr, m, Cm, r, &zero, V, m) !=
        CUBLAS_STATUS_SUCCESS) {
      set_error("cublasDgemm (eigenvectors) failed");
      return NEB_ERR_CUDA;
    }
  }
  const unsigned blocks = (unsigned)ceil_div((int64_t)m * r, threads);
  {
    KernelScope ks("scale_columns", stream, 0, 16.0 * m * r);
    scale_cols<<<blocks, threads, 0, stream>>>(V, m, r, c, nullptr, T);
    NEB_LAUNCH_CHECK();
  }
  {
    KernelScope ks("cublas_dgemm", stream, 2.0 * m * (double)m * r, 8.0 * (2.0 * m * r + m * m));
    if (cublasDgemm(blas, CUBLAS_OP_N, CUBLAS_OP_T, m, m, r, &one, T, m, V, m, &zero, G_S, m) !=
        CUBLAS_STATUS_SUCCESS) {
      set_error("cublasDgemm (G_S) failed");
      return NEB_ERR_CUDA;
    }
  }
  {
    KernelScope ks("scale_columns", stream, 0, 16.0 * m * r);
    scale_cols<<<blocks, threads, 0, stream>>>(V, m, r, c, lam, T);
    NEB_LAUNCH_CHECK();
  }
  {
    KernelScope ks("cublas_dgemm", stream, 2.0 * m * (double)m * r, 8.0 * (2.0 * m * r + m * m));
    if (cublasDgemm(blas, CUBLAS_OP_N, CUBLAS_OP_T, m, m, r, &mone, T, m, V, m, &zero, G_M, m) !=
        CUBLAS_STATUS_SUCCESS) {
      set_error("cublasDgemm (G_M) failed");
      return NEB_ERR_CUDA;
    }
  }
  if (r < m)
    NEB_CUDA_CHECK(cudaMemsetAsync(lam + r, 0, (size_t)(m - r) * sizeof(double), stream));
  {
    KernelScope ks("weighted_sum", stream, 0, 16.0 * r);
    weighted_sum<<<1, 256, 0, stream>>>(c, lam, r, loss, info);
    NEB_LAUNCH_CHECK();
  }
  return NEB_OK;
}
