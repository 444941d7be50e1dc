// Causal Rayleigh peel in Gram form, FP64 on the device, and the FP64
// products of field columns with K x K coefficient matrices.
//
// The peel (experiments/metaball/_backend/flow/cases/metaball/velocity/
// core.py:48-69 coefficient_peel): modes sorted by their raw quotients
// S_kk / M_kk (stable), the sorted mass matrix orthonormalised by a scaled
// Cholesky factor applied twice (the Gram form of two-pass modified
// Gram-Schmidt in the mass metric), losses = diag(T^T S T), and the
// coefficient adjoints Cu, Cd with dL/dU = U Cu / n, dL/dD = D Cd / n for
// L = sum(losses).  The order is a rank computation on the device (no host
// round trip); the factorisations are cuSOLVER potrf and cuBLAS trsm / gemm.
// Matrices are symmetric at the boundary (row- and column-major coincide);
// T and the adjoints are returned row-major.
#include <cublas_v2.h>
#include <cusolverDn.h>
#include <algorithm>
#include "neb_common.cuh"

namespace neb {
namespace {

struct PeelHandles {
  cusolverDnHandle_t solver = nullptr;
  cublasHandle_t blas = nullptr;
  ~PeelHandles() {
    if (solver) cusolverDnDestroy(solver);
    if (blas) cublasDestroy(blas);
  }
};
thread_local PeelHandles g_peel;

int peel_handles(cudaStream_t s) {
  if (!g_peel.solver && cusolverDnCreate(&g_peel.solver) != CUSOLVER_STATUS_SUCCESS) {
    set_error("cusolverDnCreate failed");
    return NEB_ERR_CUDA;
  }
  if (!g_peel.blas && cublasCreate(&g_peel.blas) != CUBLAS_STATUS_SUCCESS) {
    set_error("cublasCreate failed");
    return NEB_ERR_CUDA;
  }
  cusolverDnSetStream(g_peel.solver, s);
  cublasSetStream(g_peel.blas, s);
  cublasSetPointerMode(g_peel.blas, CUBLAS_POINTER_MODE_HOST);
  return NEB_OK;
}

size_t a256(size_t x) { return (x + 255) & ~size_t(255); }

#define NEB_BLAS(expr, what)                                                   \
  do {                                                                         \
    if ((expr) != CUBLAS_STATUS_SUCCESS) {                                     \
      set_error("%s failed", what);                                            \
      return NEB_ERR_CUDA;                                                     \
    }                                                                          \
  } while (0)

// raw_i = S_ii / M_ii (a non-finite quotient sorts last); stable ascending
// ranks; order[rank] = i (peel_rank).
__global__ void peel_order(const double* __restrict__ M, const double* __restrict__ S, int K,
                           int* __restrict__ order, double* __restrict__ raw) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < K; i += gridDim.x * blockDim.x) {
    double r = S[(size_t)i * K + i] / M[(size_t)i * K + i];
    raw[i] = r;
  }
}
__global__ void peel_rank(const double* __restrict__ raw, int K, int* __restrict__ order) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < K; i += gridDim.x * blockDim.x) {
    const double ri = raw[i];
    const bool fi = isfinite(ri);
    int rank = 0;
    for (int j = 0; j < K; ++j) {
      const double rj = raw[j];
      const bool fj = isfinite(rj);
      const bool before = fi ? (fj && (rj < ri || (rj == ri && j < i))) : (fj || j < i);
      rank += before;
    }
    order[rank] = i;
  }
}

__global__ void peel_fixed_order(int K, int* __restrict__ order) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < K; i += gridDim.x * blockDim.x)
    order[i] = i;
}

// ms = M[order][order], ss = S[order][order], scale = sqrt(diag ms),
// H = ms / (scale_i scale_j) (column-major, symmetric).
__global__ void peel_gather(const double* __restrict__ M, const double* __restrict__ S,
                            const int* __restrict__ order, int K, double* __restrict__ ms,
                            double* __restrict__ ss, double* __restrict__ H,
                            double* __restrict__ scale) {
  const int64_t total = (int64_t)K * K;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(e % K), j = (int)(e / K);
    const int oi = order[i], oj = order[j];
    const double m = M[(size_t)oi * K + oj];
    ms[e] = m;
    ss[e] = S[(size_t)oi * K + oj];
    const double si = sqrt(M[(size_t)oi * K + oi]), sj = sqrt(M[(size_t)oj * K + oj]);
    H[e] = m / si / sj;
    if (i == j) scale[i] = si;
  }
}

// T (column-major) rows divided by scale; also the identity for the next solve.
__global__ void scale_rows(double* __restrict__ T, const double* __restrict__ scale, int K) {
  const int64_t total = (int64_t)K * K;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
       e += (int64_t)gridDim.x * blockDim.x)
    T[e] /= scale[e % K];
}

__global__ void set_identity(double* __restrict__ X, int K) {
  const int64_t total = (int64_t)K * K;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
       e += (int64_t)gridDim.x * blockDim.x)
    X[e] = (e % K) == (e / K) ? 1.0 : 0.0;
}

__global__ void symmetrize(double* __restrict__ X, int K) {
  const int64_t total = (int64_t)K * K;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(e % K), j = (int)(e / K);
    if (i < j) {
      const double v = 0.5 * (X[e] + X[(int64_t)i * K + j]);
      X[e] = v;
      X[(int64_t)i * K + j] = v;
    }
  }
}

// Gate and the per-rank scalars: losses = diag F, norm = 1 / diag T (the
// peeled mass is norm^2), relative = norm^2 / diag ms, error = max |O - I|;
// Fu = strict upper triangle of F (in place).  mass_floor <= 0: the gate of
// velocity/core.py:60-62 (finite positive losses, relative mass >= 1e-4,
// orthogonality error <= 1e-5); mass_floor > 0: the gate of
// hardcoded_backend.py:3555-3567 (finite values, raw and peeled masses above
// the floor).  info: 0 ok, 2 gate failed.
__global__ void peel_gate(const double* __restrict__ T, const double* __restrict__ ms,
                          const double* __restrict__ O, double* __restrict__ F, int K,
                          double mass_floor,
                          double* __restrict__ loss, double* __restrict__ norm,
                          double* __restrict__ relative, double* __restrict__ error,
                          int* __restrict__ info) {
  __shared__ double emax[32];
  __shared__ int bad;
  if (threadIdx.x == 0) bad = 0;
  __syncthreads();
  double e = 0.0;
  for (int64_t x = threadIdx.x; x < (int64_t)K * K; x += blockDim.x) {
    const int i = (int)(x % K), j = (int)(x / K);
    e = fmax(e, fabs(O[x] - (i == j ? 1.0 : 0.0)));
  }
  for (int i = threadIdx.x; i < K; i += blockDim.x) {
    const double l = F[(int64_t)i * K + i];
    const double nm = 1.0 / T[(int64_t)i * K + i];
    const double rel = nm * nm / ms[(int64_t)i * K + i];
    loss[i] = l;
    norm[i] = nm;
    relative[i] = rel;
    const double m = ms[(int64_t)i * K + i];
    const bool ok = mass_floor > 0.0
                        ? (isfinite(l) && isfinite(m) && m > mass_floor && isfinite(nm) &&
                           nm * nm > mass_floor)
                        : (isfinite(l) && l > 0.0 && rel >= 1e-4);
    if (!ok) atomicOr(&bad, 1);
  }
  for (int o = 16; o > 0; o >>= 1) e = fmax(e, __shfl_down_sync(0xffffffffu, e, o));
  if ((threadIdx.x & 31) == 0) emax[threadIdx.x >> 5] = e;
  __syncthreads();
  if (threadIdx.x == 0) {
    double m = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) m = fmax(m, emax[w]);
    *error = m;
    const bool ortho_bad = mass_floor > 0.0 ? !(m == m) : !(m <= 1e-5);
    if ((ortho_bad || bad) && *info == 0) *info = 2;
  }
  __syncthreads();
  // strict upper triangle of F for C = T diag(loss) + T triu(F, 1)
  for (int64_t x = threadIdx.x; x < (int64_t)K * K; x += blockDim.x) {
    const int i = (int)(x % K), j = (int)(x / K);
    if (i >= j) F[x] = 0.0;
  }
}

// C = -2 (T diag(loss) + TF) / norm_j, B = 2 T / norm_j (sorted order,
// column-major), scattered to mode order: Cu[order_i][order_j] = C_ij,
// Cd[order_i][order_j] = B_ij, T_out[order_i][j] = T_ij (row-major).
__global__ void peel_adjoints(const double* __restrict__ T, const double* __restrict__ TF,
                              const double* __restrict__ loss, const double* __restrict__ norm,
                              const int* __restrict__ order, int K, double* __restrict__ Cu,
                              double* __restrict__ Cd, double* __restrict__ T_out) {
  const int64_t total = (int64_t)K * K;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(e % K), j = (int)(e / K);
    const double t = T[e];
    const double c = -2.0 * (t * loss[j] + TF[e]) / norm[j];
    const double b = 2.0 * t / norm[j];
    const int oi = order[i], oj = order[j];
    Cu[(size_t)oi * K + oj] = c;
    Cd[(size_t)oi * K + oj] = b;
    T_out[(size_t)oi * K + j] = t;
  }
}

// ------------------------------------------------ double-float K x K products
// C = op(A) op(B) for column-major K x K FP64 matrices, computed with pairs of
// floats: every operand is split on the way into shared memory as hi + lo
// (48 significant bits), a product a b = ah bh + (ah bl + al bh) keeps ah bh
// exactly (FMA) and the sum is carried as s + c with the TwoSum error of
// every addition (relative error ~ 2^-48 sqrt(K)).  FP64 runs at ~1 TFLOP/s
// on this GPU, FP32 some sixty times faster, so these products take the
// place of FP64 triangular multiplies.  op(X) is X^T when its flag is set.
// tri: 0 full; 1 op(A) upper (zero for k < i); 2 op(A) lower (zero for
// k > i); 3 op(B) upper (zero for k > j): the zero blocks are skipped and the
// zero entries masked.  Operands must lie within the float exponent range.
constexpr int kDfTile = 64, kDfK = 16, kDfLd = kDfTile + 4;

__device__ __forceinline__ void df_mac(float& s, float& c, float ah, float al, float bh,
                                       float bl) {
  const float p = ah * bh;
  const float e = fmaf(ah, bh, -p);
  const float t = fmaf(ah, bl, al * bh);
  const float ss = s + p;
  const float bb = ss - s;
  const float err = (s - (ss - bb)) + (p - bb);
  s = ss;
  c += err + e + t;
}

__global__ void __launch_bounds__(256)
df_gemm(int K, const double* __restrict__ A, int ta, const double* __restrict__ B, int tb, int tri,
        double* __restrict__ C) {
  __shared__ __align__(16) float Ah[kDfK][kDfLd], Al[kDfK][kDfLd], Bh[kDfK][kDfLd],
      Bl[kDfK][kDfLd];
  const int i0 = blockIdx.x * kDfTile, j0 = blockIdx.y * kDfTile;
  const int tid = threadIdx.x, tx = tid % 16, ty = tid / 16;
  int kb = 0, ke = K;
  if (tri == 1) kb = i0 / kDfK * kDfK;
  if (tri == 2) ke = min(K, i0 + kDfTile);
  if (tri == 3) ke = min(K, j0 + kDfTile);
  float s[4][4], c[4][4];
#pragma unroll
  for (int u = 0; u < 4; ++u)
#pragma unroll
    for (int v = 0; v < 4; ++v) s[u][v] = c[u][v] = 0.f;
  for (int k0 = kb; k0 < ke; k0 += kDfK) {
    for (int e = tid; e < kDfK * kDfTile; e += 256) {
      // A tile element (r, kk): consecutive threads along the contiguous index
      const int r = ta ? e / kDfK : e % kDfTile, kk = ta ? e % kDfK : e / kDfTile;
      const int i = i0 + r, k = k0 + kk;
      double x = 0.0;
      if (i < K && k < K && !(tri == 1 && k < i) && !(tri == 2 && k > i))
        x = ta ? A[(int64_t)i * K + k] : A[i + (int64_t)k * K];
      const float h = (float)x;
      Ah[kk][r] = h;
      Al[kk][r] = (float)(x - (double)h);
      // B tile element (kk, q)
      const int q = tb ? e % kDfTile : e / kDfK, kb2 = tb ? e / kDfTile : e % kDfK;
      const int j = j0 + q, kq = k0 + kb2;
      double y = 0.0;
      if (j < K && kq < K && !(tri == 3 && kq > j))
        y = tb ? B[j + (int64_t)kq * K] : B[kq + (int64_t)j * K];
      const float g = (float)y;
      Bh[kb2][q] = g;
      Bl[kb2][q] = (float)(y - (double)g);
    }
    __syncthreads();
#pragma unroll 4
    for (int kk = 0; kk < kDfK; ++kk) {
      const float4 ah = *reinterpret_cast<const float4*>(&Ah[kk][ty * 4]);
      const float4 al = *reinterpret_cast<const float4*>(&Al[kk][ty * 4]);
      const float4 bh = *reinterpret_cast<const float4*>(&Bh[kk][tx * 4]);
      const float4 bl = *reinterpret_cast<const float4*>(&Bl[kk][tx * 4]);
      const float a_h[4] = {ah.x, ah.y, ah.z, ah.w}, a_l[4] = {al.x, al.y, al.z, al.w};
      const float b_h[4] = {bh.x, bh.y, bh.z, bh.w}, b_l[4] = {bl.x, bl.y, bl.z, bl.w};
#pragma unroll
      for (int u = 0; u < 4; ++u)
#pragma unroll
        for (int v = 0; v < 4; ++v) df_mac(s[u][v], c[u][v], a_h[u], a_l[u], b_h[v], b_l[v]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int u = 0; u < 4; ++u)
#pragma unroll
    for (int v = 0; v < 4; ++v) {
      const int i = i0 + ty * 4 + u, j = j0 + tx * 4 + v;
      if (i < K && j < K) C[i + (int64_t)j * K] = (double)s[u][v] + (double)c[u][v];
    }
}

int launch_df_gemm(int K, const double* A, int ta, const double* B, int tb, int tri, double* C,
                   cudaStream_t s) {
  dim3 grid((unsigned)ceil_div(K, kDfTile), (unsigned)ceil_div(K, kDfTile));
  df_gemm<<<grid, 256, 0, s>>>(K, A, ta, B, tb, tri, C);
  NEB_LAUNCH_CHECK();
  return NEB_OK;
}

__global__ void potrf_gate(const int* __restrict__ dev_info, int* __restrict__ info) {
  if (*dev_info != 0 && *info == 0) *info = 1;
}

template <typename S, typename D>
__global__ void convert(const S* __restrict__ src, D* __restrict__ dst, int64_t n, double scale) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    dst[i] = (D)((double)src[i] * scale);
}

int grid_for(int64_t n) { return (int)std::min<int64_t>(std::max<int64_t>(ceil_div(n, 256), 1), 4096); }

}  // namespace
}  // namespace neb

using namespace neb;

extern "C" size_t neb_peel_workspace_bytes(int K) {
  if (K <= 0 || peel_handles(nullptr)) return 0;
  int lwork = 0;
  if (cusolverDnDpotrf_bufferSize(g_peel.solver, CUBLAS_FILL_MODE_LOWER, K, nullptr, K, &lwork) !=
      CUSOLVER_STATUS_SUCCESS)
    return 0;
  const size_t kk = a256((size_t)K * K * sizeof(double)), k1 = a256((size_t)K * sizeof(double));
  return 8 * kk + 5 * k1 + a256(sizeof(int) * 2) + a256((size_t)lwork * sizeof(double));
}

extern "C" int neb_coefficient_peel(int K, const double* M, const double* S, double mass_floor,
                                    int sort, double* losses,
                                    int* order, double* T_out, double* Cu, double* Cd,
                                    double* relative_mass, double* ortho_error, int* info,
                                    void* workspace, size_t workspace_bytes,
                                    neb_stream_t stream) {
  NEB_REQUIRE(K > 0 && M && S && losses && order && T_out && Cu && Cd && info,
              "neb_coefficient_peel: bad arguments");
  cudaStream_t s = (cudaStream_t)stream;
  int st = peel_handles(s);
  if (st) return st;
  int lwork = 0;
  if (cusolverDnDpotrf_bufferSize(g_peel.solver, CUBLAS_FILL_MODE_LOWER, K, nullptr, K, &lwork) !=
      CUSOLVER_STATUS_SUCCESS) {
    set_error("cusolverDnDpotrf_bufferSize failed");
    return NEB_ERR_CUDA;
  }
  const size_t kk = a256((size_t)K * K * sizeof(double)), k1 = a256((size_t)K * sizeof(double));
  const size_t need = 8 * kk + 5 * k1 + a256(sizeof(int) * 2) + a256((size_t)lwork * sizeof(double));
  if (!workspace || workspace_bytes < need) {
    set_error("neb_coefficient_peel: workspace %zu < %zu bytes", workspace_bytes, need);
    return NEB_ERR_WORKSPACE;
  }
  char* w = (char*)workspace;
  double* ms = (double*)w;
  double* ss = (double*)(w + kk);
  double* L = (double*)(w + 2 * kk);
  double* T = (double*)(w + 3 * kk);
  double* W1 = (double*)(w + 4 * kk);
  double* L2 = (double*)(w + 5 * kk);
  double* F = (double*)(w + 6 * kk);
  double* TF = (double*)(w + 7 * kk);
  double* raw = (double*)(w + 8 * kk);
  double* scale = (double*)(w + 8 * kk + k1);
  double* norm = (double*)(w + 8 * kk + 2 * k1);
  double* rel_tmp = (double*)(w + 8 * kk + 3 * k1);
  double* err_tmp = (double*)(w + 8 * kk + 4 * k1);
  int* dinfo = (int*)(w + 8 * kk + 5 * k1);
  double* work = (double*)(w + 8 * kk + 5 * k1 + a256(sizeof(int) * 2));
  double* rel = relative_mass ? relative_mass : rel_tmp;
  double* err = ortho_error ? ortho_error : err_tmp;
  const int64_t kk_n = (int64_t)K * K;
  cublasHandle_t h = g_peel.blas;
  const double one = 1.0;
  NEB_CUDA_CHECK(cudaMemsetAsync(info, 0, sizeof(int), s));
  {
    KernelScope ks("peel_order", s, 0, 8.0 * K * K);
    peel_order<<<grid_for(K), 256, 0, s>>>(M, S, K, order, raw);
    NEB_LAUNCH_CHECK();
    if (sort) peel_rank<<<grid_for(K), 256, 0, s>>>(raw, K, order);
    else peel_fixed_order<<<grid_for(K), 256, 0, s>>>(K, order);
    NEB_LAUNCH_CHECK();
    peel_gather<<<grid_for(kk_n), 256, 0, s>>>(M, S, order, K, ms, ss, L, scale);
    NEB_LAUNCH_CHECK();
  }
  // first pass: H = L L^T, T = L^-T / scale (rows)
  {
    KernelScope ks("peel_cholesky", s, 2.0 * K * (double)K * K, 0);
    if (cusolverDnDpotrf(g_peel.solver, CUBLAS_FILL_MODE_LOWER, K, L, K, work, lwork, dinfo) !=
        CUSOLVER_STATUS_SUCCESS) {
      set_error("cusolverDnDpotrf failed");
      return NEB_ERR_SOLVER;
    }
    potrf_gate<<<1, 1, 0, s>>>(dinfo, info);
    NEB_LAUNCH_CHECK();
    set_identity<<<grid_for(kk_n), 256, 0, s>>>(T, K);
    NEB_LAUNCH_CHECK();
    NEB_BLAS(cublasDtrsm(h, CUBLAS_SIDE_LEFT, CUBLAS_FILL_MODE_LOWER, CUBLAS_OP_T,
                         CUBLAS_DIAG_NON_UNIT, K, K, &one, L, K, T, K),
             "cublasDtrsm (L^-T)");
    scale_rows<<<grid_for(kk_n), 256, 0, s>>>(T, scale, K);
    NEB_LAUNCH_CHECK();
    // second pass: H2 = T^T ms T = L2 L2^T, T <- T L2^-T.  T is upper
    // triangular (a scaled inverse transpose of a lower Cholesky factor, and
    // after the second pass a product of two upper triangles), so every
    // product with it is a triangular multiply (half a GEMM's work)
    if ((st = launch_df_gemm(K, ms, 0, T, 0, 3, W1, s))) return st;   // ms T
    if ((st = launch_df_gemm(K, T, 1, W1, 0, 2, L2, s))) return st;   // T^T (ms T)
    symmetrize<<<grid_for(kk_n), 256, 0, s>>>(L2, K);
    NEB_LAUNCH_CHECK();
    if (cusolverDnDpotrf(g_peel.solver, CUBLAS_FILL_MODE_LOWER, K, L2, K, work, lwork, dinfo) !=
        CUSOLVER_STATUS_SUCCESS) {
      set_error("cusolverDnDpotrf failed");
      return NEB_ERR_SOLVER;
    }
    potrf_gate<<<1, 1, 0, s>>>(dinfo, info);
    NEB_LAUNCH_CHECK();
    NEB_BLAS(cublasDtrsm(h, CUBLAS_SIDE_RIGHT, CUBLAS_FILL_MODE_LOWER, CUBLAS_OP_T,
                         CUBLAS_DIAG_NON_UNIT, K, K, &one, L2, K, T, K),
             "cublasDtrsm (T L2^-T)");
  }
  {
    KernelScope ks("peel_objective", s, 5.0 * K * (double)K * K, 0);
    // O = T^T ms T (orthogonality), F = T^T ss T, TF = T triu(F, 1): all
    // triangular multiplies with the upper triangular T
    if ((st = launch_df_gemm(K, ms, 0, T, 0, 3, W1, s))) return st;   // ms T
    if ((st = launch_df_gemm(K, T, 1, W1, 0, 2, L, s))) return st;    // O = T^T ms T
    if ((st = launch_df_gemm(K, ss, 0, T, 0, 3, W1, s))) return st;   // ss T
    if ((st = launch_df_gemm(K, T, 1, W1, 0, 2, F, s))) return st;    // F = T^T ss T
    peel_gate<<<1, 1024, 0, s>>>(T, ms, L, F, K, mass_floor, losses, norm, rel, err, info);
    NEB_LAUNCH_CHECK();
    if ((st = launch_df_gemm(K, T, 0, F, 0, 1, TF, s))) return st;    // T triu(F, 1)
    peel_adjoints<<<grid_for(kk_n), 256, 0, s>>>(T, TF, losses, norm, order, K, Cu, Cd, T_out);
    NEB_LAUNCH_CHECK();
  }
  return NEB_OK;
}

extern "C" size_t neb_column_apply_workspace_bytes(int64_t rows, int K) {
  if (rows <= 0 || K <= 0) return 0;
  return 2 * a256((size_t)K * K * sizeof(float));
}

// scale * C (FP64) as an unevaluated sum of two floats: hi = fl(x), lo = fl(x - hi).
__global__ void split_scaled(const double* __restrict__ C, double scale, int64_t n,
                             float* __restrict__ hi, float* __restrict__ lo) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const double x = scale * C[i];
    const float h = (float)x;
    hi[i] = h;
    lo[i] = (float)(x - (double)h);
  }
}

// out = scale * A C, A [rows][K] (row-major), C [K][K] FP64 row-major, out
// in A's type.  FP64: one cuBLAS DGEMM.  FP32: A is exact in FP32 and
// scale * C enters as hi + lo (48 bits), two FP32 SGEMMs (out = A hi, then
// out += A lo) -- the FP32 accumulation is the only rounding beyond the
// output's own, and FP64 DGEMM runs at ~1/60 of the FP32 rate on this GPU.
extern "C" int neb_column_apply(int precision, int64_t rows, int K, const void* A,
                                const double* Cm, double scale, void* out, void* workspace,
                                size_t workspace_bytes, neb_stream_t stream) {
  NEB_REQUIRE(precision == NEB_PREC_FP32 || precision == NEB_PREC_FP64 ||
                  precision == NEB_PREC_TF32 || precision == NEB_PREC_BF16X9,
              "neb_column_apply: FP32 (also TF32 / BF16x9 products) or FP64");
  NEB_REQUIRE(rows > 0 && rows <= (int64_t)1 << 31 && K > 0 && A && Cm && out,
              "neb_column_apply: bad arguments");
  cudaStream_t s = (cudaStream_t)stream;
  int st = peel_handles(s);
  if (st) return st;
  cublasHandle_t h = g_peel.blas;
  if (precision == NEB_PREC_FP64) {
    const double zero = 0.0;
    KernelScope ks("cublas_dgemm", s, 2.0 * rows * (double)K * K, 0);
    // row-major out = A C  <=>  column-major out^T = C^T A^T
    NEB_BLAS(cublasDgemm(h, CUBLAS_OP_N, CUBLAS_OP_N, K, (int)rows, K, &scale, Cm, K,
                         (const double*)A, K, &zero, (double*)out, K),
             "cublasDgemm (columns)");
    return NEB_OK;
  }
  if (!workspace || workspace_bytes < neb_column_apply_workspace_bytes(rows, K)) {
    set_error("neb_column_apply: workspace too small");
    return NEB_ERR_WORKSPACE;
  }
  const int64_t kk = (int64_t)K * K;
  float* hi = (float*)workspace;
  float* lo = (float*)((char*)workspace + a256((size_t)kk * sizeof(float)));
  {
    KernelScope ks("split_scaled", s, 0, 16.0 * kk);
    split_scaled<<<grid_for(kk), 256, 0, s>>>(Cm, scale, kk, hi, lo);
    NEB_LAUNCH_CHECK();
  }
  if (precision != NEB_PREC_FP32) {
    // the tensor-core forms: the two products through cuBLAS with their compute type
    KernelScope ks("cublas_gemm_tc", s, 4.0 * rows * (double)K * K, 0);
    const cublasComputeType_t ct = precision == NEB_PREC_TF32 ? CUBLAS_COMPUTE_32F_FAST_TF32
                                                              : CUBLAS_COMPUTE_32F_EMULATED_16BFX9;
    const float one = 1.f, zero = 0.f;
    const cublasStatus_t r1 =
        cublasGemmEx(h, CUBLAS_OP_N, CUBLAS_OP_N, K, (int)rows, K, &one, hi, CUDA_R_32F, K, A,
                     CUDA_R_32F, K, &zero, out, CUDA_R_32F, K, ct, CUBLAS_GEMM_DEFAULT);
    const cublasStatus_t r2 =
        cublasGemmEx(h, CUBLAS_OP_N, CUBLAS_OP_N, K, (int)rows, K, &one, lo, CUDA_R_32F, K, A,
                     CUDA_R_32F, K, &one, out, CUDA_R_32F, K, ct, CUBLAS_GEMM_DEFAULT);
    if (r1 != CUBLAS_STATUS_SUCCESS || r2 != CUBLAS_STATUS_SUCCESS) {
      set_error("cublasGemmEx (columns) failed");
      return NEB_ERR_CUDA;
    }
    return NEB_OK;
  }
  {
    KernelScope ks("cublas_sgemm", s, 4.0 * rows * (double)K * K, 0);
    cublasSetMathMode(h, CUBLAS_PEDANTIC_MATH);  // plain FP32 products, no TF32
    const float one = 1.f, zero = 0.f;
    const cublasStatus_t r1 = cublasSgemm(h, CUBLAS_OP_N, CUBLAS_OP_N, K, (int)rows, K, &one,
                                          hi, K, (const float*)A, K, &zero, (float*)out, K);
    const cublasStatus_t r2 = cublasSgemm(h, CUBLAS_OP_N, CUBLAS_OP_N, K, (int)rows, K, &one,
                                          lo, K, (const float*)A, K, &one, (float*)out, K);
    cublasSetMathMode(h, CUBLAS_DEFAULT_MATH);
    if (r1 != CUBLAS_STATUS_SUCCESS || r2 != CUBLAS_STATUS_SUCCESS) {
      set_error("cublasSgemm (columns) failed");
      return NEB_ERR_CUDA;
    }
  }
  return NEB_OK;
}
