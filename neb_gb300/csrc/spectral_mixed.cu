// Mixed-precision spectral stage for m <= 512 (neb_spectral_mixed).
//
// Precision follows where the conditioning lives.  The mass matrix M carries
// the condition number of the basis (1e4 and more), so its Cholesky factor
// and the reduction C = L^-1 S L^-T (whose products cancel by up to cond(M))
// are computed with FP64-class accuracy.  On GB300 the FP64 pipe issues about
// 1.65 FMA per cycle per SM and a dependent FP64 FMA takes 64 cycles, so that
// accuracy comes from compensated FP32 arithmetic (value = hi + lo, TwoProd /
// TwoSum, relative 2^-44 or better), with the FP64 matrices as storage.
// After the reduction the standard problem is well conditioned (cond(C) =
// lam_max / lam_min, tens): C is rounded to FP32 and reduced to a tridiagonal
// T by FP32 Householder steps.  Eigenvalues of T are bracketed by FP32 Sturm
// multisection, eigenvectors come from FP32 twisted factorisations, and the
// eigenvalues are finally the FP64 Rayleigh quotients of those vectors.  On
// GB300 a dependent FP64 FMA costs 64 cycles and an FP64 divide 600+, so no
// sequential recurrence runs in FP64.  Back-transformation, V = L^-T Q Z, and
// the objective adjoints G_S = V diag(c) V^T, G_M = -V diag(c lam) V^T run in
// FP32 (they only feed the reverse pass).
//
// Pipeline (one stream, no host synchronisation):
//   chol_diag / chol_panel / chol_update   blocked Cholesky, 32 x 32 blocks,
//                                          compensated FP32 (FP64-class)
//   2 x df_trsm                            C = L^-1 S L^-T by two triangular
//                                          solves, compensated FP32
//   tridiag_cluster                        FP32 Householder tridiagonalisation in
//                                          one 8-CTA cluster, the matrix held in
//                                          distributed shared memory, 2 cluster
//                                          barriers per column
//   tri_eigvals                            eigenvalue brackets of T, warp per eigenvalue
//   tri_eigvecs                            eigenvectors of T by twisted factorisations,
//                                          eigenvalues refined to FP64 Rayleigh quotients
//   householder_apply                      x_k = Q z_k (FP32), warp per vector
//   df_trsm, SGEMMs                        V rows = (L^-T x_k)^T, G_S, G_M
#include <cooperative_groups.h>
#include <cublas_v2.h>
#include "elementwise.cuh"

namespace cg = cooperative_groups;

namespace neb {
namespace {

constexpr int kCB = 32;          // Cholesky block
constexpr int kMaxM = 512;
constexpr int kCluster = 8;
constexpr int kTriThreads = 512;

size_t al(size_t x) { return (x + 255) & ~size_t(255); }

// ------------------------------------------------ compensated FP32 ("df")
// A value is an unevaluated sum hi + lo of two floats (about 48 significant
// bits).  Products use TwoProd through fma, sums TwoSum: every operation runs
// on the FP32 pipe, whose dependent latency is a few cycles against 64 for an
// FP64 FMA on GB300, with FP64-class accuracy (relative 2^-44 or better).
struct df {
  float h, l;
};
__device__ __forceinline__ df df_quick(float a, float b) {
  float s = a + b;
  return {s, b - (s - a)};
}
__device__ __forceinline__ df df_add(df x, df y) {
  float s = x.h + y.h;
  float bb = s - x.h;
  float e = (x.h - (s - bb)) + (y.h - bb);
  e += x.l + y.l;
  return df_quick(s, e);
}
__device__ __forceinline__ df df_neg(df x) { return {-x.h, -x.l}; }
__device__ __forceinline__ df df_mul(df x, df y) {
  float p = x.h * y.h;
  float e = fmaf(x.h, y.h, -p);
  e = fmaf(x.h, y.l, fmaf(x.l, y.h, e));
  return df_quick(p, e);
}
__device__ __forceinline__ df df_from(double v) {
  float h = (float)v;
  return {h, (float)(v - (double)h)};
}
__device__ __forceinline__ double df_to(df x) { return (double)x.h + (double)x.l; }
// 1 / x with one Newton step: r + r (1 - x r)
__device__ __forceinline__ df df_recip(df x) {
  float r = 1.0f / x.h;
  df xr = df_mul(x, df{r, 0.f});
  df res = df_add(df{1.f, 0.f}, df_neg(xr));
  return df_add(df{r, 0.f}, df_mul(df{r, 0.f}, res));
}
// sqrt(x) with one Newton correction
__device__ __forceinline__ df df_sqrt(df x) {
  float s = sqrtf(x.h);
  float p = s * s;
  float pe = fmaf(s, s, -p);
  float r = ((x.h - p) - pe) + x.l;
  return df_quick(s, r / (2.f * s));
}
__device__ __forceinline__ df df_shfl_xor(df x, int o) {
  return {__shfl_xor_sync(0xffffffffu, x.h, o), __shfl_xor_sync(0xffffffffu, x.l, o)};
}

// ------------------------------------------------------------ Cholesky
// Blocked right-looking Cholesky of the FP64 matrix A (lower factor written
// back in FP64), 32 x 32 blocks, compensated FP32 arithmetic.
__global__ void __launch_bounds__(1024) chol_diag(double* __restrict__ A, int m, int p,
                                                  double* __restrict__ Linv_pp,
                                                  int* __restrict__ info) {
  __shared__ df a[kCB][kCB + 1];
  __shared__ df x[kCB][kCB + 1];
  __shared__ df rpiv[kCB];
  __shared__ int bad;
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  const int r0 = p * kCB;
  a[ty][tx] = df_from(A[(size_t)(r0 + ty) * m + r0 + tx]);
  if (threadIdx.x == 0) bad = 0;
  __syncthreads();
  for (int k = 0; k < kCB; ++k) {
    if (threadIdx.x == 0) {
      df v = a[k][k];
      if (!(v.h > 0.f)) {  // not positive definite (or NaN)
        if (!bad) bad = k + 1;
        v = df{1.f, 0.f};
      }
      df sq = df_sqrt(v);
      a[k][k] = sq;
      rpiv[k] = df_recip(sq);
    }
    __syncthreads();
    if (ty == 0 && tx > k) a[tx][k] = df_mul(a[tx][k], rpiv[k]);
    __syncthreads();
    if (ty > k && tx > k && tx <= ty) a[ty][tx] = df_add(a[ty][tx], df_neg(df_mul(a[ty][k], a[tx][k])));
    __syncthreads();
  }
  if (tx <= ty) A[(size_t)(r0 + ty) * m + r0 + tx] = df_to(a[ty][tx]);
  // inverse of the diagonal block, row by row (column j per lane of warp 0)
  for (int i = 0; i < kCB; ++i) {
    if (ty == 0) {
      const int j = tx;
      df s = (i == j) ? df{1.f, 0.f} : df{0.f, 0.f};
      for (int k = j; k < i; ++k) s = df_add(s, df_neg(df_mul(a[i][k], x[k][j])));
      x[i][j] = i < j ? df{0.f, 0.f} : df_mul(s, rpiv[i]);
    }
    __syncwarp();
  }
  __syncthreads();
  Linv_pp[ty * kCB + tx] = df_to(x[ty][tx]);
  if (threadIdx.x == 0 && bad && *info == 0) *info = m + r0 + bad;
}

// L_ip = A_ip L_pp^-T for the row blocks below the diagonal block.
__global__ void __launch_bounds__(1024) chol_panel(double* __restrict__ A, int m, int p,
                                                   const double* __restrict__ Linv_pp) {
  __shared__ df a[kCB][kCB + 1];
  __shared__ df li[kCB][kCB + 1];
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  const int rb = (p + 1 + blockIdx.x) * kCB, cb = p * kCB;
  a[ty][tx] = df_from(A[(size_t)(rb + ty) * m + cb + tx]);
  li[ty][tx] = df_from(Linv_pp[ty * kCB + tx]);
  __syncthreads();
  df s0{0.f, 0.f}, s1{0.f, 0.f};
#pragma unroll
  for (int k = 0; k < kCB; k += 2) {
    s0 = df_add(s0, df_mul(a[ty][k], li[tx][k]));
    s1 = df_add(s1, df_mul(a[ty][k + 1], li[tx][k + 1]));
  }
  A[(size_t)(rb + ty) * m + cb + tx] = df_to(df_add(s0, s1));
}

// A_ij -= L_ip L_jp^T for the lower-triangle tiles p < j <= i.
__global__ void __launch_bounds__(1024) chol_update(double* __restrict__ A, int m, int p) {
  __shared__ df li[kCB][kCB + 1];
  __shared__ df lj[kCB][kCB + 1];
  int t = blockIdx.x, bi = p + 1;
  while (t >= bi - p) {  // tile index -> (bi, bj) with p < bj <= bi
    t -= bi - p;
    ++bi;
  }
  const int bj = p + 1 + t;
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  const int cb = p * kCB;
  li[ty][tx] = df_from(A[(size_t)(bi * kCB + ty) * m + cb + tx]);
  lj[ty][tx] = df_from(A[(size_t)(bj * kCB + ty) * m + cb + tx]);
  __syncthreads();
  df s0{0.f, 0.f}, s1{0.f, 0.f};
#pragma unroll
  for (int k = 0; k < kCB; k += 2) {
    s0 = df_add(s0, df_mul(li[ty][k], lj[tx][k]));
    s1 = df_add(s1, df_mul(li[ty][k + 1], lj[tx][k + 1]));
  }
  double* o = A + (size_t)(bi * kCB + ty) * m + bj * kCB + tx;
  *o = df_to(df_add(df_from(*o), df_neg(df_add(s0, s1))));
}

// The lower factor as float pairs, and its transpose (so both solves read
// rows): Ld[i][j] = L[i][j] (j <= i, else 0), LTd[j][i] = L[i][j].
__global__ void split_factor(const double* __restrict__ L, int m, df* __restrict__ Ld,
                             df* __restrict__ LTd) {
  __shared__ df t[32][33];
  const int bx = blockIdx.x * 32, by = blockIdx.y * 32;
  for (int r = threadIdx.y; r < 32; r += blockDim.y) {
    const int i = by + r, j = bx + threadIdx.x;
    df v = i >= j ? df_from(L[(size_t)i * m + j]) : df{0.f, 0.f};
    Ld[(size_t)i * m + j] = v;
    t[r][threadIdx.x] = v;
  }
  __syncthreads();
  for (int r = threadIdx.y; r < 32; r += blockDim.y)
    LTd[(size_t)(bx + r) * m + by + threadIdx.x] = t[threadIdx.x][r];
}

// Blocked triangular solves, compensated FP32, 8 right-hand-side columns per
// 256-thread block:
//   upper == 0:  L Y = B   (forward;  T = L as float pairs, rows of L)
//   upper == 1:  L^T Y = B (backward; T = L^T as float pairs, rows of L^T)
// Per 32-row block: the contribution of every solved row is a small
// matrix product over 32 x 32 tiles of T staged in shared memory (one output
// per thread, two accumulation chains); then the 32 x 32 diagonal block is
// solved by one warp per column with shuffles.  B(r, c) = b_trans ? B[c][r] :
// B[r][c] (FP64 or FP32); Y(r, c) goes to out[r][c] or, with out_trans,
// out[c][r] (FP64 or FP32).
constexpr int kTrsmCols = 8;
__global__ void __launch_bounds__(256) df_trsm(const df* __restrict__ T, int m, int upper,
                                               const void* __restrict__ B, int b_f32, int b_trans,
                                               void* __restrict__ out, int out_f32, int out_trans) {
  extern __shared__ df ys[];  // [m][kTrsmCols] solved values
  __shared__ df tile[32][33];
  __shared__ df acc[32][kTrsmCols + 1];
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int c0 = blockIdx.x * kTrsmCols;
  const int r_t = tid >> 3, c_t = tid & 7;  // phase-1 output (row in block, column)
  const int nb = m / 32;
  for (int bb = 0; bb < nb; ++bb) {
    const int b = upper ? nb - 1 - bb : bb;  // block of rows being solved
    const int rb0 = b * 32;
    // phase 1: acc = B - sum over solved blocks of T[rows][solved] y[solved]
    const int r = rb0 + r_t, c = c0 + c_t;
    {
      const size_t bi = b_trans ? (size_t)c * m + r : (size_t)r * m + c;
      const double bv = b_f32 ? (double)((const float*)B)[bi] : ((const double*)B)[bi];
      df s0 = df_from(bv), s1{0.f, 0.f};
      for (int kk = 0; kk < bb; ++kk) {
        const int kb = upper ? nb - 1 - kk : kk;
        __syncthreads();
        for (int t = tid; t < 32 * 32; t += 256) {
          const int tr = t >> 5, tc = t & 31;
          tile[tr][tc] = T[(size_t)(rb0 + tr) * m + kb * 32 + tc];
        }
        __syncthreads();
#pragma unroll 8
        for (int q = 0; q < 32; q += 2) {
          s0 = df_add(s0, df_neg(df_mul(tile[r_t][q], ys[(size_t)(kb * 32 + q) * kTrsmCols + c_t])));
          s1 = df_add(s1, df_neg(df_mul(tile[r_t][q + 1], ys[(size_t)(kb * 32 + q + 1) * kTrsmCols + c_t])));
        }
      }
      __syncthreads();
      acc[r_t][c_t] = df_add(s0, s1);
      for (int t = tid; t < 32 * 32; t += 256) {
        const int tr = t >> 5, tc = t & 31;
        tile[tr][tc] = T[(size_t)(rb0 + tr) * m + rb0 + tc];
      }
      __syncthreads();
    }
    // phase 2: solve the diagonal block, warp w -> column c0 + w, lane -> row
    if (warp < kTrsmCols) {
      df v = acc[lane][warp];
      for (int step = 0; step < 32; ++step) {
        const int q = upper ? 31 - step : step;  // row finalised at this step
        df yq{0.f, 0.f};
        if (lane == q) {
          yq = df_mul(v, df_recip(tile[q][q]));
          ys[(size_t)(rb0 + q) * kTrsmCols + warp] = yq;
        }
        yq.h = __shfl_sync(0xffffffffu, yq.h, q);
        yq.l = __shfl_sync(0xffffffffu, yq.l, q);
        const bool pending = upper ? lane < q : lane > q;
        if (pending) v = df_add(v, df_neg(df_mul(tile[lane][q], yq)));
      }
    }
    __syncthreads();
  }
  for (int t = tid; t < m * kTrsmCols; t += 256) {
    const int rr = t / kTrsmCols, cc = t % kTrsmCols;
    const df y = ys[t];
    const size_t oi = out_trans ? (size_t)(c0 + cc) * m + rr : (size_t)rr * m + c0 + cc;
    if (out_f32) ((float*)out)[oi] = y.h + y.l;
    else ((double*)out)[oi] = df_to(y);
  }
}

// ------------------------------------------------- cluster tridiagonalisation
struct TriShared {
  int rb, m;
};

__device__ __forceinline__ float block_sum(float v, float* red) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  __syncthreads();
  if (lane == 0) red[warp] = v;
  __syncthreads();
  float s = 0.f;
  for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += red[w];
  return s;
}

// C: [m][m] FP32 (symmetrised on load).  Outputs: d[m], e[m-1] (FP64 of the
// FP32 tridiagonal), Vh[m][m] (row k = Householder vector of step k, zero up
// to index k), tau[m].  Rows are dealt cyclically (row i on CTA i % 8) so
// every CTA keeps a share of the shrinking trailing matrix.  Per column:
// push the column and its squared norm, cluster barrier, p = tau A v on own
// rows and push it, cluster barrier, rank-2 update of own rows, block
// barrier.  The first entry of v (x1 - alpha) is applied through scalar
// corrections so no extra barrier is needed to patch it.
__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

__global__ void __cluster_dims__(kCluster, 1, 1) __launch_bounds__(kTriThreads, 1)
tridiag_cluster(const float* __restrict__ C, int m, double* __restrict__ d_out,
                double* __restrict__ e_out, float* __restrict__ Vh, float* __restrict__ tau_out) {
  cg::cluster_group cluster = cg::this_cluster();
  const int rank = (int)cluster.block_rank();
  const int rb = m / kCluster;  // local rows; global row of local li is li * 8 + rank
  extern __shared__ __align__(16) float sm[];
  float* Aloc = sm;                              // [rb][m]
  float* vbuf = Aloc + (size_t)rb * m;           // [2][m]
  float* pbuf = vbuf + 2 * m;                    // [2][m]
  float* sig = pbuf + 2 * m;                     // [2][kCluster]
  const int tid = threadIdx.x, nthr = blockDim.x;
  const int warp = tid >> 5, lane = tid & 31, nwarps = nthr >> 5;
  const int m4 = m >> 2;

  for (int li = warp; li < rb; li += nwarps) {
    const int i = li * kCluster + rank;
    for (int j = lane; j < m; j += 32)
      Aloc[(size_t)li * m + j] = 0.5f * (C[(size_t)i * m + j] + C[(size_t)j * m + i]);
  }
  __syncthreads();

  for (int k = 0; k + 2 < m; ++k) {
    const int par = k & 1;
    float* vb = vbuf + par * m;
    float* pb = pbuf + par * m;
    float* sg = sig + par * kCluster;
    // own rows i > k are local indices li >= lo
    const int lo = (k + 1 - rank + kCluster - 1) / kCluster > 0 ? (k + 1 - rank + kCluster - 1) / kCluster : 0;
    // (a) push column k of own rows; warp 0 pushes the squared norm
    for (int li = lo + warp; li < rb; li += nwarps)
      if (lane < kCluster) {
        float* rv = cluster.map_shared_rank(vb, lane);
        rv[li * kCluster + rank] = Aloc[(size_t)li * m + k];
      }
    if (warp == 0) {
      float part = 0.f;
      for (int li = lo + lane; li < rb; li += 32) {
        float x = Aloc[(size_t)li * m + k];
        part += x * x;
      }
      part = warp_sum(part);
      if (lane < kCluster) {
        float* rs = cluster.map_shared_rank(sg, lane);
        rs[rank] = part;
      }
    }
    cluster.sync();
    // (b) Householder vector v = x - alpha e_1 (x1 = vb[k + 1] is left unpatched)
    float sigma = 0.f;
#pragma unroll
    for (int c = 0; c < kCluster; ++c) sigma += sg[c];
    const float x1 = vb[k + 1];
    const float alpha = sigma > 0.f ? -copysignf(sqrtf(sigma), x1) : 0.f;
    const float v1 = x1 - alpha;
    const float vv = sigma - x1 * x1 + v1 * v1;
    const float tau = vv > 0.f ? 2.f / vv : 0.f;
    if (tid == 0) {
      if (rank == 0) {
        e_out[k] = alpha;
        tau_out[k] = tau;
      }
      if (k % kCluster == rank) d_out[k] = Aloc[(size_t)(k / kCluster) * m + k];
    }
    for (int li = lo + tid; li < rb; li += nthr) {
      const int i = li * kCluster + rank;
      Vh[(size_t)k * m + i] = i == k + 1 ? v1 : vb[i];
    }
    if (rank == 0)
      for (int i = tid; i <= k; i += nthr) Vh[(size_t)k * m + i] = 0.f;
    // (c) p_i = tau (A_i . v) on own rows (v_{k+1} = x1 - alpha by correction)
    const int j4 = (k + 1) >> 2;
    const float4* vb4 = reinterpret_cast<const float4*>(vb);
    for (int li = lo + warp; li < rb; li += nwarps) {
      const float* Ai = Aloc + (size_t)li * m;
      const float4* Ai4 = reinterpret_cast<const float4*>(Ai);
      float sacc = 0.f;
      for (int q = j4 + lane; q < m4; q += 32) {
        float4 a = Ai4[q], v = vb4[q];
        const int j = q << 2;
        sacc += (j >= k + 1 ? a.x * v.x : 0.f) + (j + 1 >= k + 1 ? a.y * v.y : 0.f) +
                (j + 2 >= k + 1 ? a.z * v.z : 0.f) + (j + 3 >= k + 1 ? a.w * v.w : 0.f);
      }
      sacc = warp_sum(sacc);
      const float p = tau * (sacc - alpha * Ai[k + 1]);
      if (lane < kCluster) {
        float* rp = cluster.map_shared_rank(pb, lane);
        rp[li * kCluster + rank] = p;
      }
    }
    cluster.sync();
    // (d) 2K = tau p^T v (each warp redundantly), then A -= v p^T + w v^T
    float kp = 0.f;
    const float4* pb4 = reinterpret_cast<const float4*>(pb);
    for (int q = j4 + lane; q < m4; q += 32) {
      float4 a = pb4[q], v = vb4[q];
      const int j = q << 2;
      kp += (j >= k + 1 ? a.x * v.x : 0.f) + (j + 1 >= k + 1 ? a.y * v.y : 0.f) +
            (j + 2 >= k + 1 ? a.z * v.z : 0.f) + (j + 3 >= k + 1 ? a.w * v.w : 0.f);
    }
    const float K2 = tau * (warp_sum(kp) - alpha * pb[k + 1]);
    for (int li = lo + warp; li < rb; li += nwarps) {
      const int i = li * kCluster + rank;
      float* Ai = Aloc + (size_t)li * m;
      float4* Ai4 = reinterpret_cast<float4*>(Ai);
      const float vi = i == k + 1 ? v1 : vb[i];
      const float pi = pb[i];
      const float wi = pi - K2 * vi;
      for (int q = j4 + lane; q < m4; q += 32) {  // entries j <= k are dead
        float4 a = Ai4[q], p = pb4[q], v = vb4[q];
        a.x -= vi * p.x + wi * v.x;
        a.y -= vi * p.y + wi * v.y;
        a.z -= vi * p.z + wi * v.z;
        a.w -= vi * p.w + wi * v.w;
        Ai4[q] = a;
      }
      __syncwarp();
      if (lane == 0) Ai[k + 1] += wi * alpha;  // v_{k+1} = vb[k+1] - alpha
    }
    __syncthreads();
  }
  if (tid == 0) {
    if ((m - 2) % kCluster == rank) {
      const float* Ar = Aloc + (size_t)((m - 2) / kCluster) * m;
      d_out[m - 2] = Ar[m - 2];
      e_out[m - 2] = Ar[m - 1];
    }
    if ((m - 1) % kCluster == rank) d_out[m - 1] = Aloc[(size_t)((m - 1) / kCluster) * m + m - 1];
  }
  if (rank == 0)
    for (int k = m - 2; k < m; ++k) {
      if (tid == 0) tau_out[k] = 0.f;
      for (int i = tid; i < m; i += nthr) Vh[(size_t)k * m + i] = 0.f;
    }
  cluster.sync();
}

// ------------------------------------------------------- tridiagonal eigen
// Number of eigenvalues of T below x (Sturm count), FP32 with the fast
// reciprocal (only the signs of the pivots matter).
__device__ __forceinline__ int sturm_count(const float* __restrict__ d,
                                           const float* __restrict__ e2, int m, float x,
                                           float pivmin) {
  int cnt = 0;
  float q = d[0] - x;
  if (fabsf(q) < pivmin) q = -pivmin;
  cnt += q < 0.f;
  for (int i = 1; i < m; ++i) {
    q = (d[i] - x) - __fdividef(e2[i - 1], q);
    if (fabsf(q) < pivmin) q = -pivmin;
    cnt += q < 0.f;
  }
  return cnt;
}

// Warp per eigenvalue: 32-way multisection of a Gershgorin interval in FP32
// down to a few ulps (the FP64 value comes from the Rayleigh quotient of the
// eigenvector).
__global__ void __launch_bounds__(256) tri_eigvals(const double* __restrict__ d,
                                                   const double* __restrict__ e, int m,
                                                   double* __restrict__ lam) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  extern __shared__ float shf[];
  float* dd = shf;
  float* e2 = shf + m;
  for (int i = threadIdx.x; i < m; i += blockDim.x) {
    dd[i] = (float)d[i];
    e2[i] = i + 1 < m ? (float)(e[i] * e[i]) : 0.f;
  }
  __syncthreads();
  if (warp >= m) return;
  float glo = 3e38f, ghi = -3e38f, emax = 0.f;
  for (int i = lane; i < m; i += 32) {
    float rr = (i > 0 ? fabsf((float)e[i - 1]) : 0.f) + (i + 1 < m ? fabsf((float)e[i]) : 0.f);
    glo = fminf(glo, dd[i] - rr);
    ghi = fmaxf(ghi, dd[i] + rr);
    emax = fmaxf(emax, e2[i]);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    glo = fminf(glo, __shfl_xor_sync(0xffffffffu, glo, o));
    ghi = fmaxf(ghi, __shfl_xor_sync(0xffffffffu, ghi, o));
    emax = fmaxf(emax, __shfl_xor_sync(0xffffffffu, emax, o));
  }
  const float span = fmaxf(ghi - glo, 1e-30f);
  glo -= 1e-6f * span;
  ghi += 1e-6f * span;
  const float pivmin = 1.17549435e-38f * fmaxf(1.f, emax) * 16.f;
  const int k = warp;
  float a = glo, b = ghi;
  for (int round = 0; round < 12; ++round) {
    const float x = a + (b - a) * (float)(lane + 1) / 33.f;
    const int c = sturm_count(dd, e2, m, x, pivmin);
    const unsigned ge = __ballot_sync(0xffffffffu, c >= k + 1);
    float na, nb;
    if (ge) {
      int l = __ffs(ge) - 1;
      nb = __shfl_sync(0xffffffffu, x, l);
      na = l > 0 ? __shfl_sync(0xffffffffu, x, l - 1) : a;
    } else {
      na = __shfl_sync(0xffffffffu, x, 31);
      nb = b;
    }
    a = na;
    b = nb;
    if (b - a <= 4.f * 1.1920929e-7f * fmaxf(fabsf(a), fabsf(b)) + pivmin) break;
  }
  if (lane == 0) lam[k] = 0.5 * ((double)a + (double)b);
}

// Thread per eigenvector: twisted factorisation of T - lam I in FP32 (forward
// and backward pivots, twist at the smallest |gamma|); the eigenvalue is then
// refined to the FP64 Rayleigh quotient z^T T z / z^T z (error below
// (eps_32 |T|)^2 / gap).  Z[i][k] (column k) FP32.  The pivots of the 32
// threads of a block live in shared memory, [i][thread].
__global__ void __launch_bounds__(32) tri_eigvecs(const double* __restrict__ d,
                                                  const double* __restrict__ e, int m,
                                                  double* __restrict__ lam, float* __restrict__ Z) {
  extern __shared__ float piv[];  // dp [m][32], dm [m][32]
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= m) return;
  float* dp = piv + threadIdx.x - (size_t)0;      // dp[i * 32]
  float* dm = piv + (size_t)m * 32 + threadIdx.x;  // dm[i * 32]
  const float l = (float)lam[k];
  const float tiny = 1e-30f;
  float q = (float)d[0] - l;
  if (fabsf(q) < tiny) q = tiny;
  dp[0] = q;
  for (int i = 1; i < m; ++i) {
    const float ei = (float)e[i - 1];
    q = ((float)d[i] - l) - __fdividef(ei * ei, q);
    if (fabsf(q) < tiny) q = tiny;
    dp[i * 32] = q;
  }
  q = (float)d[m - 1] - l;
  if (fabsf(q) < tiny) q = tiny;
  dm[(m - 1) * 32] = q;
  float best = fabsf(dp[(m - 1) * 32] + q - ((float)d[m - 1] - l));
  int r = m - 1;
  for (int i = m - 2; i >= 0; --i) {
    const float ei = (float)e[i];
    q = ((float)d[i] - l) - __fdividef(ei * ei, q);
    if (fabsf(q) < tiny) q = tiny;
    dm[i * 32] = q;
    const float g = fabsf(dp[i * 32] + q - ((float)d[i] - l));
    if (g < best) {
      best = g;
      r = i;
    }
  }
  float z = 1.f;
  Z[(size_t)r * m + k] = 1.f;
  for (int i = r - 1; i >= 0; --i) {
    z = -__fdividef((float)e[i], dp[i * 32]) * z;
    if (fabsf(z) < 1e-30f) z = 0.f;
    Z[(size_t)i * m + k] = z;
  }
  z = 1.f;
  for (int i = r + 1; i < m; ++i) {
    z = -__fdividef((float)e[i - 1], dm[i * 32]) * z;
    if (fabsf(z) < 1e-30f) z = 0.f;
    Z[(size_t)i * m + k] = z;
  }
  // FP64 norm and Rayleigh quotient, four independent partial sums
  double n0 = 0, n1 = 0, q0 = 0, q1 = 0;
  double zp = 0.0;
  for (int i = 0; i < m; ++i) {
    const double zi = (double)Z[(size_t)i * m + k];
    if (i & 1) {
      n1 += zi * zi;
      q1 += zi * (d[i] * zi + 2.0 * (i > 0 ? e[i - 1] * zp : 0.0));
    } else {
      n0 += zi * zi;
      q0 += zi * (d[i] * zi + 2.0 * (i > 0 ? e[i - 1] * zp : 0.0));
    }
    zp = zi;
  }
  const double nrm = n0 + n1;
  lam[k] = (q0 + q1) / nrm;
  const float sc = (float)(1.0 / sqrt(nrm));
  for (int i = 0; i < m; ++i) Z[(size_t)i * m + k] *= sc;
}

// Warp per eigenvector: x_k = H_0 ... H_{m-3} z_k, applying the reflectors
// from the last to the first; reflector rows are staged through shared
// memory 16 at a time for the 4 warps of a block.  X row k = x_k (FP32).
constexpr int kHChunk = 16;
__global__ void __launch_bounds__(128) householder_apply(const float* __restrict__ Vh,
                                                         const float* __restrict__ tau, int m,
                                                         const float* __restrict__ Z,
                                                         float* __restrict__ X) {
  extern __shared__ float vs[];  // [kHChunk][m]
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int k = blockIdx.x * 4 + warp;
  const bool active = k < m;
  float z[kMaxM / 32];
  const int per = (m + 31) / 32;
#pragma unroll
  for (int t = 0; t < kMaxM / 32; ++t) {
    int i = lane + 32 * t;
    z[t] = (active && t < per && i < m) ? Z[(size_t)i * m + k] : 0.f;
  }
  for (int j_hi = m - 3; j_hi >= 0; j_hi -= kHChunk) {
    const int j_lo = max(0, j_hi - kHChunk + 1);
    const int cnt = j_hi - j_lo + 1;
    __syncthreads();
    for (int q = warp; q < cnt; q += 4)
      for (int i = lane; i < m; i += 32) vs[(size_t)q * m + i] = Vh[(size_t)(j_hi - q) * m + i];
    __syncthreads();
    for (int q = 0; q < cnt; ++q) {
      const int j = j_hi - q;
      const float tj = tau[j];
      const float* v = vs + (size_t)q * m;
      float s = 0.f;
#pragma unroll
      for (int t = 0; t < kMaxM / 32; ++t) {
        int i = lane + 32 * t;
        if (t < per && i > j && i < m) s += v[i] * z[t];
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
      s *= tj;
#pragma unroll
      for (int t = 0; t < kMaxM / 32; ++t) {
        int i = lane + 32 * t;
        if (t < per && i > j && i < m) z[t] -= s * v[i];
      }
    }
  }
  if (active)
#pragma unroll
    for (int t = 0; t < kMaxM / 32; ++t) {
      int i = lane + 32 * t;
      if (t < per && i < m) X[(size_t)k * m + i] = z[t];
    }
}

// Scale rows of E by f_k = c_k (G_S) or c_k lam_k (G_M) into Es.
__global__ void scale_rows(const float* __restrict__ E, const double* __restrict__ c,
                           const double* __restrict__ lam, int m, float* __restrict__ Es) {
  const size_t n = (size_t)m * m;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x) {
    int k = (int)(i / m);
    Es[i] = E[i] * (float)(c[k] * (lam ? lam[k] : 1.0));
  }
}

__global__ void f32_to_f64(const float* __restrict__ a, double* __restrict__ b, size_t n,
                           double scale) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x)
    b[i] = scale * (double)a[i];
}

__global__ void f64_to_f32(const double* __restrict__ a, float* __restrict__ b, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x)
    b[i] = (float)a[i];
}

__global__ void mixed_loss(const double* __restrict__ c, const double* __restrict__ lam, int m,
                           double* __restrict__ loss, int* __restrict__ info) {
  __shared__ double red[32];
  double s = 0.0;
  for (int i = threadIdx.x; i < m; i += blockDim.x) s += c[i] * lam[i];
  for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double v = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) v += red[w];
    *loss = v;
    if (*info == 0 && !isfinite(v)) *info = -1;
  }
}

struct MixedWs {
  size_t Mw, linv_pp, LT, Y, C, Vh, tau, d, e, Z, X, E, Es, G, total;
};

MixedWs mixed_ws(int m) {
  MixedWs w{};
  size_t mm = (size_t)m * m, off = 0;
  auto take = [&](size_t bytes) {
    size_t o = off;
    off += al(bytes);
    return o;
  };
  w.Mw = take(mm * 8);
  w.linv_pp = take((size_t)(m / kCB) * kCB * kCB * 8);
  w.LT = take(mm * 8 * 2);   // L and L^T as float pairs
  w.Y = take(mm * 8);    // L^-1 S (FP64)
  w.C = take(mm * 4);
  w.Vh = take(mm * 4);
  w.tau = take((size_t)m * 4);
  w.d = take((size_t)m * 8);
  w.e = take((size_t)m * 8);
  w.Z = take(mm * 4);
  w.X = take(mm * 4);
  w.E = take(mm * 4);
  w.Es = take(mm * 4);
  w.G = take(mm * 4);
  w.total = off;
  return w;
}

// Row-major single-precision C[m][n] = alpha op(A) op(B) + beta C via cuBLAS.
int sgemm_rm(cublasHandle_t h, bool ta, bool tb, int m, int n, int k, float alpha,
             const float* A, int lda, const float* B, int ldb, float beta, float* C, int ldc) {
  cublasStatus_t st = cublasSgemm(h, tb ? CUBLAS_OP_T : CUBLAS_OP_N, ta ? CUBLAS_OP_T : CUBLAS_OP_N,
                                  n, m, k, &alpha, B, ldb, A, lda, &beta, C, ldc);
  if (st != CUBLAS_STATUS_SUCCESS) {
    set_error("cublasSgemm failed (%d)", (int)st);
    return NEB_ERR_CUDA;
  }
  return NEB_OK;
}

thread_local cublasHandle_t g_blas32 = nullptr;

int blas32(cudaStream_t s, cublasHandle_t* out) {
  if (!g_blas32 && cublasCreate(&g_blas32) != CUBLAS_STATUS_SUCCESS) {
    set_error("cublasCreate failed");
    return NEB_ERR_CUDA;
  }
  cublasSetStream(g_blas32, s);
  cublasSetMathMode(g_blas32, CUBLAS_DEFAULT_MATH);  // true FP32, no TF32
  *out = g_blas32;
  return NEB_OK;
}

}  // namespace
}  // namespace neb

using namespace neb;

extern "C" size_t neb_spectral_mixed_workspace_bytes(int m) {
  if (m < 64 || m > kMaxM || m % 64) return 0;
  return mixed_ws(m).total;
}

extern "C" int neb_spectral_mixed(int m, const double* M, const double* S, const double* c,
                                  double* lam, double* V, double* G_M, double* G_S, double* loss,
                                  int* info, void* workspace, size_t workspace_bytes,
                                  neb_stream_t stream_) {
  NEB_REQUIRE(m >= 64 && m <= kMaxM && m % 64 == 0,
              "neb_spectral_mixed: m = %d must be a multiple of 64 in [64, %d]", m, kMaxM);
  NEB_REQUIRE(M && S && c && lam && V && G_M && G_S && loss && info,
              "neb_spectral_mixed: null pointer");
  MixedWs w = mixed_ws(m);
  if (!workspace || workspace_bytes < w.total) {
    set_error("neb_spectral_mixed: workspace %zu < %zu bytes", workspace_bytes, w.total);
    return NEB_ERR_WORKSPACE;
  }
  cudaStream_t s = (cudaStream_t)stream_;
  char* ws = (char*)workspace;
  double* Mw = (double*)(ws + w.Mw);
  double* linv_pp = (double*)(ws + w.linv_pp);
  df* Ld = (df*)(ws + w.LT);
  df* LTd = Ld + (size_t)m * m;
  double* Y = (double*)(ws + w.Y);
  float* C = (float*)(ws + w.C);
  float* Vh = (float*)(ws + w.Vh);
  float* tau = (float*)(ws + w.tau);
  double* d = (double*)(ws + w.d);
  double* e = (double*)(ws + w.e);
  float* Z = (float*)(ws + w.Z);
  float* X = (float*)(ws + w.X);
  float* E = (float*)(ws + w.E);
  float* Es = (float*)(ws + w.Es);
  float* G = (float*)(ws + w.G);
  const size_t mm = (size_t)m * m;
  const int nb = m / kCB;

  NEB_CUDA_CHECK(cudaMemsetAsync(info, 0, sizeof(int), s));
  NEB_CUDA_CHECK(cudaMemcpyAsync(Mw, M, mm * 8, cudaMemcpyDeviceToDevice, s));
  {
    KernelScope ks("spec_cholesky_df", s, (double)m * m * m / 3.0, 16.0 * mm, 3 * nb - 2);
    for (int p = 0; p < nb; ++p) {
      chol_diag<<<1, 1024, 0, s>>>(Mw, m, p, linv_pp + (size_t)p * kCB * kCB, info);
      NEB_LAUNCH_CHECK();
      if (p + 1 < nb) {
        chol_panel<<<nb - p - 1, 1024, 0, s>>>(Mw, m, p, linv_pp + (size_t)p * kCB * kCB);
        NEB_LAUNCH_CHECK();
        int tiles = (nb - p - 1) * (nb - p) / 2;
        chol_update<<<tiles, 1024, 0, s>>>(Mw, m, p);
        NEB_LAUNCH_CHECK();
      }
    }
  }
  int st;
  const size_t trsm_smem = (size_t)kTrsmCols * m * sizeof(df);
  {
    // C = L^-1 S L^-T as two solves: Y = L^-1 S, C = L^-1 Y^T (S symmetric)
    KernelScope ks("spec_reduce_df", s, 2.0 * m * mm, 32.0 * mm, 3);
    split_factor<<<dim3(m / 32, m / 32), dim3(32, 8), 0, s>>>(Mw, m, Ld, LTd);
    NEB_LAUNCH_CHECK();
    df_trsm<<<m / kTrsmCols, 256, trsm_smem, s>>>(Ld, m, 0, S, 0, 0, Y, 0, 0);
    NEB_LAUNCH_CHECK();
    df_trsm<<<m / kTrsmCols, 256, trsm_smem, s>>>(Ld, m, 0, Y, 0, 1, C, 1, 0);
    NEB_LAUNCH_CHECK();
  }
  cublasHandle_t h;
  if ((st = blas32(s, &h))) return st;
  {
    static bool configured = false;
    const int rb = m / kCluster;
    const size_t smem = ((size_t)rb * m + 4 * m + 2 * kCluster) * sizeof(float);
    if (!configured) {
      NEB_CUDA_CHECK(cudaFuncSetAttribute(tridiag_cluster,
                                          cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int)(((size_t)kMaxM / kCluster * kMaxM + 4 * kMaxM +
                                                 2 * kCluster + 64) * sizeof(float))));
      configured = true;
    }
    KernelScope ks("spec_tridiag_cluster_fp32", s, 4.0 / 3.0 * m * mm, 8.0 * mm);
    tridiag_cluster<<<kCluster, kTriThreads, smem, s>>>(C, m, d, e, Vh, tau);
    NEB_LAUNCH_CHECK();
  }
  {
    KernelScope ks("spec_tridiag_eig", s, 0, 16.0 * m, 2);
    tri_eigvals<<<(m * 32 + 255) / 256, 256, (size_t)2 * m * 4, s>>>(d, e, m, lam);
    NEB_LAUNCH_CHECK();
    static bool vec_configured = false;
    if (!vec_configured) {
      NEB_CUDA_CHECK(cudaFuncSetAttribute(tri_eigvecs, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          2 * kMaxM * 32 * (int)sizeof(float)));
      vec_configured = true;
    }
    tri_eigvecs<<<(m + 31) / 32, 32, (size_t)2 * m * 32 * sizeof(float), s>>>(d, e, m, lam, Z);
    NEB_LAUNCH_CHECK();
  }
  {
    KernelScope ks("spec_backtransform_fp32", s, 2.0 * m * mm, 4.0 * mm * ((m + 3) / 4));
    householder_apply<<<(m + 3) / 4, 128, (size_t)kHChunk * m * 4, s>>>(Vh, tau, m, Z, X);
    NEB_LAUNCH_CHECK();
  }
  {
    KernelScope ks("spec_adjoints_fp32", s, 6.0 * m * mm, 24.0 * mm, 9);
    // rows of V: e_k = (L^-T x_k)^T, a backward solve with L^T on the columns of X^T
    df_trsm<<<m / kTrsmCols, 256, trsm_smem, s>>>(LTd, m, 1, X, 1, 1, E, 1, 1);
    NEB_LAUNCH_CHECK();
    int blocks = (int)std::min<size_t>((mm + 255) / 256, 2048);
    f32_to_f64<<<blocks, 256, 0, s>>>(E, V, mm, 1.0);
    NEB_LAUNCH_CHECK();
    // G_S = E^T diag(c) E ; G_M = -E^T diag(c lam) E
    scale_rows<<<blocks, 256, 0, s>>>(E, c, nullptr, m, Es);
    NEB_LAUNCH_CHECK();
    if ((st = sgemm_rm(h, true, false, m, m, m, 1.f, E, m, Es, m, 0.f, G, m))) return st;
    f32_to_f64<<<blocks, 256, 0, s>>>(G, G_S, mm, 1.0);
    NEB_LAUNCH_CHECK();
    scale_rows<<<blocks, 256, 0, s>>>(E, c, lam, m, Es);
    NEB_LAUNCH_CHECK();
    if ((st = sgemm_rm(h, true, false, m, m, m, 1.f, E, m, Es, m, 0.f, G, m))) return st;
    f32_to_f64<<<blocks, 256, 0, s>>>(G, G_M, mm, -1.0);
    NEB_LAUNCH_CHECK();
    mixed_loss<<<1, 256, 0, s>>>(c, lam, m, loss, info);
    NEB_LAUNCH_CHECK();
  }
  return NEB_OK;
}
