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
// Pipeline (no host synchronisation; the caller's stream plus one side
// stream that forks after the tridiagonalisation and joins before the
// back-transformation):
//   chol_first / chol_step                 blocked Cholesky, 32-column panels,
//                                          compensated FP32 (FP64-class); the
//                                          panel launches overlap their
//                                          predecessor (programmatic dependent
//                                          launch)
//   2 x df_solve                           C = L^-1 S L^-T by two left-looking
//                                          blocked triangular solves with inverse
//                                          diagonal blocks, compensated FP32
//   tridiag_cluster                        FP32 Householder tridiagonalisation in
//                                          one 16-CTA cluster, the rows held in
//                                          registers, per-column exchange by bulk
//                                          copies into mbarrier-guarded shared
//                                          memory; the last 64 columns by one
//                                          CTA with the block in shared memory
//   tri_eigvals                            eigenvalue brackets of T, warp per eigenvalue
//   tri_eigvecs                            eigenvectors of T by twisted factorisations,
//                                          eigenvalues refined to FP64 Rayleigh quotients
//   side: wy_factor / wy_apply on I        Q^T (FP32), 32 reflectors per block in
//                                          compact WY form, during the two above
//   gemm_tn                                X = Z^T Q^T (rows x_k = Q z_k)
//   df_solve, gemm_tn                      V rows = (L^-T x_k)^T; G_S and G_M in one pass
#include <cooperative_groups.h>
#include "elementwise.cuh"

namespace cg = cooperative_groups;

namespace neb {
namespace {

constexpr int kCB = 32;          // Cholesky block
constexpr int kMaxM = 512;

size_t al(size_t x) { return (x + 255) & ~size_t(255); }

// Asynchronous global -> shared copies (cp.async): a staging loop issues all
// of its copies before waiting once, instead of one dependent load per
// element.
__device__ __forceinline__ uint32_t sh_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void cp_async4(void* dst, const void* src) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(sh_u32(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async8(void* dst, const void* src) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(sh_u32(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async16(void* dst, const void* src) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(sh_u32(dst)), "l"(src)
               : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() {
  asm volatile("cp.async.commit_group;\n cp.async.wait_group 0;" ::: "memory");
}

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
// Compensated dot product (the Dot2 scheme of Ogita, Rump and Oishi): a
// running FP32 sum s with TwoSum error terms and the TwoProd / cross-term
// product errors collected in c, about 11 FP32 operations per term against
// 18 for df_add(acc, df_mul(x, y)), and the accuracy of twice FP32
// precision for the dot products of the Cholesky and the solves.
struct dot2 {
  float s = 0.f, c = 0.f;
};
__device__ __forceinline__ void dot2_add(dot2& a, df x, df y) {
  const float p = x.h * y.h;
  float pe = fmaf(x.h, y.h, -p);
  pe = fmaf(x.h, y.l, fmaf(x.l, y.h, pe));
  const float t = a.s + p, bb = t - a.s;
  a.c += ((a.s - (t - bb)) + (p - bb)) + pe;
  a.s = t;
}
__device__ __forceinline__ df dot2_df(dot2 a) { return df_quick(a.s, a.c); }
__device__ __forceinline__ df dot2_sum(dot2 a, dot2 b) {
  return df_add(dot2_df(a), dot2_df(b));
}

// FP64 -> float pairs (the Cholesky works on float pairs in memory, so its
// per-panel kernels do no FP64 conversions).
__global__ void to_df(const double* __restrict__ a, df* __restrict__ b, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x)
    b[i] = df_from(a[i]);
}

// ------------------------------------------------------------ Cholesky
// Blocked right-looking Cholesky of the FP64 matrix A, 32 x 32 tiles,
// compensated FP32 arithmetic, one launch per panel.  chol_step(p) has one
// CTA per trailing lower tile (i, j), p < j <= i: it forms the panel tiles
// L_ip = A_ip L_pp^-T (and L_jp) from the inverse diagonal factor, updates
// A_ij -= L_ip L_jp^T, writes L_ip (the CTA with j = p + 1) to the factor
// matrix Lw, and the CTA of tile (p + 1, p + 1) goes on to factor that tile
// and invert it for the next panel.  A keeps only trailing updates; the
// factor lives in Lw (lower tiles), the inverse diagonal tiles in linv_pp.

// 1 / sqrt(v): rsqrtf, then one Newton step r + r (1 - v r^2) / 2 with the
// residual 1 - v r^2 formed in compensated arithmetic (error ~ (2^-22)^2).
__device__ __forceinline__ df df_rsqrt(df v) {
  const float r0 = rsqrtf(v.h);
  const float q = r0 * r0;
  const df e = df_add(df{1.f, 0.f}, df_neg(df_mul(v, df{q, fmaf(r0, r0, -q)})));
  return df_quick(r0, 0.5f * r0 * e.h);
}

__device__ __forceinline__ void bar_named(int id, int n) {
  asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(n) : "memory");
}

// Programmatic dependent launch: a kernel launched with the
// programmatic-stream-serialization attribute may start while the previous
// kernel of the stream runs; it waits here until that kernel has completed
// and its writes are visible.  The previous kernel lets it start early.
__device__ __forceinline__ void pdl_wait() {
  asm volatile("griddepcontrol.wait;" ::: "memory");
}
__device__ __forceinline__ void pdl_allow_next() {
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

// Launch with the programmatic-stream-serialization attribute (the kernel
// calls pdl_wait before touching what its predecessor wrote).
template <typename... KArgs, typename... Args>
cudaError_t launch_pdl(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem,
                       cudaStream_t s, Args... args) {
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kernel, static_cast<KArgs>(args)...);
}

// Factor the SPD tile a (shared, 1024 threads: thread (i, j) = (ty, tx))
// into L and its inverse X = L^-1 (both lower).  One barrier per column:
// every thread forms l_ik = a_ik r with r = 1 / sqrt(a_kk), and the trailing
// entries take a_ij -= l_ik (a_jk r).  Column k concerns rows i >= k only, so
// warp i leaves the loop after its column and the barrier of column k counts
// warps k+1..31 (named barrier 1).  The reciprocal square root of the next
// pivot is taken once, by the thread that finished it.  The inverse comes
// out of the same loop (forward substitution on the identity, right-looking):
// B = I, and at column k the lanes j <= k of row i > k take
// B_ij -= l_ik (B_kj r); row k of B is final after column k-1, so row k of X
// is B_kj r, formed by warp k in its last column.  No barrier is added: rows
// of B are written only by their own warp, and row k is read after the
// barrier of column k-1.  Tm holds B.  Returns (through *bad) the first
// failing pivot + 1.
__device__ void tile_factor(df (*a)[kCB + 1], df (*L)[kCB + 1], df (*X)[kCB + 1],
                            df (*Tm)[kCB + 1], df* rinv, int* bad) {
  const int j = threadIdx.x & 31, i = threadIdx.x >> 5;
  L[i][j] = df{0.f, 0.f};
  X[i][j] = df{0.f, 0.f};
  Tm[i][j] = df{i == j ? 1.f : 0.f, 0.f};
  if (threadIdx.x == 0) {
    df a00 = a[0][0];
    if (!(a00.h > 0.f)) {  // not positive definite (or NaN)
      if (*bad == 0) *bad = 1;
      a00 = df{1.f, 0.f};
    }
    rinv[0] = df_rsqrt(a00);
  }
  __syncthreads();
  for (int k = 0; k <= i; ++k) {
    const df r = rinv[k];
    const df lik = df_mul(a[i][k], r);
    if (j == k) L[i][k] = lik;
    if (k == i) {  // this row's last column: its row of the inverse
      if (j <= i) X[i][j] = df_mul(Tm[i][j], r);
      break;
    }
    if (j <= i) {
      // one update form for both lane groups (no divergent second path):
      // j > k: a_ij -= l_ik (a_jk r);  j <= k: B_ij -= l_ik (B_kj r)
      df* x = j > k ? &a[i][j] : &Tm[i][j];
      const df* y = j > k ? &a[j][k] : &Tm[k][j];
      df v = df_add(*x, df_neg(df_mul(lik, df_mul(*y, r))));
      *x = v;
      if (i == k + 1 && j == k + 1) {
        if (!(v.h > 0.f)) {
          if (*bad == 0) *bad = k + 2;
          v = df{1.f, 0.f};
        }
        rinv[k + 1] = df_rsqrt(v);
      }
    }
    bar_named(1, (kCB - 1 - k) * 32);  // exactly warps k+1..31 arrive
  }
  __syncthreads();
}

__global__ void __launch_bounds__(1024) chol_first(const df* __restrict__ A, int m,
                                                   df* __restrict__ Lw, df* __restrict__ linv_pp,
                                                   int* __restrict__ info) {
  __shared__ df a[kCB][kCB + 1], L[kCB][kCB + 1], X[kCB][kCB + 1], Tm[kCB][kCB + 1];
  __shared__ df rinv[kCB];
  __shared__ int bad;
  pdl_allow_next();  // the first panel launch may take its SMs now
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  a[ty][tx] = A[(size_t)ty * m + tx];
  if (threadIdx.x == 0) bad = 0;
  __syncthreads();
  tile_factor(a, L, X, Tm, rinv, &bad);
  Lw[(size_t)ty * m + tx] = L[ty][tx];
  linv_pp[ty * kCB + tx] = X[ty][tx];
  if (threadIdx.x == 0 && bad && *info == 0) *info = m + bad;
}

__global__ void __launch_bounds__(1024) chol_step(df* __restrict__ A, int m, int p,
                                                  df* __restrict__ Lw, df* __restrict__ linv_pp,
                                                  int* __restrict__ info) {
  __shared__ df xi[kCB][kCB + 1];  // L_pp^-1, later L of the next diagonal tile
  __shared__ df li[kCB][kCB + 1];  // A_ip, then L_ip
  __shared__ df lj[kCB][kCB + 1];  // A_jp, then L_jp
  __shared__ df tl[kCB][kCB + 1];  // the updated tile
  __shared__ df rinv[kCB];
  __shared__ int bad;
  pdl_allow_next();
  pdl_wait();  // the previous panel (or chol_first) has finished
  int t = blockIdx.x, bi = p + 1;
  while (t >= bi - p) {  // tile index -> (bi, bj) with p < bj <= bi
    t -= bi - p;
    ++bi;
  }
  const int bj = p + 1 + t;
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  const int cb = p * kCB;
  xi[ty][tx] = linv_pp[(size_t)p * kCB * kCB + ty * kCB + tx];
  const df aip = A[(size_t)(bi * kCB + ty) * m + cb + tx];
  const df ajp = bj == bi ? aip : A[(size_t)(bj * kCB + ty) * m + cb + tx];
  const df aij = A[(size_t)(bi * kCB + ty) * m + bj * kCB + tx];
  if (threadIdx.x == 0) bad = 0;
  __syncthreads();
  // L_ip[r][c] = sum_k A_ip[r][k] X[c][k] (X lower: k <= c)
  dot2 d0, d1;
  li[ty][tx] = aip;
  lj[ty][tx] = ajp;
  __syncthreads();
  for (int k = 0; k <= tx; ++k) dot2_add(d0, li[ty][k], xi[tx][k]);
  if (bj != bi)
    for (int k = 0; k <= tx; ++k) dot2_add(d1, lj[ty][k], xi[tx][k]);
  const df s0 = dot2_df(d0), s1 = dot2_df(d1);
  __syncthreads();
  li[ty][tx] = s0;
  lj[ty][tx] = bj != bi ? s1 : s0;
  if (bj == p + 1) Lw[(size_t)(bi * kCB + ty) * m + cb + tx] = s0;
  __syncthreads();
  dot2 u0, u1;
#pragma unroll
  for (int k = 0; k < kCB; k += 2) {
    dot2_add(u0, li[ty][k], lj[tx][k]);
    dot2_add(u1, li[ty][k + 1], lj[tx][k + 1]);
  }
  const df upd = df_add(aij, df_neg(dot2_sum(u0, u1)));
  if (!(bi == p + 1 && bj == p + 1)) {
    A[(size_t)(bi * kCB + ty) * m + bj * kCB + tx] = upd;
    return;
  }
  // the next diagonal tile: factor and invert it here
  tl[ty][tx] = upd;
  __syncthreads();
  tile_factor(tl, xi, li, lj, rinv, &bad);
  const int r0 = (p + 1) * kCB;
  Lw[(size_t)(r0 + ty) * m + r0 + tx] = xi[ty][tx];
  linv_pp[(size_t)(p + 1) * kCB * kCB + ty * kCB + tx] = li[ty][tx];
  if (threadIdx.x == 0 && bad && *info == 0) *info = m + r0 + bad;
}

// The lower factor as float pairs, and its transpose (so both solves read
// rows): Ld[i][j] = L[i][j] (j <= i, else 0), LTd[j][i] = L[i][j].
__global__ void split_factor(const df* __restrict__ L, int m, df* __restrict__ Ld,
                             df* __restrict__ LTd) {
  __shared__ df t[32][33];
  const int bx = blockIdx.x * 32, by = blockIdx.y * 32;
  for (int r = threadIdx.y; r < 32; r += blockDim.y) {
    const int i = by + r, j = bx + threadIdx.x;
    df v = i >= j ? L[(size_t)i * m + j] : df{0.f, 0.f};
    Ld[(size_t)i * m + j] = v;
    t[r][threadIdx.x] = v;
  }
  __syncthreads();
  for (int r = threadIdx.y; r < 32; r += blockDim.y)
    LTd[(size_t)(bx + r) * m + by + threadIdx.x] = t[threadIdx.x][r];
}

// Inverses of the 32 x 32 diagonal blocks of L as float pairs, for both
// solves: DL[b] = L_bb^-1 (lower), DU[b] = (L_bb^-1)^T = (L^T)_bb^-1 (upper).
__global__ void __launch_bounds__(1024) split_dinv(const df* __restrict__ linv_pp,
                                                   df* __restrict__ DL, df* __restrict__ DU) {
  const int b = blockIdx.x, r = threadIdx.x >> 5, c = threadIdx.x & 31;
  const size_t base = (size_t)b * kCB * kCB;
  const df v = linv_pp[base + r * kCB + c];
  DL[base + r * kCB + c] = v;
  DU[base + c * kCB + r] = v;
}

constexpr int kSolveCols = 4;  // eigenvectors per block of the back-transformation

// Left-looking blocked triangular solve, compensated FP32: A Y = B with
// A = L (upper == 0, forward) or A = L^T (upper == 1, backward), kRLCols
// right-hand sides per CTA of 512 threads (m <= 512).  F holds the columns of
// A as rows, F[j][i] = A[i][j] (L^T as float pairs for the forward solve, L
// for the backward one), so a warp reading one row of the current block per
// lane reads 256 contiguous bytes.  Per 32-row block b, in elimination order:
//   every warp sums A_(r0+lane),j y_j over its share of the finished rows j
//   (Dot2, one sum per right-hand side), so the block's work is spread over
//   all sixteen warps instead of falling on the warps of the later blocks;
//   four warps (one per right-hand side) take B_b minus the sixteen partial
//   sums and multiply by the inverse diagonal block; y_b joins the finished
//   rows in shared memory.
// The factor entries of the next block do not depend on y, so they are
// loaded while the current block is reduced and solved.  The inverse
// diagonal blocks (rows padded to 33 pairs: a warp reading one row per lane
// is free of bank conflicts), B and Y live in shared memory.
// B(r, c) = b_trans ? B[c][r] : B[r][c] (FP64 or FP32); Y(r, c) goes to
// out[r][c] or, with out_trans, out[c][r].
constexpr int kRLCols = 4;
constexpr int kDPad = kCB + 1;
constexpr int kSolveWarps = kMaxM / 32;                  // 16
constexpr int kMaxJ = (kMaxM - kCB) / kSolveWarps;       // finished rows per warp, at most
size_t solve_smem(int m) {
  return ((size_t)(m / kCB) * kCB * kDPad + 2 * (size_t)m * kRLCols +
          (size_t)kSolveWarps * kRLCols * kCB) *
         sizeof(df);
}
__global__ void __launch_bounds__(kMaxM) df_solve(const df* __restrict__ F,
                                                  const df* __restrict__ D, int m, int upper,
                                                  const void* __restrict__ B, int b_f32,
                                                  int b_trans, void* __restrict__ out,
                                                  int out_f32, int out_trans) {
  extern __shared__ df dsh[];  // [nb][kCB][kDPad] inverse diagonal blocks
  __shared__ df stage[kRLCols][kCB];
  const int nb = m / kCB;
  df* ysh = dsh + (size_t)nb * kCB * kDPad;      // [kRLCols][m] solution
  df* bsh = ysh + (size_t)kRLCols * m;           // [kRLCols][m] right-hand sides
  df* part = bsh + (size_t)kRLCols * m;          // [kSolveWarps][kRLCols][kCB] partial sums
  const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
  const int c0 = blockIdx.x * kRLCols;
  for (int t = tid; t < nb * kCB * kCB; t += blockDim.x)
    cp_async8(dsh + (size_t)(t / kCB) * kDPad + t % kCB, D + t);
  for (int t = tid; t < m * kRLCols; t += blockDim.x) {
    const int r = b_trans ? t % m : t / kRLCols, c = b_trans ? t / m : t % kRLCols;
    const size_t bi = b_trans ? (size_t)(c0 + c) * m + r : (size_t)r * m + c0 + c;
    bsh[(size_t)c * m + r] =
        df_from(b_f32 ? (double)((const float*)B)[bi] : ((const double*)B)[bi]);
  }
  cp_async_wait_all();
  __syncthreads();
  df fv[kMaxJ];  // F entries of this warp's finished rows for the current block
  for (int bb = 0; bb < nb; ++bb) {
    const int b = upper ? nb - 1 - bb : bb, r0 = b * kCB;
    const int d0 = upper ? r0 + kCB : 0;       // finished rows [d0, d0 + bb kCB)
    const int nj = bb * kCB / kSolveWarps;     // of which this warp takes nj
    dot2 u[kRLCols];
    // nj is uniform over the CTA: leaving the unrolled loop by a branch issues
    // only the nj terms (a guard would issue all kMaxJ, predicated off)
#pragma unroll
    for (int q = 0; q < kMaxJ; ++q) {
      if (q >= nj) break;
      const int j = d0 + w + kSolveWarps * q;
#pragma unroll
      for (int c = 0; c < kRLCols; ++c) dot2_add(u[c], fv[q], ysh[(size_t)c * m + j]);
    }
    if (bb + 1 < nb) {  // the next block's entries, in flight during the reduction
      const int b1 = upper ? nb - 2 - bb : bb + 1, r1 = b1 * kCB;
      const int e0 = upper ? r1 + kCB : 0, nj1 = (bb + 1) * kCB / kSolveWarps;
#pragma unroll
      for (int q = 0; q < kMaxJ; ++q) {
        if (q >= nj1) break;
        fv[q] = F[(size_t)(e0 + w + kSolveWarps * q) * m + r1 + lane];
      }
    }
#pragma unroll
    for (int c = 0; c < kRLCols; ++c)
      part[((size_t)w * kRLCols + c) * kCB + lane] = dot2_df(u[c]);
    __syncthreads();
    if (w < kRLCols) {  // warp c: right-hand side c of the block
      const int c = w, row = r0 + lane;
      df s = bsh[(size_t)c * m + row];
#pragma unroll
      for (int v = 0; v < kSolveWarps; ++v)
        s = df_add(s, df_neg(part[((size_t)v * kRLCols + c) * kCB + lane]));
      stage[c][lane] = s;
      __syncwarp();
      const df* dp = dsh + ((size_t)b * kCB + lane) * kDPad;  // row lane of D_b
      dot2 y;
#pragma unroll 8
      for (int j = 0; j < kCB; ++j) dot2_add(y, dp[j], stage[c][j]);
      ysh[(size_t)c * m + row] = dot2_df(y);
    }
    __syncthreads();
  }
  for (int t = tid; t < m * kRLCols; t += blockDim.x) {
    const int r = out_trans ? t % m : t / kRLCols, c = out_trans ? t / m : t % kRLCols;
    const size_t oi = out_trans ? (size_t)(c0 + c) * m + r : (size_t)r * m + c0 + c;
    const df v = ysh[(size_t)c * m + r];
    if (out_f32) ((float*)out)[oi] = v.h + v.l;
    else ((double*)out)[oi] = df_to(v);
  }
}

// ------------------------------------------------- cluster tridiagonalisation
// C: [m][m] FP32 (symmetrised on load).  Outputs: d[m], e[m-1] (FP64 of the
// FP32 tridiagonal), Vh[m][m] (row k = Householder vector of step k, zero up
// to index k), tau[m].
//
// One cluster of kTriCluster CTAs on kTriCluster SMs.  Rows are dealt
// cyclically (row i on CTA i % kTriCluster) and live in REGISTERS: eight
// threads share a row, thread `sub` holding chunks of four columns
// q = sub + 8 t as a[t] (16 float4 at m = 512).  Every CTA keeps a replica of
// the current pivot row, so the Householder vector of column k (row k by
// symmetry) is formed locally.  Per column k:
//   sigma = |row_k[k+1:]|^2 (warp partials left by the previous column),
//   alpha, tau;
//   one pass over the own rows applies the pending rank-2 update of column
//   k-1 (A -= v p^T + w v^T, w = p - K2 v) and forms p_i = tau A_i v;
//   every CTA stages (p_i, A_{i,k+1}) of its rows (column k+1 before
//   update k, = row k+1 by symmetry) and its warp partials of p.v in one
//   288-byte message and bulk-copies it into every CTA of the cluster
//   (sixteen copies, one per issuing thread), completing on the receiver's
//   mbarrier (no cluster barrier): the receivers wait for the byte count;
//   K2 = tau p.v; the next pivot row, row k+1 after update k, is formed by
//   every CTA from the pushed column; one __syncthreads.
// The update is lazy by one column, so each element of the trailing matrix
// is read and written once per column.  Every 32 columns the front chunk of
// every thread dies and the register array shifts down by one, so the chunk
// holding column k+1 is always a[0] of thread (k+1)/4 % 8 (no dynamic
// register indexing).  v_{k+1} = x1 - alpha is applied through scalar
// corrections, so the replica holds the raw row.
// Near the end a column costs the cluster mostly exchange latency, so at
// column k0 = m - min(m, kTriTail) every CTA applies the pending update to its
// rows and stores the trailing block into CTA 0's shared memory
// (distributed shared memory), and CTA 0 finishes the columns alone with
// __syncthreads in place of the exchange; the other CTAs exit.
constexpr int kTriCluster = 16;
constexpr int kTriThreads = 8 * kMaxM / kTriCluster;  // 8 threads per row
constexpr int kTriWarps = kTriThreads / 32;
constexpr int kTriRows = kMaxM / kTriCluster;          // rows per CTA at m = 512
constexpr int kTriMsg = 2 * kTriRows + kTriWarps;      // floats per CTA message
constexpr int kTriChunks = kMaxM / 32;                 // float4 per thread
constexpr int kTriTail = 64;  // trailing block finished by one CTA in shared memory
constexpr int kTriTailRows = kTriTail / 32;  // rows per eight-thread group in the tail
// the handoff column k0 = m - min(m, kTriTail) must be a multiple of 32 (a
// whole number of register-array shifts); m is a multiple of 64
static_assert(kTriTail % 32 == 0 && kTriTail >= 32 && kTriTail <= kMaxM, "tail size");

__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ uint32_t smem_addr(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ uint32_t cluster_map(uint32_t a, int rank) {
  uint32_t r;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(a), "r"(rank));
  return r;
}
// Bulk copy of `bytes` (a multiple of 16) from this CTA's shared memory to
// another CTA's, completing (complete_tx) on that CTA's mbarrier; the
// issuing thread tracks the reads of its source through bulk async-groups.
__device__ __forceinline__ void bulk_to_cluster(uint32_t dst, uint32_t src, uint32_t bytes,
                                                uint32_t rbar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.shared::cta.mbarrier::complete_tx::bytes [%0], [%1], %2, "
      "[%3];" ::"r"(dst),
      "r"(src), "r"(bytes), "r"(rbar)
      : "memory");
}
__device__ __forceinline__ void bulk_commit() {
  asm volatile("cp.async.bulk.commit_group;" ::: "memory");
}
template <int N>
__device__ __forceinline__ void bulk_wait_read() {
  asm volatile("cp.async.bulk.wait_group.read %0;" ::"n"(N) : "memory");
}
// Bounded wait (acquire at cluster scope) for the phase of parity `parity`;
// the thread sleeps in the hardware up to 20 us per try; false after ~2^32
// cycles (about two seconds).
__device__ __forceinline__ bool cluster_bar_wait(uint32_t bar, uint32_t parity) {
  const long long t0 = clock64();
  uint32_t done;
  do {
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.acquire.cluster.shared::cta.b64 p, [%1], "
        "%2, %3;\n selp.u32 %0, 1, 0, p;\n}"
        : "=r"(done)
        : "r"(bar), "r"(parity), "r"(20000u)
        : "memory");
    if (done) return true;
  } while (clock64() - t0 < (1ll << 32));
  return false;
}

__global__ void __launch_bounds__(kTriThreads, 1)
tridiag_cluster(const float* __restrict__ C, int m, int k0, double* __restrict__ d_out,
                double* __restrict__ e_out, float* __restrict__ Vh, float* __restrict__ tau_out,
                int* __restrict__ info) {
  cg::cluster_group cluster = cg::this_cluster();
  const int rank = (int)cluster.block_rank();
  const int rb = m / kTriCluster;
  extern __shared__ __align__(16) float sm[];
  float* vrow = sm;                        // [2][m] pivot rows k (parity k & 1), zero at j <= k
  float* pnat = vrow + 2 * m;              // [2][m] p of column k, natural order
  float* recv = pnat + 2 * m;              // [2][kTriCluster][kTriMsg] received messages
  float* stage = recv + 2 * kTriCluster * kTriMsg;  // [2][kTriMsg] this CTA's message
  float* red = stage + 2 * kTriMsg;        // [2][kTriWarps] partials of sigma
  float* T = red + 2 * kTriWarps;           // [R][R] trailing block (CTA 0), R = m - k0
  __shared__ __align__(8) unsigned long long bars[2];
  __shared__ int tail_abort;               // CTA 0: some CTA's exchange stalled
  const int tid = threadIdx.x;
  const int warp = tid >> 5, lane = tid & 31;
  const int li = tid >> 3, sub = tid & 7;
  const bool has_row = li < rb;
  const int gi = li * kTriCluster + rank;  // global row of this thread
  const int m4 = m >> 2, nsub = m4 >> 3;   // float4 chunks per row, per thread

  float4 a[kTriChunks];
#pragma unroll
  for (int t = 0; t < kTriChunks; ++t) {
    a[t] = make_float4(0.f, 0.f, 0.f, 0.f);
    if (has_row && t < nsub) {
      const int j = 4 * (sub + 8 * t);
      const float* ci = C + (size_t)gi * m + j;
      a[t].x = 0.5f * (ci[0] + C[(size_t)(j + 0) * m + gi]);
      a[t].y = 0.5f * (ci[1] + C[(size_t)(j + 1) * m + gi]);
      a[t].z = 0.5f * (ci[2] + C[(size_t)(j + 2) * m + gi]);
      a[t].w = 0.5f * (ci[3] + C[(size_t)(j + 3) * m + gi]);
    }
  }
  {  // pivot row 0 and its sigma partials
    float part = 0.f;
    for (int j = tid; j < m; j += kTriThreads) {
      const float x0 = 0.5f * (C[j] + C[(size_t)j * m]);
      if (j == 0 && rank == 0) d_out[0] = x0;
      const float x = j > 0 ? x0 : 0.f;
      vrow[j] = x;
      vrow[m + j] = 0.f;
      pnat[j] = 0.f;
      pnat[m + j] = 0.f;
      part += x * x;
    }
    part = warp_sum(part);
    if (lane == 0) red[warp] = part;
  }
  if (tid == 0) {
    tail_abort = 0;
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(&bars[0])) : "memory");
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(&bars[1])) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  const uint32_t base = smem_addr(sm);
  // threads tid < kTriCluster each copy the message to CTA tid
  const uint32_t rdst = cluster_map(base, tid % kTriCluster);
  const uint32_t bar_off = smem_addr(&bars[0]) - base;  // the same in every CTA
  bool failed = false;
  cluster.sync();  // barriers initialised and every CTA running before the first push
  float pprev = 0.f, vprev = 0.f, K2prev = 0.f;  // this row's p, v and K2 of column k-1

  for (int k = 0; k < k0; ++k) {
    const int par = k & 1, npar = par ^ 1;
    const float* vcur = vrow + par * m;
    float* vprv = vrow + npar * m;
    const float* pbp = pnat + npar * m;
    float sigma = 0.f;
    {
      const float4* r4 = reinterpret_cast<const float4*>(red + par * kTriWarps);
#pragma unroll
      for (int c = 0; c < kTriWarps / 4; ++c) {
        const float4 r = r4[c];
        sigma += (r.x + r.y) + (r.z + r.w);
      }
    }
    const float x1 = vcur[k + 1];
    const float alpha = sigma > 0.f ? -copysignf(sigma * rsqrtf(sigma), x1) : 0.f;
    const float v1 = x1 - alpha;
    const float vv = sigma - x1 * x1 + v1 * v1;
    const float tau = vv > 0.f ? __fdividef(2.f, vv) : 0.f;
    if (tid == 0)
      asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(
                       smem_addr(&bars[par])),
                   "r"(4u * kTriCluster * kTriMsg)
                   : "memory");
    if (rank == 0 && tid == 0) {
      e_out[k] = alpha;
      tau_out[k] = tau;
    }
    if (tid < rb) {
      const int j = rank * rb + tid;
      Vh[(size_t)k * m + j] = j == k + 1 ? v1 : vcur[j];
    }
    // pending update of column k-1 fused with p_i = tau A_i v of column k
    if (k > 0 && ((k + 1) & 31) == 0) {
#pragma unroll
      for (int t = 0; t < kTriChunks - 1; ++t) a[t] = a[t + 1];
    }
    const int j4 = (k + 1) >> 2, T = j4 >> 3, sk = j4 & 7;  // a[t] = chunk sub + 8 (t + T)
    const bool active = has_row && gi > k;
    float pi = 0.f, vi = 0.f, sacc = 0.f;
    if (active) {
      const float wprev = pprev - K2prev * vprev;
      const float4* vc4 = reinterpret_cast<const float4*>(vcur);
      const float4* vp4 = reinterpret_cast<const float4*>(vprv);
      const float4* pp4 = reinterpret_cast<const float4*>(pbp);
      float s0 = 0.f, s1 = 0.f, s2 = 0.f, s3 = 0.f;
#pragma unroll
      for (int t = 0; t < kTriChunks; ++t) {
        if ((t > 0 || sub >= sk) && t + T < nsub) {
          const int q = sub + 8 * (t + T);
          const float4 pp = pp4[q], vp = vp4[q], vc = vc4[q];
          a[t].x = fmaf(-wprev, vp.x, fmaf(-vprev, pp.x, a[t].x));
          a[t].y = fmaf(-wprev, vp.y, fmaf(-vprev, pp.y, a[t].y));
          a[t].z = fmaf(-wprev, vp.z, fmaf(-vprev, pp.z, a[t].z));
          a[t].w = fmaf(-wprev, vp.w, fmaf(-vprev, pp.w, a[t].w));
          s0 = fmaf(a[t].x, vc.x, s0);
          s1 = fmaf(a[t].y, vc.y, s1);
          s2 = fmaf(a[t].z, vc.z, s2);
          s3 = fmaf(a[t].w, vc.w, s3);
        }
      }
      sacc = (s0 + s1) + (s2 + s3);
    }
    sacc += __shfl_xor_sync(0xffffffffu, sacc, 1);
    sacc += __shfl_xor_sync(0xffffffffu, sacc, 2);
    sacc += __shfl_xor_sync(0xffffffffu, sacc, 4);
    const int ck = (k + 1) & 3;  // A_{i,k+1}: component ck of a[0] of thread sk
    const float own = ck == 0 ? a[0].x : ck == 1 ? a[0].y : ck == 2 ? a[0].z : a[0].w;
    const float aik1 = __shfl_sync(0xffffffffu, own, (lane & ~7) | sk);
    if (active) {
      pi = tau * (sacc - alpha * aik1);
      vi = gi == k + 1 ? v1 : vcur[gi];
    }
    // every lane of a row holds its p_i v_i: two levels sum the warp's four rows
    float part = pi * vi;
    part += __shfl_xor_sync(0xffffffffu, part, 8);
    part += __shfl_xor_sync(0xffffffffu, part, 16);
    {
      float* stg = stage + par * kTriMsg;  // (p_i, A_{i,k+1}) by local row, then partials
      if (has_row && sub == 0) {
        stg[2 * li] = pi;
        stg[2 * li + 1] = aik1;
      }
      if (lane == 0) stg[2 * kTriRows + warp] = part;
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      __syncthreads();
      if (tid < kTriCluster) {
        bulk_to_cluster(rdst + 4u * (uint32_t)(recv + (par * kTriCluster + rank) * kTriMsg - sm),
                        smem_addr(stg), 4u * kTriMsg, rdst + bar_off + 8u * par);
        bulk_commit();
      }
    }
    failed = !cluster_bar_wait(smem_addr(&bars[par]), (uint32_t)(k >> 1) & 1u);
    const float* rv = recv + par * kTriCluster * kTriMsg;  // message of CTA r at rv + r kTriMsg
    float pv;
    {
      static_assert(kTriCluster == 16 && kTriWarps == 8, "two float4 of p.v partials per CTA");
      const float4 q =
          reinterpret_cast<const float4*>(rv + (lane >> 1) * kTriMsg + 2 * kTriRows)[lane & 1];
      pv = warp_sum((q.x + q.y) + (q.z + q.w));
    }
    const float K2 = tau * pv;
    // pivot row k+1 after update k, from column k+1 as it stood before it;
    // row j travels in the message of CTA j % 16 at local row j / 16
    const int k1 = k + 1;
    const float w1 = rv[(k1 % kTriCluster) * kTriMsg + 2 * (k1 / kTriCluster)] - K2 * v1;
    part = 0.f;
    for (int j = tid; j < m; j += kTriThreads) {
      const float2 pc = *reinterpret_cast<const float2*>(rv + (j % kTriCluster) * kTriMsg +
                                                         2 * (j / kTriCluster));
      pnat[par * m + j] = pc.x;
      float nv = 0.f;
      if (j > k) {
        nv = pc.y - (v1 * pc.x + w1 * vcur[j]);
        if (j == k + 1) {
          if (rank == 0) d_out[k + 1] = nv + w1 * alpha;
          nv = 0.f;
        }
      }
      part += nv * nv;
      vprv[j] = nv;
    }
    part = warp_sum(part);
    if (lane == 0) red[npar * kTriWarps + warp] = part;
    if (tid < kTriCluster) bulk_wait_read<1>();  // column k-1's copies have read their stage
    pprev = pi;
    vprev = vi;
    K2prev = K2;
    failed = __syncthreads_or(failed);
    if (failed) break;
  }
  if (tid < kTriCluster) bulk_wait_read<0>();
  const int R = m - k0, R4 = R >> 2;
  if (failed) {
    // a stalled exchange: report it, and let copies still in flight land
    // before any CTA of the cluster exits
    if (tid == 0) {
      atomicExch(info, -2);
      *cluster.map_shared_rank(&tail_abort, 0) = 1;
    }
    __nanosleep(50000);
  } else {
    // hand the trailing block (rows and columns k0.., update of column k0-1
    // applied) to CTA 0; after k0 / 32 shifts a[t] holds chunk sub + 8 (t + S)
    const int par = k0 & 1, npar = par ^ 1;
    const float4* vp4 = reinterpret_cast<const float4*>(vrow + npar * m);
    const float4* pp4 = reinterpret_cast<const float4*>(pnat + npar * m);
    const float wprev = pprev - K2prev * vprev;
    const int S = k0 >> 5;
    float4* T0 = reinterpret_cast<float4*>(cluster.map_shared_rank(T, 0));
    if (has_row && gi >= k0) {
#pragma unroll
      for (int t = 0; t < kTriChunks; ++t) {
        if (t + S < nsub) {
          const int q = sub + 8 * (t + S);
          const float4 pp = pp4[q], vp = vp4[q];
          float4 x = a[t];
          x.x = fmaf(-wprev, vp.x, fmaf(-vprev, pp.x, x.x));
          x.y = fmaf(-wprev, vp.y, fmaf(-vprev, pp.y, x.y));
          x.z = fmaf(-wprev, vp.z, fmaf(-vprev, pp.z, x.z));
          x.w = fmaf(-wprev, vp.w, fmaf(-vprev, pp.w, x.w));
          T0[(size_t)(gi - k0) * R4 + q - (k0 >> 2)] = x;
        }
      }
    }
    // reflector rows k0.. are zero left of column k0
    for (int idx = rank * kTriThreads + tid; idx < R * k0; idx += kTriCluster * kTriThreads)
      Vh[(size_t)(k0 + idx / k0) * m + idx % k0] = 0.f;
  }
  cluster.sync();  // the trailing block is in CTA 0; the other CTAs are done
  if (rank != 0 || tail_abort) return;

  // ---- tail: columns k0 .. m-3 by this CTA alone, the block in shared
  // memory (local indices r = global - k0).  The same lazy scheme as above:
  // per column one pass over rows c+1.. applies the update of column c-1 and
  // forms p = tau T v; the pivot row c+1 after update c is formed from the
  // updated row; two __syncthreads per column.  xr[2][.] holds pivot rows
  // (raw, zero at j <= c), pn[2][.] p of the last two columns.
  float* xr = vrow;
  float* pn = pnat;
  float* pvred = stage;  // [kTriWarps] partials of p.v
  {
    float part = 0.f;
    for (int j = tid; j < R; j += kTriThreads) {
      const float x = j > 0 ? T[j] : 0.f;
      xr[j] = x;
      xr[m + j] = 0.f;
      pn[j] = 0.f;
      pn[m + j] = 0.f;
      part += x * x;
    }
    part = warp_sum(part);
    if (lane == 0) red[warp] = part;
  }
  __syncthreads();
  const float4* T4 = reinterpret_cast<const float4*>(T);
  float K2p = 0.f;  // K2 of column c-1 (no pending update before column 0)
  for (int c = 0; c + 2 < R; ++c) {
    const int k = k0 + c;
    const int par = c & 1, npar = par ^ 1;
    const float* xc = xr + par * m;  // raw pivot row c
    float* xp = xr + npar * m;       // raw pivot row c-1; becomes row c+1
    float* pc = pn + par * m;
    const float* pp = pn + npar * m;
    float sigma = 0.f;
#pragma unroll
    for (int w = 0; w < kTriWarps; ++w) sigma += red[par * kTriWarps + w];
    const float x1 = xc[c + 1];
    const float alpha = sigma > 0.f ? -copysignf(sigma * rsqrtf(sigma), x1) : 0.f;
    const float v1 = x1 - alpha;
    const float vv = sigma - x1 * x1 + v1 * v1;
    const float tau = vv > 0.f ? __fdividef(2.f, vv) : 0.f;
    if (tid == 0) {
      e_out[k] = alpha;
      tau_out[k] = tau;
    }
    for (int j = tid; j < R; j += kTriThreads)
      Vh[(size_t)k * m + k0 + j] = j == c + 1 ? v1 : xc[j];
    // rows c+1+li+32u: pending update of column c-1, then T_i . x
    const int q0 = (c + 1) >> 2;
    float vpi[kTriTailRows], wpi[kTriTailRows], acc[kTriTailRows];
#pragma unroll
    for (int u = 0; u < kTriTailRows; ++u) {
      const int i = c + 1 + li + 32 * u;
      vpi[u] = i < R ? xp[i] : 0.f;
      wpi[u] = i < R ? pp[i] - K2p * vpi[u] : 0.f;
      acc[u] = 0.f;
    }
    const float4* pp4 = reinterpret_cast<const float4*>(pp);
    const float4* xp4 = reinterpret_cast<const float4*>(xp);
    const float4* xc4 = reinterpret_cast<const float4*>(xc);
    float4* Tw4 = reinterpret_cast<float4*>(T);
    // two chunks per trip keep twice the shared-memory loads in flight
    for (int q = q0 + sub; q < R4; q += 16) {
      const bool two = q + 8 < R4;
      const int q2 = two ? q + 8 : q;
      const float4 pq = pp4[q], vq = xp4[q], xq = xc4[q];
      const float4 pq2 = pp4[q2], vq2 = xp4[q2], xq2 = xc4[q2];
#pragma unroll
      for (int u = 0; u < kTriTailRows; ++u) {
        const int i = c + 1 + li + 32 * u;
        if (i < R) {
          float4* row = Tw4 + (size_t)i * R4;
          float4 x = T4[(size_t)i * R4 + q];
          float4 y = T4[(size_t)i * R4 + q2];
          x.x = fmaf(-wpi[u], vq.x, fmaf(-vpi[u], pq.x, x.x));
          x.y = fmaf(-wpi[u], vq.y, fmaf(-vpi[u], pq.y, x.y));
          x.z = fmaf(-wpi[u], vq.z, fmaf(-vpi[u], pq.z, x.z));
          x.w = fmaf(-wpi[u], vq.w, fmaf(-vpi[u], pq.w, x.w));
          row[q] = x;
          acc[u] = fmaf(x.x, xq.x, fmaf(x.y, xq.y, fmaf(x.z, xq.z, fmaf(x.w, xq.w, acc[u]))));
          if (two) {
            y.x = fmaf(-wpi[u], vq2.x, fmaf(-vpi[u], pq2.x, y.x));
            y.y = fmaf(-wpi[u], vq2.y, fmaf(-vpi[u], pq2.y, y.y));
            y.z = fmaf(-wpi[u], vq2.z, fmaf(-vpi[u], pq2.z, y.z));
            y.w = fmaf(-wpi[u], vq2.w, fmaf(-vpi[u], pq2.w, y.w));
            row[q2] = y;
            acc[u] = fmaf(y.x, xq2.x, fmaf(y.y, xq2.y, fmaf(y.z, xq2.z, fmaf(y.w, xq2.w, acc[u]))));
          }
        }
      }
    }
    __syncwarp();  // the group's chunk holding column c+1 is stored
    float part = 0.f;
#pragma unroll
    for (int u = 0; u < kTriTailRows; ++u) {
      float sacc = acc[u];
      sacc += __shfl_xor_sync(0xffffffffu, sacc, 1);
      sacc += __shfl_xor_sync(0xffffffffu, sacc, 2);
      sacc += __shfl_xor_sync(0xffffffffu, sacc, 4);
      const int i = c + 1 + li + 32 * u;
      if (i < R && sub == 0) {
        const float pi = tau * (sacc - alpha * T[(size_t)i * R + c + 1]);
        pc[i] = pi;
        part += pi * (i == c + 1 ? v1 : xc[i]);
      }
    }
    part = warp_sum(part);
    if (lane == 0) pvred[warp] = part;
    __syncthreads();
    float pv = 0.f;
#pragma unroll
    for (int w = 0; w < kTriWarps; ++w) pv += pvred[w];
    const float K2 = tau * pv;
    const float w1 = pc[c + 1] - K2 * v1;
    // pivot row c+1 after update c
    part = 0.f;
    for (int j = tid; j < R; j += kTriThreads) {
      float nv = 0.f;
      if (j > c + 1) nv = T[(size_t)(c + 1) * R + j] - (v1 * pc[j] + w1 * xc[j]);
      if (j == c + 1) d_out[k + 1] = T[(size_t)(c + 1) * R + j] - (v1 * pc[j] + w1 * v1);
      xp[j] = nv;
      part += nv * nv;
    }
    part = warp_sum(part);
    if (lane == 0) red[npar * kTriWarps + warp] = part;
    K2p = K2;
    __syncthreads();
  }
  const int pl = (R - 3) & 1;  // parity of the last column
  if (tid == 0) {
    e_out[m - 2] = xr[(pl ^ 1) * m + R - 1];
    tau_out[m - 2] = 0.f;
    tau_out[m - 1] = 0.f;
    // d_{m-1}: the last element with the pending update of column m-3
    const float vl = xr[pl * m + R - 1], pl_ = pn[pl * m + R - 1];
    const float w = pl_ - K2p * vl;
    d_out[m - 1] = T[(size_t)(R - 1) * R + R - 1] - (vl * pl_ + w * vl);
  }
  for (int k = m - 2; k < m; ++k)
    for (int j = tid; j < R; j += kTriThreads) Vh[(size_t)k * m + k0 + j] = 0.f;
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

// Two threads per eigenvector: twisted factorisation of T - lam I in FP32.
// Warp 0 of a 64-thread block runs the forward pivots of 32 eigenvectors
// and warp 1 the backward pivots, at the same time; the twist index r is the
// smallest |gamma| (each warp scans half of the rows); then warp 0 solves
// z upwards from r and warp 1 downwards.  The eigenvalue is refined to the
// Rayleigh quotient z^T T z / z^T z, accumulated in compensated FP32 (T is
// FP32, so every product is exact as a float pair) with an error below
// (eps_32 |T|)^2 / gap, each warp summing half of the rows.  Z[i][k] (column
// k) FP32.  T and the pivots ([i][eigenvector]) live in shared memory.
__device__ __forceinline__ df two_prod(float a, float b) {
  const float p = a * b;
  return {p, fmaf(a, b, -p)};
}

__global__ void __launch_bounds__(64) tri_eigvecs(const double* __restrict__ d,
                                                  const double* __restrict__ e, int m,
                                                  double* __restrict__ lam, float* __restrict__ Z) {
  extern __shared__ float piv[];  // dp [m][32], dm [m][32], dd [m], ee [m]
  __shared__ float best_g[2][32];
  __shared__ int best_i[2][32];
  __shared__ df part_n[2][32], part_q[2][32];
  __shared__ float scale[32];
  const int v = threadIdx.x & 31, half = threadIdx.x >> 5;
  float* dp = piv + v;                       // dp[i * 32]
  float* dm = piv + (size_t)m * 32 + v;      // dm[i * 32]
  float* dd = piv + (size_t)m * 64;
  float* ee = dd + m;
  for (int i = threadIdx.x; i < m; i += blockDim.x) {
    dd[i] = (float)d[i];
    ee[i] = i + 1 < m ? (float)e[i] : 0.f;
  }
  __syncthreads();
  const int k = blockIdx.x * 32 + v;
  const bool has = k < m;
  const float l = has ? (float)lam[k] : 0.f;
  const float tiny = 1e-30f;
  if (has) {
    if (half == 0) {  // forward pivots
      float q = dd[0] - l;
      if (fabsf(q) < tiny) q = tiny;
      dp[0] = q;
      for (int i = 1; i < m; ++i) {
        const float ei = ee[i - 1];
        q = (dd[i] - l) - __fdividef(ei * ei, q);
        if (fabsf(q) < tiny) q = tiny;
        dp[i * 32] = q;
      }
    } else {  // backward pivots
      float q = dd[m - 1] - l;
      if (fabsf(q) < tiny) q = tiny;
      dm[(m - 1) * 32] = q;
      for (int i = m - 2; i >= 0; --i) {
        const float ei = ee[i];
        q = (dd[i] - l) - __fdividef(ei * ei, q);
        if (fabsf(q) < tiny) q = tiny;
        dm[i * 32] = q;
      }
    }
  }
  __syncthreads();
  // twist: smallest |gamma_i| = |dp_i + dm_i - (d_i - lam)|, ties to the higher i
  const int hm = m / 2;
  if (has) {
    const int i0 = half ? hm : 0, i1 = half ? m : hm;
    float best = 3e38f;
    int r = i1 - 1;
    for (int i = i1 - 1; i >= i0; --i) {
      const float g = fabsf(dp[i * 32] + dm[i * 32] - (dd[i] - l));
      if (g < best) {
        best = g;
        r = i;
      }
    }
    best_g[half][v] = best;
    best_i[half][v] = r;
  }
  __syncthreads();
  const int r = best_g[1][v] <= best_g[0][v] ? best_i[1][v] : best_i[0][v];
  if (has) {
    float z = 1.f;
    if (half == 0) {
      Z[(size_t)r * m + k] = 1.f;
      for (int i = r - 1; i >= 0; --i) {
        z = -__fdividef(ee[i], dp[i * 32]) * z;
        if (fabsf(z) < 1e-30f) z = 0.f;
        Z[(size_t)i * m + k] = z;
      }
    } else {
      for (int i = r + 1; i < m; ++i) {
        z = -__fdividef(ee[i - 1], dm[i * 32]) * z;
        if (fabsf(z) < 1e-30f) z = 0.f;
        Z[(size_t)i * m + k] = z;
      }
    }
  }
  __syncthreads();
  // Rayleigh quotient and norm in compensated FP32, two chains per half
  const int i0 = half ? hm : 0, i1 = half ? m : hm;
  if (has) {
    df n0{0.f, 0.f}, n1{0.f, 0.f}, q0{0.f, 0.f}, q1{0.f, 0.f};
    float zp = i0 > 0 ? Z[(size_t)(i0 - 1) * m + k] : 0.f;
    for (int i = i0; i < i1; ++i) {
      const float zi = Z[(size_t)i * m + k];
      df t = df_mul(two_prod(dd[i], zi), df{zi, 0.f});
      if (i > 0) t = df_add(t, df_mul(two_prod(2.f * ee[i - 1], zp), df{zi, 0.f}));
      if (i & 1) {
        n1 = df_add(n1, two_prod(zi, zi));
        q1 = df_add(q1, t);
      } else {
        n0 = df_add(n0, two_prod(zi, zi));
        q0 = df_add(q0, t);
      }
      zp = zi;
    }
    part_n[half][v] = df_add(n0, n1);
    part_q[half][v] = df_add(q0, q1);
  }
  __syncthreads();
  if (has && half == 0) {
    const double nrm = df_to(df_add(part_n[0][v], part_n[1][v]));
    lam[k] = df_to(df_add(part_q[0][v], part_q[1][v])) / nrm;
    scale[v] = (float)(1.0 / sqrt(nrm));
  }
  __syncthreads();
  if (has) {
    const float sc = scale[v];
    for (int i = i0; i < i1; ++i) Z[(size_t)i * m + k] *= sc;
  }
}

// Back-transformation x_k = H_0 H_1 ... H_{m-3} z_k in blocks of 32
// reflectors (compact WY form, FP32): Q_B = H_j0 ... H_j0+31 = I - V T V^T
// with T upper triangular (T_aa = tau_a, T[0:a, a] = -tau_a T[0:a, 0:a]
// V^T v_a), applied from the last block to the first as
// Z <- Z - V (T (V^T Z)).
constexpr int kWY = 32;

// T_B for every block B (one CTA per block): the Gram V_B^T V_B, then the
// column recursion by one warp.  Vh row j = reflector j (zero up to j).
__global__ void __launch_bounds__(1024) wy_factor(const float* __restrict__ Vh,
                                                  const float* __restrict__ tau, int m,
                                                  float* __restrict__ Tw) {
  extern __shared__ float vsh[];  // [kWY][m + 1] (padded rows: no bank conflicts)
  __shared__ float G[kWY][kWY + 1];
  __shared__ float T[kWY][kWY + 1];
  const int B = blockIdx.x, j0 = B * kWY, ld = m + 1;
  const int cnt = min(kWY, m - 2 - j0);
  for (int t = threadIdx.x; t < kWY * m; t += blockDim.x) {
    const int a = t / m, i = t % m;
    if (a < cnt) cp_async4(vsh + a * ld + i, Vh + (size_t)(j0 + a) * m + i);
    else vsh[a * ld + i] = 0.f;
  }
  cp_async_wait_all();
  __syncthreads();
  {
    const int a = threadIdx.x >> 5, b = threadIdx.x & 31;
    float g = 0.f;
    for (int i = j0 + 1; i < m; ++i) g = fmaf(vsh[a * ld + i], vsh[b * ld + i], g);
    G[a][b] = g;
    T[a][b] = 0.f;
  }
  __syncthreads();
  if (threadIdx.x < 32) {
    const int i = threadIdx.x;
    for (int a = 0; a < cnt; ++a) {
      const float ta = tau[j0 + a];
      float t = 0.f;
      if (i < a)
        for (int k = i; k < a; ++k) t = fmaf(T[i][k], G[k][a], t);
      __syncwarp();
      if (i < a) T[i][a] = -ta * t;
      if (i == a) T[a][a] = ta;
      __syncwarp();
    }
  }
  __syncthreads();
  Tw[(size_t)B * kWY * kWY + threadIdx.x] = T[threadIdx.x >> 5][threadIdx.x & 31];
}

// X row k = Q z_k for kSolveCols eigenvectors per 256-thread block.
__global__ void __launch_bounds__(256) wy_apply(const float* __restrict__ Vh,
                                                const float* __restrict__ Tw, int m,
                                                const float* __restrict__ Z,
                                                float* __restrict__ X) {
  extern __shared__ float zc[];  // [kSolveCols][m], then the block's reflectors [kWY][m]
  float* vb = zc + (size_t)kSolveCols * m;
  __shared__ float W[kWY][kSolveCols];
  __shared__ float W2[kWY][kSolveCols];
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int k0 = blockIdx.x * kSolveCols;
  for (int t = tid; t < kSolveCols * m; t += 256) {
    const int c = t % kSolveCols, i = t / kSolveCols;
    zc[c * m + i] = Z[(size_t)i * m + k0 + c];
  }
  const int nblk = (m - 2 + kWY - 1) / kWY;
  for (int B = nblk - 1; B >= 0; --B) {
    const int j0 = B * kWY;
    const int cnt = min(kWY, m - 2 - j0);
    __syncthreads();
    for (int t = 4 * tid; t < cnt * m; t += 4 * 256) cp_async16(vb + t, Vh + (size_t)j0 * m + t);
    cp_async_wait_all();
    __syncthreads();
    // W = V^T Z: warp w takes reflectors a = w, w + 8, ...; lanes over rows
    for (int a = warp; a < kWY; a += 8) {
      float acc[kSolveCols] = {};
      if (a < cnt) {
        const float* v = vb + (size_t)a * m;
        for (int i = j0 + 1 + lane; i < m; i += 32) {
          const float vi = v[i];
#pragma unroll
          for (int c = 0; c < kSolveCols; ++c) acc[c] = fmaf(vi, zc[c * m + i], acc[c]);
        }
      }
#pragma unroll
      for (int c = 0; c < kSolveCols; ++c) {
        float x = acc[c];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
        if (lane == 0) W[a][c] = x;
      }
    }
    __syncthreads();
    // W2 = T W (T upper triangular)
    if (tid < kWY * kSolveCols) {
      const int a = tid & 31, c = tid >> 5;
      const float* tr = Tw + (size_t)B * kWY * kWY + a * kWY;
      float x = 0.f;
      for (int b = a; b < kWY; ++b) x = fmaf(tr[b], W[b][c], x);
      W2[a][c] = x;
    }
    __syncthreads();
    // Z -= V W2
    for (int i = j0 + 1 + tid; i < m; i += 256) {
      float acc[kSolveCols] = {};
      for (int a = 0; a < cnt; ++a) {
        const float vi = vb[(size_t)a * m + i];
#pragma unroll
        for (int c = 0; c < kSolveCols; ++c) acc[c] = fmaf(vi, W2[a][c], acc[c]);
      }
#pragma unroll
      for (int c = 0; c < kSolveCols; ++c) zc[c * m + i] -= acc[c];
    }
  }
  __syncthreads();
  for (int t = tid; t < kSolveCols * m; t += 256) {
    const int c = t / m, i = t % m;
    X[(size_t)(k0 + c) * m + i] = zc[c * m + i];
  }
}

// C1 = s1 A^T diag(w1) B and, with TWO, C2 = s2 A^T diag(w2) B, for A, B
// [m][m] FP32 row-major: C[i][j] = sum_k A[k][i] w_k B[k][j], w1_k = f_k (1
// without f), w2_k = f_k g_k.  The back-transformation X = Z^T Q^T and the
// objective adjoints G_S = E^T diag(c) E, G_M = -E^T diag(c lam) E have this
// form.  32 x 32 output tiles, 256 threads with 2 x 2 outputs each, FP32
// products and sums; k in chunks of 32 staged in shared memory, the next
// chunk loaded into registers while the current one is multiplied.  sym
// (A = B): only the tiles with bj <= bi, every entry computed once and
// mirrored, so the outputs are exactly symmetric.
constexpr int kGT = 32;
template <typename TOut, bool TWO>
__global__ void __launch_bounds__(256) gemm_tn(const float* __restrict__ A,
                                               const float* __restrict__ B,
                                               const double* __restrict__ f,
                                               const double* __restrict__ g, int m, int sym,
                                               TOut* __restrict__ C1, float s1,
                                               TOut* __restrict__ C2, float s2) {
  __shared__ __align__(16) float as[kGT][kGT];
  __shared__ __align__(16) float bs1[kGT][kGT];
  __shared__ __align__(16) float bs2[TWO ? kGT : 1][kGT];
  const int nt = m / kGT;
  int t = blockIdx.x, bi = 0, bj;
  if (sym) {
    while (t > bi) {
      t -= bi + 1;
      ++bi;
    }
    bj = t;
  } else {
    bi = t / nt;
    bj = t % nt;
  }
  const int i0 = bi * kGT, j0 = bj * kGT;
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  const int lc = tid & 31, lr = tid >> 5;  // staged elements: rows lr + 8 q, column lc
  float ra[4], rb1[4], rb2[4];
  auto fetch = [&](int k0) {
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int k = k0 + lr + 8 * q;
      ra[q] = A[(size_t)k * m + i0 + lc];
      const float bv = B[(size_t)k * m + j0 + lc];
      const double w = f ? f[k] : 1.0;
      rb1[q] = bv * (float)w;
      if constexpr (TWO) rb2[q] = bv * (float)(w * g[k]);
    }
  };
  float acc1[2][2] = {}, acc2[2][2] = {};
  fetch(0);
  for (int k0 = 0; k0 < m; k0 += kGT) {
    __syncthreads();  // every read of the previous chunk is done
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      as[lr + 8 * q][lc] = ra[q];
      bs1[lr + 8 * q][lc] = rb1[q];
      if constexpr (TWO) bs2[lr + 8 * q][lc] = rb2[q];
    }
    __syncthreads();
    if (k0 + kGT < m) fetch(k0 + kGT);
#pragma unroll 8
    for (int kk = 0; kk < kGT; ++kk) {
      const float2 a = *reinterpret_cast<const float2*>(&as[kk][2 * ty]);
      const float2 b = *reinterpret_cast<const float2*>(&bs1[kk][2 * tx]);
      acc1[0][0] = fmaf(a.x, b.x, acc1[0][0]);
      acc1[0][1] = fmaf(a.x, b.y, acc1[0][1]);
      acc1[1][0] = fmaf(a.y, b.x, acc1[1][0]);
      acc1[1][1] = fmaf(a.y, b.y, acc1[1][1]);
      if constexpr (TWO) {
        const float2 d = *reinterpret_cast<const float2*>(&bs2[kk][2 * tx]);
        acc2[0][0] = fmaf(a.x, d.x, acc2[0][0]);
        acc2[0][1] = fmaf(a.x, d.y, acc2[0][1]);
        acc2[1][0] = fmaf(a.y, d.x, acc2[1][0]);
        acc2[1][1] = fmaf(a.y, d.y, acc2[1][1]);
      }
    }
  }
#pragma unroll
  for (int r = 0; r < 2; ++r)
#pragma unroll
    for (int cc = 0; cc < 2; ++cc) {
      const int i = i0 + 2 * ty + r, j = j0 + 2 * tx + cc;
      if (sym && j > i) continue;  // diagonal tiles: the lower triangle, mirrored
      C1[(size_t)i * m + j] = (TOut)(s1 * acc1[r][cc]);
      if (sym && i != j) C1[(size_t)j * m + i] = (TOut)(s1 * acc1[r][cc]);
      if constexpr (TWO) {
        C2[(size_t)i * m + j] = (TOut)(s2 * acc2[r][cc]);
        if (sym && i != j) C2[(size_t)j * m + i] = (TOut)(s2 * acc2[r][cc]);
      }
    }
}

__global__ void fill_identity(float* __restrict__ I, int m) {
  const size_t n = (size_t)m * m;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x)
    I[i] = (i / m == i % m) ? 1.f : 0.f;
}

__global__ void f32_to_f64(const float* __restrict__ a, double* __restrict__ b, size_t n,
                           double scale) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x)
    b[i] = scale * (double)a[i];
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
  size_t Mw, Lw, linv_pp, Dinv, LT, Y, C, Vh, tau, Tw, d, e, Z, X, E, Es, G, total;
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
  w.Lw = take(mm * 8);  // Cholesky factor (lower tiles)
  w.linv_pp = take((size_t)(m / kCB) * kCB * kCB * 8);
  w.Dinv = take((size_t)2 * (m / kCB) * kCB * kCB * sizeof(df));  // DL, DU
  w.LT = take(mm * 8 * 2);   // L and L^T as float pairs
  w.Y = take(mm * 8);    // L^-1 S (FP64)
  w.C = take(mm * 4);
  w.Vh = take(mm * 4);
  w.tau = take((size_t)m * 4);
  w.Tw = take((size_t)((m - 2 + kWY - 1) / kWY) * kWY * kWY * 4);
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
  df* Mw = (df*)(ws + w.Mw);  // working copy of M, float pairs
  df* Lw = (df*)(ws + w.Lw);  // Cholesky factor (lower tiles), float pairs
  df* linv_pp = (df*)(ws + w.linv_pp);
  df* Ld = (df*)(ws + w.LT);
  df* LTd = Ld + (size_t)m * m;
  double* Y = (double*)(ws + w.Y);
  float* C = (float*)(ws + w.C);
  float* Vh = (float*)(ws + w.Vh);
  float* tau = (float*)(ws + w.tau);
  float* Tw = (float*)(ws + w.Tw);
  double* d = (double*)(ws + w.d);
  double* e = (double*)(ws + w.e);
  float* Z = (float*)(ws + w.Z);
  float* X = (float*)(ws + w.X);
  float* E = (float*)(ws + w.E);
  float* Es = (float*)(ws + w.Es);
  float* G = (float*)(ws + w.G);
  const size_t mm = (size_t)m * m;
  const int nb = m / kCB;

  {
    int dev = 0, sms = 0;
    int st0;
    if ((st0 = device_sms(&dev, &sms))) return st0;
    static bool solve_configured[kMaxDevices] = {};
    if (!solve_configured[dev]) {
      NEB_CUDA_CHECK(cudaFuncSetAttribute(df_solve, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int)solve_smem(kMaxM)));
      solve_configured[dev] = true;
    }
  }
  NEB_CUDA_CHECK(cudaMemsetAsync(info, 0, sizeof(int), s));
  {
    KernelScope ks("spec_cholesky_df", s, (double)m * m * m / 3.0, 16.0 * mm, nb + 1);
    to_df<<<(int)std::min<size_t>((mm + 255) / 256, 1024), 256, 0, s>>>(M, Mw, mm);
    NEB_LAUNCH_CHECK();
    chol_first<<<1, 1024, 0, s>>>(Mw, m, Lw, linv_pp, info);
    NEB_LAUNCH_CHECK();
    // the panel launches start while their predecessor finishes (programmatic
    // dependent launch): the launch latency leaves the panel-to-panel chain
    for (int p = 0; p + 1 < nb; ++p) {
      NEB_CUDA_CHECK(launch_pdl(chol_step, dim3((nb - p - 1) * (nb - p) / 2), dim3(1024), 0, s,
                                Mw, m, p, Lw, linv_pp, info));
      NEB_LAUNCH_CHECK();
    }
  }
  int st;
  df* DL = (df*)(ws + w.Dinv);
  df* DU = DL + (size_t)nb * kCB * kCB;
  {
    // C = L^-1 S L^-T as two solves: Y = L^-1 S, C = L^-1 Y^T (S symmetric)
    KernelScope ks("spec_reduce_df", s, 2.0 * m * mm, 32.0 * mm, 4);
    {
      KernelScope k1("split_factor", s, 0, 0, 0);
      split_factor<<<dim3(m / 32, m / 32), dim3(32, 8), 0, s>>>(Lw, m, Ld, LTd);
      NEB_LAUNCH_CHECK();
      split_dinv<<<nb, 1024, 0, s>>>(linv_pp, DL, DU);
      NEB_LAUNCH_CHECK();
    }
    {
      KernelScope k2("df_solve", s, 0, 0, 0);
      df_solve<<<m / kRLCols, kMaxM, solve_smem(m), s>>>(LTd, DL, m, 0, S, 0, 0, Y, 0, 0);
      NEB_LAUNCH_CHECK();
    }
    KernelScope k3("df_solve", s, 0, 0, 0);
    df_solve<<<m / kRLCols, kMaxM, solve_smem(m), s>>>(LTd, DL, m, 0, Y, 0, 1, C, 1, 0);
    NEB_LAUNCH_CHECK();
  }
  {
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = kTriCluster;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(kTriCluster);
    cfg.blockDim = dim3(kTriThreads);
    // columns 0 .. k0-1 by the cluster, the trailing R x R block by CTA 0
    const int R = std::min(m, kTriTail), k0 = m - R;
    auto tri_smem = [](int m_, int r_) {
      return ((size_t)4 * m_ + 2 * kTriCluster * kTriMsg + 2 * kTriMsg + 2 * kTriWarps +
              (size_t)r_ * r_) *
             sizeof(float);
    };
    cfg.dynamicSmemBytes = tri_smem(m, R);
    cfg.stream = s;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    int dev = 0, sms = 0;
    if ((st = device_sms(&dev, &sms))) return st;
    static int clusters[kMaxDevices];  // co-resident 16-CTA clusters (non-portable size)
    static bool probed[kMaxDevices] = {};
    if (!probed[dev]) {
      NEB_CUDA_CHECK(cudaFuncSetAttribute(tridiag_cluster,
                                          cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
      NEB_CUDA_CHECK(cudaFuncSetAttribute(tridiag_cluster,
                                          cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int)tri_smem(kMaxM, kTriTail)));
      cudaLaunchConfig_t probe = cfg;  // the largest block
      probe.dynamicSmemBytes = tri_smem(kMaxM, kTriTail);
      NEB_CUDA_CHECK(cudaOccupancyMaxActiveClusters(&clusters[dev], tridiag_cluster, &probe));
      probed[dev] = true;
    }
    NEB_REQUIRE(clusters[dev] >= 1,
                "neb_spectral_mixed: the GPU cannot co-schedule a %d-CTA thread-block cluster",
                kTriCluster);
    KernelScope ks("spec_tridiag_cluster_fp32", s, 4.0 / 3.0 * m * mm, 8.0 * mm);
    NEB_CUDA_CHECK(cudaLaunchKernelEx(&cfg, tridiag_cluster, (const float*)C, m, k0, d, e, Vh,
                                      tau, info));
    NEB_LAUNCH_CHECK();
  }
  // The back-transformation depends only on the reflectors: on a side stream
  // (one per host thread and device) wy_factor forms the compact-WY factors
  // and wy_apply applies Q to the identity (G = Q^T) while the tridiagonal
  // eigenproblem is solved on the main stream; X = Z^T Q^T is then one SGEMM.
  {
    int dev = 0, sms = 0;
    if ((st = device_sms(&dev, &sms))) return st;
    static thread_local cudaStream_t side[kMaxDevices] = {};
    static thread_local cudaEvent_t ev_fork[kMaxDevices] = {}, ev_join[kMaxDevices] = {};
    if (!side[dev]) {
      NEB_CUDA_CHECK(cudaStreamCreateWithFlags(&side[dev], cudaStreamNonBlocking));
      NEB_CUDA_CHECK(cudaEventCreateWithFlags(&ev_fork[dev], cudaEventDisableTiming));
      NEB_CUDA_CHECK(cudaEventCreateWithFlags(&ev_join[dev], cudaEventDisableTiming));
    }
    static bool wy_configured[kMaxDevices] = {};
    if (!wy_configured[dev]) {
      NEB_CUDA_CHECK(cudaFuncSetAttribute(wy_factor, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          kWY * (kMaxM + 1) * (int)sizeof(float)));
      NEB_CUDA_CHECK(cudaFuncSetAttribute(wy_apply, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (kSolveCols + kWY) * kMaxM * (int)sizeof(float)));
      NEB_CUDA_CHECK(cudaFuncSetAttribute(tri_eigvecs, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (2 * kMaxM * 32 + 2 * kMaxM) * (int)sizeof(float)));
      wy_configured[dev] = true;
    }
    NEB_CUDA_CHECK(cudaEventRecord(ev_fork[dev], s));
    NEB_CUDA_CHECK(cudaStreamWaitEvent(side[dev], ev_fork[dev], 0));
    SideStreamJoin join{s, side[dev], ev_join[dev], true};
    {
      KernelScope ks("wy_factor", side[dev], 2.0 * m * mm, 4.0 * mm, 1);
      const int nblk = (m - 2 + kWY - 1) / kWY;
      wy_factor<<<nblk, 1024, (size_t)kWY * (m + 1) * sizeof(float), side[dev]>>>(Vh, tau, m, Tw);
      NEB_LAUNCH_CHECK();
    }
    {
      KernelScope ks("wy_form_q", side[dev], 2.0 * m * mm, 4.0 * mm * (m / kSolveCols), 2);
      const int blocks = (int)std::min<size_t>((mm + 255) / 256, 2048);
      fill_identity<<<blocks, 256, 0, side[dev]>>>(Es, m);
      NEB_LAUNCH_CHECK();
      wy_apply<<<m / kSolveCols, 256, (size_t)(kSolveCols + kWY) * m * sizeof(float), side[dev]>>>(
          Vh, Tw, m, Es, G);
      NEB_LAUNCH_CHECK();
    }
    NEB_CUDA_CHECK(cudaEventRecord(ev_join[dev], side[dev]));
    {
      KernelScope ks("spec_tridiag_eig", s, 0, 16.0 * m, 2);
      {
        KernelScope k1("tri_eigvals", s, 0, 0, 0);
        tri_eigvals<<<(m * 32 + 255) / 256, 256, (size_t)2 * m * 4, s>>>(d, e, m, lam);
        NEB_LAUNCH_CHECK();
      }
      tri_eigvecs<<<(m + 31) / 32, 64, ((size_t)2 * m * 32 + 2 * m) * sizeof(float), s>>>(
          d, e, m, lam, Z);
      NEB_LAUNCH_CHECK();
    }
    NEB_CUDA_CHECK(cudaStreamWaitEvent(s, ev_join[dev], 0));
    join.armed = false;
    KernelScope ks("spec_backtransform_fp32", s, 2.0 * m * mm, 12.0 * mm, 1);
    const int nt = m / kGT;
    gemm_tn<float, false><<<nt * nt, 256, 0, s>>>(Z, G, nullptr, nullptr, m, 0, X, 1.f,
                                                   (float*)nullptr, 0.f);
    NEB_LAUNCH_CHECK();
  }
  {
    KernelScope ks("spec_adjoints_fp32", s, 6.0 * m * mm, 24.0 * mm, 4);
    // rows of V: e_k = (L^-T x_k)^T, a backward solve with L^T on the columns of X^T
    {
      KernelScope k1("df_solve", s, 0, 0, 0);
      df_solve<<<m / kRLCols, kMaxM, solve_smem(m), s>>>(Ld, DU, m, 1, X, 1, 1, E, 1, 1);
      NEB_LAUNCH_CHECK();
    }
    int blocks = (int)std::min<size_t>((mm + 255) / 256, 2048);
    f32_to_f64<<<blocks, 256, 0, s>>>(E, V, mm, 1.0);
    NEB_LAUNCH_CHECK();
    // G_S = E^T diag(c) E ; G_M = -E^T diag(c lam) E, one pass over E
    const int nt = m / kGT;
    gemm_tn<double, true><<<nt * (nt + 1) / 2, 256, 0, s>>>(E, E, c, lam, m, 1, G_S, 1.f, G_M,
                                                             -1.f);
    NEB_LAUNCH_CHECK();
    mixed_loss<<<1, 256, 0, s>>>(c, lam, m, loss, info);
    NEB_LAUNCH_CHECK();
  }
  return NEB_OK;
}
