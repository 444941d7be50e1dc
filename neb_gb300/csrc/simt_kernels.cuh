// SIMT kernels of the jet MLP (FP32 and FP64 forms, no tensor cores), plus the
// elementwise and reduction kernels every precision shares.
//
//  * jet_gemm_fwd   : Z = X W^T (+ b on the value channel) with the tanh-jet
//                     chain rule fused into the epilogue.
//  * jet_gemm_bwd   : Xbar = s_p (A B_sel(c)), then the tanh-jet transpose of
//                     the previous layer in the epilogue.  B_sel(c) picks the
//                     matrix by jet channel (the hidden-Gram adjoint uses
//                     G_M for the gradient channels and G_S for the Laplacian).
//  * rowsum_gemm    : Out[m][n] = sum over rows r in a point chunk and a
//                     channel subset of w_p P[r][m] Q[r][n]; one FP64 partial
//                     per chunk (Grams and weight gradients).
//  * reduce_chunks  : deterministic FP64 sum of the per-chunk partials.
#pragma once
#include "neb_common.cuh"

namespace neb {
namespace simt {

constexpr int kThreads = 256;
constexpr int kBN = 128;
constexpr int kBK = 8;

// Points per thread: a thread owns whole points (all C channel rows) so the
// jet epilogue needs no data exchange.  C = 4 -> 2 points (8 rows), C = 10 ->
// 1 point (10 rows), C = 1 (plain row-major matrices) -> 8 rows.
template <int C> struct Tile {
  static constexpr int P = (C == 4) ? 2 : (C == 1 ? 8 : 1);
  static constexpr int TM = C * P;
  static constexpr int BM = TM * 16;
};

template <typename T>
__device__ __forceinline__ void store4(T* dst, const T* v, int nvalid) {
  if (nvalid == 4 && ((reinterpret_cast<uintptr_t>(dst) & 15) == 0)) {
    if constexpr (sizeof(T) == 4) {
      *reinterpret_cast<float4*>(dst) = make_float4(v[0], v[1], v[2], v[3]);
    } else {
      reinterpret_cast<double2*>(dst)[0] = make_double2(v[0], v[1]);
      reinterpret_cast<double2*>(dst)[1] = make_double2(v[2], v[3]);
    }
  } else {
    for (int i = 0; i < nvalid; ++i) dst[i] = v[i];
  }
}

template <typename T>
__device__ __forceinline__ void load4(const T* src, T* v, int nvalid) {
  if (nvalid == 4 && ((reinterpret_cast<uintptr_t>(src) & 15) == 0)) {
    if constexpr (sizeof(T) == 4) {
      float4 q = *reinterpret_cast<const float4*>(src);
      v[0] = q.x; v[1] = q.y; v[2] = q.z; v[3] = q.w;
    } else {
      double2 a = reinterpret_cast<const double2*>(src)[0];
      double2 b = reinterpret_cast<const double2*>(src)[1];
      v[0] = a.x; v[1] = a.y; v[2] = b.x; v[3] = b.y;
    }
  } else {
    for (int i = 0; i < 4; ++i) v[i] = i < nvalid ? src[i] : T(0);
  }
}

// ---------------------------------------------------------------------------
// Z = X W^T (+ b), Y = tanh-jet(Z).   X: [n*C][K], W: [N][K], Z, Y: [n*C][N].
// Y may be null (output layer: Z only).  grid = (ceil(N/128), ceil(n*C/BM)).
// ---------------------------------------------------------------------------
template <typename T, int C, bool ACT>
__global__ void __launch_bounds__(kThreads)
jet_gemm_fwd(const T* __restrict__ X, const T* __restrict__ W, const T* __restrict__ bias,
             T* __restrict__ Z, T* __restrict__ Y, int64_t n_points, int K, int N, int ldo) {
  using Tl = Tile<C>;
  constexpr int TM = Tl::TM, BM = Tl::BM, P = Tl::P;
  constexpr int NA = BM * kBK / kThreads;   // A elements per thread per tile
  constexpr int NB = kBN * kBK / kThreads;  // B elements per thread per tile
  __shared__ __align__(16) T As[kBK][BM + 4];
  __shared__ __align__(16) T Bs[kBK][kBN + 4];
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  const int64_t rows = n_points * C;
  const int64_t row0 = (int64_t)blockIdx.y * BM;
  const int col0 = blockIdx.x * kBN;

  T acc[TM][8];
#pragma unroll
  for (int i = 0; i < TM; ++i)
#pragma unroll
    for (int j = 0; j < 8; ++j) acc[i][j] = T(0);

  T ra[NA], rb[NB];
  auto fetch = [&](int k0) {
#pragma unroll
    for (int i = 0; i < NA; ++i) {
      int e = tid + i * kThreads, m = e / kBK, k = e % kBK;
      int64_t r = row0 + m;
      int kk = k0 + k;
      ra[i] = (r < rows && kk < K) ? X[r * K + kk] : T(0);
    }
#pragma unroll
    for (int i = 0; i < NB; ++i) {
      int e = tid + i * kThreads, n = e / kBK, k = e % kBK;
      int c = col0 + n, kk = k0 + k;
      rb[i] = (c < N && kk < K) ? W[(int64_t)c * K + kk] : T(0);
    }
  };
  fetch(0);
  for (int k0 = 0; k0 < K; k0 += kBK) {
#pragma unroll
    for (int i = 0; i < NA; ++i) {
      int e = tid + i * kThreads;
      As[e % kBK][e / kBK] = ra[i];
    }
#pragma unroll
    for (int i = 0; i < NB; ++i) {
      int e = tid + i * kThreads;
      Bs[e % kBK][e / kBK] = rb[i];
    }
    __syncthreads();
    if (k0 + kBK < K) fetch(k0 + kBK);
#pragma unroll
    for (int k = 0; k < kBK; ++k) {
      T a[TM], b[8];
#pragma unroll
      for (int i = 0; i < TM; ++i) a[i] = As[k][ty * TM + i];
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        b[j] = Bs[k][tx * 4 + j];
        b[4 + j] = Bs[k][64 + tx * 4 + j];
      }
#pragma unroll
      for (int i = 0; i < TM; ++i)
#pragma unroll
        for (int j = 0; j < 8; ++j) acc[i][j] = fma(a[i], b[j], acc[i][j]);
    }
    __syncthreads();
  }

  // epilogue: bias on the value channel, store Z, tanh jet, store Y
#pragma unroll
  for (int q = 0; q < P; ++q) {
    int64_t p = (row0 + ty * TM) / C + q;
    if (p >= n_points) continue;
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      int cb = col0 + h * 64 + tx * 4;
      int nvalid = N - cb;
      if (nvalid <= 0) continue;
      if (nvalid > 4) nvalid = 4;
      T z[4][C];
#pragma unroll
      for (int j = 0; j < 4; ++j) {
#pragma unroll
        for (int c = 0; c < C; ++c) z[j][c] = acc[q * C + c][h * 4 + j];
        if (bias != nullptr && j < nvalid) z[j][0] += bias[cb + j];
      }
#pragma unroll
      for (int c = 0; c < C; ++c) {
        T v[4] = {z[0][c], z[1][c], z[2][c], z[3][c]};
        store4(Z + (p * C + c) * (int64_t)ldo + cb, v, nvalid);
      }
      if constexpr (ACT) {
#pragma unroll
        for (int j = 0; j < 4; ++j) jet_act_forward<C>(z[j]);
#pragma unroll
        for (int c = 0; c < C; ++c) {
          T v[4] = {z[0][c], z[1][c], z[2][c], z[3][c]};
          store4(Y + (p * C + c) * (int64_t)ldo + cb, v, nvalid);
        }
      }
    }
  }
}

// ---------------------------------------------------------------------------
// Out[r][n] = s_p * sum_k A[r][k] B_{map(c)}[k][n], then (if Zprev) the
// tanh-jet transpose with the pre-activation Zprev.  A: [n*C][K];
// B0, B1: [K][N] row-major; map (compile time): MAP == 0 -> every channel uses
// B0; MAP == 1 -> 2D Gram adjoint: value channel zero, gradient channels B0
// (G_M), Laplacian B1 (G_S); MAP == 2 -> 3D field adjoint on the field layout
// of fields.cuh: channels 1-3 (velocity) B0 (G_M), 4-6 (vorticity) B1 (G_S),
// the rest zero.  rowscale: per-point s_p (nullable) times scale.
// ---------------------------------------------------------------------------
template <int MAP, int C> __device__ __forceinline__ int chan_b(int c) {
  if constexpr (MAP == 0) return 0;
  else if constexpr (MAP == 1) return c == 0 ? -1 : (c == 3 ? 1 : 0);
  else return (c >= 1 && c <= 3) ? 0 : ((c >= 4 && c <= 6) ? 1 : -1);
}

template <typename T, int C, int MAP, bool ACT>
__global__ void __launch_bounds__(kThreads)
jet_gemm_bwd(const T* __restrict__ A, const T* __restrict__ B0, const T* __restrict__ B1,
             const T* __restrict__ rowscale, T scale, const T* __restrict__ Zprev,
             T* __restrict__ Out, int64_t n_points, int K, int N) {
  using Tl = Tile<C>;
  constexpr int TM = Tl::TM, BM = Tl::BM, P = Tl::P;
  constexpr int NBM = (MAP == 0) ? 1 : 2;
  constexpr int NA = BM * kBK / kThreads;
  constexpr int NB = kBN * kBK / kThreads;
  __shared__ __align__(16) T As[kBK][BM + 4];
  __shared__ __align__(16) T Bs[NBM][kBK][kBN + 4];
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  const int64_t rows = n_points * C;
  const int64_t row0 = (int64_t)blockIdx.y * BM;
  const int col0 = blockIdx.x * kBN;

  T acc[TM][8];
#pragma unroll
  for (int i = 0; i < TM; ++i)
#pragma unroll
    for (int j = 0; j < 8; ++j) acc[i][j] = T(0);

  T ra[NA], rb[NBM][NB];
  auto fetch = [&](int k0) {
#pragma unroll
    for (int i = 0; i < NA; ++i) {
      int e = tid + i * kThreads, m = e / kBK, k = e % kBK;
      int64_t r = row0 + m;
      int kk = k0 + k;
      ra[i] = (r < rows && kk < K) ? A[r * K + kk] : T(0);
    }
#pragma unroll
    for (int s = 0; s < NBM; ++s) {
      const T* Bp = s == 0 ? B0 : B1;
#pragma unroll
      for (int i = 0; i < NB; ++i) {
        int e = tid + i * kThreads, k = e / kBN, n = e % kBN;
        int c = col0 + n, kk = k0 + k;
        rb[s][i] = (c < N && kk < K) ? Bp[(int64_t)kk * N + c] : T(0);
      }
    }
  };
  fetch(0);
  for (int k0 = 0; k0 < K; k0 += kBK) {
#pragma unroll
    for (int i = 0; i < NA; ++i) {
      int e = tid + i * kThreads;
      As[e % kBK][e / kBK] = ra[i];
    }
#pragma unroll
    for (int s = 0; s < NBM; ++s)
#pragma unroll
      for (int i = 0; i < NB; ++i) {
        int e = tid + i * kThreads;
        Bs[s][e / kBN][e % kBN] = rb[s][i];
      }
    __syncthreads();
    if (k0 + kBK < K) fetch(k0 + kBK);
#pragma unroll
    for (int k = 0; k < kBK; ++k) {
      T a[TM], b[NBM][8];
#pragma unroll
      for (int i = 0; i < TM; ++i) a[i] = As[k][ty * TM + i];
#pragma unroll
      for (int s = 0; s < NBM; ++s)
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          b[s][j] = Bs[s][k][tx * 4 + j];
          b[s][4 + j] = Bs[s][k][64 + tx * 4 + j];
        }
#pragma unroll
      for (int i = 0; i < TM; ++i) {
        const int sel = chan_b<MAP, C>(i % C);
        if (sel < 0) continue;
#pragma unroll
        for (int j = 0; j < 8; ++j) acc[i][j] = fma(a[i], b[sel][j], acc[i][j]);
      }
    }
    __syncthreads();
  }

#pragma unroll
  for (int q = 0; q < P; ++q) {
    int64_t p = (row0 + ty * TM) / C + q;
    if (p >= n_points) continue;
    T s = scale * (rowscale != nullptr ? rowscale[p] : T(1));
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      int cb = col0 + h * 64 + tx * 4;
      int nvalid = N - cb;
      if (nvalid <= 0) continue;
      if (nvalid > 4) nvalid = 4;
      T xb[4][C];
#pragma unroll
      for (int j = 0; j < 4; ++j)
#pragma unroll
        for (int c = 0; c < C; ++c) xb[j][c] = s * acc[q * C + c][h * 4 + j];
      if constexpr (ACT) {
        T zp[C][4];
#pragma unroll
        for (int c = 0; c < C; ++c) load4(Zprev + (p * C + c) * (int64_t)N + cb, zp[c], nvalid);
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          T z[C];
#pragma unroll
          for (int c = 0; c < C; ++c) z[c] = zp[c][j];
          jet_act_backward<C>(z, xb[j]);
        }
      }
#pragma unroll
      for (int c = 0; c < C; ++c) {
        T v[4] = {xb[0][c], xb[1][c], xb[2][c], xb[3][c]};
        store4(Out + (p * C + c) * (int64_t)N + cb, v, nvalid);
      }
    }
  }
}

// ---------------------------------------------------------------------------
// Per-chunk partial of Out[m][n] = sum_{p in chunk} sum_{c in chans} w_p
// P[p*C + c][m] Q[p*C + c][n].  P: [n*C][ldp], Q: [n*C][ldq].  Tiles (mt, nt)
// with blockIdx.x enumerating the tile pairs (upper triangle only when sym);
// blockIdx.y is the point chunk.  part: [chunks][M][N] double.
//
// COMP (FP32 only): every product is split exactly into p + e (e = fma(a, b,
// -p)) and the running sum is kept as an unevaluated pair hi + lo updated
// by TwoSum, so a chunk sum is accurate to about eps_32^2 relative to its
// terms instead of eps_32 times the number of terms.  The Grams of a nearly
// dependent basis need this: a plain FP32 sum perturbs every entry by ~1e-7
// of the largest, independently, which moves the small eigenvalues of the
// mass matrix by that much.
// ---------------------------------------------------------------------------
struct ChanSet {
  int n;
  int c[10];
};

template <typename T, bool COMP> struct RowAcc;
template <typename T> struct RowAcc<T, false> {
  T s;
  __device__ __forceinline__ void zero() { s = T(0); }
  __device__ __forceinline__ void add(T a, T b) { s = fma(a, b, s); }
  __device__ __forceinline__ double value() const { return (double)s; }
};
template <> struct RowAcc<float, true> {
  float hi, lo;
  __device__ __forceinline__ void zero() { hi = lo = 0.f; }
  __device__ __forceinline__ void add(float a, float b) {
    const float p = a * b;
    const float e = fmaf(a, b, -p);  // a * b = p + e exactly
    const float s = hi + p;
    const float bb = s - hi;
    lo += ((hi - (s - bb)) + (p - bb)) + e;
    hi = s;
  }
  __device__ __forceinline__ double value() const { return (double)hi + (double)lo; }
};

template <typename T, int C, bool COMP = false>
__global__ void __launch_bounds__(kThreads)
rowsum_gemm(const T* __restrict__ Pm, int ldp, const T* __restrict__ Qm, int ldq,
            const T* __restrict__ wts, ChanSet chans, int64_t n_points, int64_t chunk_pts,
            int M, int N, int sym, double* __restrict__ part) {
  static_assert(!COMP || sizeof(T) == 4, "compensated sums are the FP32 form");
  constexpr int BMr = 128;
  __shared__ __align__(16) T Ps[kBK][BMr + 4];
  __shared__ __align__(16) T Qs[kBK][kBN + 4];
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  // tile pair
  const int mtiles = (M + BMr - 1) / BMr, ntiles = (N + kBN - 1) / kBN;
  int mt, nt;
  if (sym) {
    int idx = blockIdx.x, r = 0;
    while (idx >= ntiles - r) { idx -= ntiles - r; ++r; }
    mt = r; nt = r + idx;
  } else {
    mt = blockIdx.x / ntiles; nt = blockIdx.x % ntiles;
  }
  (void)mtiles;
  const int m0 = mt * BMr, n0 = nt * kBN;
  const int64_t p_begin = (int64_t)blockIdx.y * chunk_pts;
  int64_t p_end = p_begin + chunk_pts;
  if (p_end > n_points) p_end = n_points;
  const int64_t klen = (p_end - p_begin) * chans.n;

  RowAcc<T, COMP> acc[8][8];
#pragma unroll
  for (int i = 0; i < 8; ++i)
#pragma unroll
    for (int j = 0; j < 8; ++j) acc[i][j].zero();

  // each thread loads 4 P and 4 Q elements per k tile: k = e / 128, m = e % 128
  T rp[4], rq[4];
  auto fetch = [&](int64_t k0) {
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      int e = tid + i * kThreads, k = e / BMr, m = e % BMr;
      int64_t kk = k0 + k;
      T pv = T(0), qv = T(0);
      if (kk < klen) {
        int64_t p = p_begin + kk / chans.n;
        int c = chans.c[kk % chans.n];
        int64_t r = p * C + c;
        T w = wts != nullptr ? wts[p] : T(1);
        if (m0 + m < M) pv = w * Pm[r * ldp + m0 + m];
        if (n0 + m < N) qv = Qm[r * ldq + n0 + m];
      }
      rp[i] = pv;
      rq[i] = qv;
    }
  };
  fetch(0);
  for (int64_t k0 = 0; k0 < klen; k0 += kBK) {
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      int e = tid + i * kThreads;
      Ps[e / BMr][e % BMr] = rp[i];
      Qs[e / BMr][e % BMr] = rq[i];
    }
    __syncthreads();
    if (k0 + kBK < klen) fetch(k0 + kBK);
#pragma unroll
    for (int k = 0; k < kBK; ++k) {
      T a[8], b[8];
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        a[j] = Ps[k][ty * 4 + j];
        a[4 + j] = Ps[k][64 + ty * 4 + j];
        b[j] = Qs[k][tx * 4 + j];
        b[4 + j] = Qs[k][64 + tx * 4 + j];
      }
#pragma unroll
      for (int i = 0; i < 8; ++i)
#pragma unroll
        for (int j = 0; j < 8; ++j) acc[i][j].add(a[i], b[j]);
    }
    __syncthreads();
  }
  double* out = part + (int64_t)blockIdx.y * M * N;
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    int m = m0 + (i < 4 ? ty * 4 + i : 64 + ty * 4 + i - 4);
    if (m >= M) continue;
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      int n = n0 + (j < 4 ? tx * 4 + j : 64 + tx * 4 + j - 4);
      if (n < N) out[(int64_t)m * N + n] = acc[i][j].value();
    }
  }
}

// out[i] (+)= scale * sum_chunks part[chunk][i]  (sym: lower triangle
// mirrored from the upper one).  OutT = double or float.
template <typename OutT>
__global__ void reduce_chunks(const double* __restrict__ part, int chunks, int M, int N, int sym,
                              double scale, int accumulate, OutT* __restrict__ out) {
  int64_t total = (int64_t)M * N;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total;
       i += (int64_t)gridDim.x * blockDim.x) {
    int m = (int)(i / N), n = (int)(i % N);
    int64_t src = (sym && m > n) ? ((int64_t)n * N + m) : i;
    double s = 0.0;
    for (int c = 0; c < chunks; ++c) s += part[(int64_t)c * total + src];
    if (accumulate) out[i] = (OutT)((double)out[i] + scale * s);
    else out[i] = (OutT)(scale * s);
  }
}

// Per-chunk column sums of the value-channel rows: partb[chunk][o].
template <typename T, int C>
__global__ void bias_partial(const T* __restrict__ Zb, int64_t n_points, int64_t chunk_pts,
                             int N, double* __restrict__ partb) {
  int o = blockIdx.x * blockDim.x + threadIdx.x;
  if (o >= N) return;
  int64_t p0 = (int64_t)blockIdx.y * chunk_pts;
  int64_t p1 = p0 + chunk_pts < n_points ? p0 + chunk_pts : n_points;
  double s = 0.0;
  for (int64_t p = p0; p < p1; ++p) s += (double)Zb[(p * C) * (int64_t)N + o];
  partb[(int64_t)blockIdx.y * N + o] = s;
}

}  // namespace simt
}  // namespace neb
