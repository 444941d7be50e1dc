// Periodic evaluation of a trained per-mode basis: third-order feature jets,
// the stream-function fields of every mode on a grid, the normalised Ritz
// pencil, and the matrix-free Galerkin ETDRK4 rollout in the Ritz basis
// (experiments/periodic/paper_rollout.py:31-103 rollout, :171-203 the
// normalisation and Ritz stage; experiments/2d/_backend/periodic_core/
// vortex_merger/canonical_gauge/scripts/evaluate_large_comparison.py:16-39
// the Jet3 field channels).
//
// The basis stays as the network produced it (raw fields, FP32 for FP32
// networks); the column normalisation and the Ritz rotation are one K x K
// FP64 matrix R = D^-1 T applied to coefficient vectors, so the rotated
// basis g R is never formed.  One right-hand side
//   rhs(a) = R^T [U^T (w omega .* v) - V^T (w omega .* u)],  (u, v, omega) = (U, V, W) R a
// reads the basis twice (the three fields per point, then U and V again);
// for FP32 fields every dot product is compensated (exact products by FMA,
// TwoSum accumulation, the FP64 factor carried as two floats), so the sums
// keep FP64-class accuracy at FP32 throughput.
#include <algorithm>
#include "neb_common.cuh"

namespace neb {
namespace {

int grid_for(int64_t n, int block = 256) {
  return (int)std::min<int64_t>(std::max<int64_t>(ceil_div(n, block), 1), 8192);
}
size_t a256(size_t x) { return (x + 255) & ~size_t(255); }
constexpr int kChunkPts = 256;   // most points per block of the transposed pass
constexpr int kMinChunkPts = 32; // fewest (small grids: more blocks in flight)
constexpr int kColsPerBlock = 256;

// ------------------------------------------------------------ feature jets
// Periodic Fourier features of points already shifted to the box origin:
// for axis (x, y), harmonic h = 1..F: sin, cos of k s with k = 2 pi h / L
// (the reference's pi h (s_n + 1), s_n normalised to [-1, 1]), with their
// derivatives along the axis: first, second (xx or yy) and third (xxx or
// yyy).  out [n][C][4F], C = 3, 6, 10 for order 1, 2, 3.
template <typename T>
__global__ void periodic_features_kernel(int order, int F, double kx, double ky,
                                         const double* __restrict__ pts, int64_t n,
                                         T* __restrict__ out) {
  const int C = order == 1 ? 3 : (order == 2 ? 6 : 10), W = 4 * F;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n * W;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t p = e / W;
    const int f = (int)(e % W);
    const int axis = f / (2 * F), h = (f % (2 * F)) / 2 + 1;
    const bool is_cos = f & 1;
    const double k = (axis == 0 ? kx : ky) * h;
    double sn, cs;
    sincos(k * pts[2 * p + axis], &sn, &cs);
    const double v = is_cos ? cs : sn, d1 = is_cos ? -k * sn : k * cs;
    T* o = out + p * C * W + f;
    for (int c = 0; c < C; ++c) o[(int64_t)c * W] = T(0);
    o[0] = (T)v;
    o[(int64_t)(1 + axis) * W] = (T)d1;
    if (order >= 2) o[(int64_t)(axis == 0 ? 3 : 5) * W] = (T)(-k * k * v);
    if (order == 3) o[(int64_t)(axis == 0 ? 6 : 9) * W] = (T)(-k * k * d1);
  }
}

// ------------------------------------------------------------ basis fields
// Output jets [B][n][C][1] of modes [start, start + B) -> columns of
// UV [n][2][K] (u = psi_y, v = -psi_x), Om [n][K] (omega = -lap psi) and,
// for third-order jets when diag is set, diag [n][3][K] (psi, -lap u, -lap v).
template <typename T>
__global__ void stream_fields_kernel(const T* __restrict__ out, int C, int start, int B,
                                     int64_t n, int K, T* __restrict__ UV, T* __restrict__ Om,
                                     T* __restrict__ diag) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n * B;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t p = e / B;
    const int b = (int)(e % B), k = start + b;
    const T* o = out + ((int64_t)b * n + p) * C;
    UV[(p * 2) * K + k] = o[2];
    UV[(p * 2 + 1) * K + k] = -o[1];
    Om[p * K + k] = -(o[3] + o[5]);
    if (diag && C == 10) {
      diag[(p * 3) * K + k] = o[0];
      diag[(p * 3 + 1) * K + k] = -(o[7] + o[9]);
      diag[(p * 3 + 2) * K + k] = o[6] + o[8];
    }
  }
}

// ------------------------------------------------------------ Ritz pencil
__global__ void pencil_norms(int K, const double* __restrict__ M, double* __restrict__ norm) {
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < K; k += gridDim.x * blockDim.x)
    norm[k] = sqrt(M[(int64_t)k * K + k]);
}
__global__ void pencil_scale(int K, double* __restrict__ M, double* __restrict__ S,
                             const double* __restrict__ norm) {
  const int64_t total = (int64_t)K * K;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
       e += (int64_t)gridDim.x * blockDim.x) {
    const double d = norm[e / K] * norm[e % K];
    M[e] /= d;
    S[e] /= d;
  }
}
// R[k][i] = V[i][k] / norm[k] (rows of V are M-orthonormal eigenvectors),
// and its transpose Rt[i][k] = R[k][i] right after it, so that both R x and
// R^T y are row-wise (coalesced) products.
__global__ void ritz_transform(int K, const double* __restrict__ V,
                               const double* __restrict__ norm, double* __restrict__ R) {
  const int64_t total = (int64_t)K * K;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int k = (int)(e / K), i = (int)(e % K);
    R[e] = V[(int64_t)i * K + k] / norm[k];
    R[total + e] = V[e] / norm[i];  // Rt[k][i] = R[i][k] = V[k][i] / norm[i]
  }
}

// ------------------------------------------------------------ ETDRK4 weights
struct Cplx {
  double re, im;
};
__device__ __forceinline__ Cplx cadd(Cplx a, Cplx b) { return {a.re + b.re, a.im + b.im}; }
__device__ __forceinline__ Cplx cmul(Cplx a, Cplx b) {
  return {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re};
}
__device__ __forceinline__ Cplx cscale(Cplx a, double s) { return {a.re * s, a.im * s}; }
__device__ __forceinline__ Cplx cdiv(Cplx a, Cplx b) {
  const double d = b.re * b.re + b.im * b.im;
  return {(a.re * b.re + a.im * b.im) / d, (a.im * b.re - a.re * b.im) / d};
}
__device__ __forceinline__ Cplx cexp(Cplx a) {
  double s, c;
  sincos(a.im, &s, &c);
  const double r = exp(a.re);
  return {r * c, r * s};
}

// coef [6][K] = (e, e2, q, f1, f2, f3) of the ETDRK4 scheme with linear
// part L = -nu lam and step h: e = exp(hL), e2 = exp(hL / 2) and the phi
// functions by the mean over 32 points r_j = exp(i pi (j - 1/2) / 32) of the
// contour hL + r_j (paper_rollout.py:56-64).
__global__ void etdrk4_coef_kernel(int K, const double* __restrict__ lam, double nu, double h,
                                   double* __restrict__ coef) {
  const double kPi = 3.14159265358979323846;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < K; k += gridDim.x * blockDim.x) {
    const double hl = h * (-nu * lam[k]);
    double q = 0, f1 = 0, f2 = 0, f3 = 0;
    for (int j = 1; j <= 32; ++j) {
      double s, c;
      sincos(kPi * (j - 0.5) / 32.0, &s, &c);
      const Cplx z{hl + c, s};
      const Cplx ez = cexp(z), ez2 = cexp(cscale(z, 0.5));
      const Cplx z2 = cmul(z, z), z3 = cmul(z2, z);
      q += cdiv(cadd(ez2, {-1.0, 0.0}), z).re;
      // (-4 - z + e^z (4 - 3z + z^2)) / z^3
      const Cplx a1 = cadd(cadd({-4.0, 0.0}, cscale(z, -1.0)),
                           cmul(ez, cadd(cadd({4.0, 0.0}, cscale(z, -3.0)), z2)));
      f1 += cdiv(a1, z3).re;
      // (2 + z + e^z (-2 + z)) / z^3
      const Cplx a2 = cadd(cadd({2.0, 0.0}, z), cmul(ez, cadd({-2.0, 0.0}, z)));
      f2 += cdiv(a2, z3).re;
      // (-4 - 3z - z^2 + e^z (4 - z)) / z^3
      const Cplx a3 = cadd(cadd(cadd({-4.0, 0.0}, cscale(z, -3.0)), cscale(z2, -1.0)),
                           cmul(ez, cadd({4.0, 0.0}, cscale(z, -1.0))));
      f3 += cdiv(a3, z3).re;
    }
    coef[k] = exp(hl);
    coef[K + k] = exp(0.5 * hl);
    coef[2 * K + k] = h * q / 32.0;
    coef[3 * K + k] = h * f1 / 32.0;
    coef[4 * K + k] = h * f2 / 32.0;
    coef[5 * K + k] = h * f3 / 32.0;
  }
}

// ------------------------------------------------------------ compensated sums
// (s, c): an unevaluated sum s + c.  add_prod adds a * (bh + bl) with the
// product a bh formed exactly (FMA) and the TwoSum error kept.
struct Acc2 {
  float s, c;
};
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = a + b;
  const float bb = s - a;
  e = (a - (s - bb)) + (b - bb);
}
__device__ __forceinline__ void add_prod(Acc2& x, float a, float bh, float bl) {
  const float p = a * bh;
  const float pe = fmaf(a, bh, -p);
  float s, e;
  two_sum(x.s, p, s, e);
  x.s = s;
  x.c += e + pe + a * bl;
}
__device__ __forceinline__ Acc2 warp_sum(Acc2 x) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const float s2 = __shfl_xor_sync(0xffffffffu, x.s, o);
    const float c2 = __shfl_xor_sync(0xffffffffu, x.c, o);
    float s, e;
    two_sum(x.s, s2, s, e);
    x.s = s;
    x.c += c2 + e;
  }
  return x;
}
__device__ __forceinline__ void split2(double x, float& h, float& l) {
  h = (float)x;
  l = (float)(x - (double)h);
}

// b = R x (row-major R [K][K]), one warp per row; b64 and its float split.
__global__ void gemv_rows(int K, const double* __restrict__ R, const double* __restrict__ x,
                          double* __restrict__ b64, float* __restrict__ bh,
                          float* __restrict__ bl) {
  const int lane = threadIdx.x & 31;
  for (int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < K;
       i += (gridDim.x * blockDim.x) >> 5) {
    double s = 0.0;
    for (int k = lane; k < K; k += 32) s += R[(int64_t)i * K + k] * x[k];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) {
      b64[i] = s;
      split2(s, bh[i], bl[i]);
    }
  }
}

// Pass 1, one warp per point: (u, v, omega) = (UV[p][0], UV[p][1], Om[p]) . b.
// mode 0: q1 = w omega v, q2 = w omega u (the nonlinear products of the
// right-hand side); mode 1: the fields themselves into f [3][n].
template <typename T>
__global__ void rollout_pass1(int64_t n, int K, const T* __restrict__ UV,
                              const T* __restrict__ Om, const double* __restrict__ b64,
                              const float* __restrict__ bh, const float* __restrict__ bl,
                              double weight, int mode, double* __restrict__ q,
                              float* __restrict__ qh, float* __restrict__ ql) {
  const int lane = threadIdx.x & 31;
  for (int64_t p = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5; p < n;
       p += ((int64_t)gridDim.x * blockDim.x) >> 5) {
    double u, v, w;
    const T* ru = UV + (p * 2) * K;
    const T* rv = ru + K;
    const T* rw = Om + p * K;
    if constexpr (sizeof(T) == 4) {
      Acc2 au{0.f, 0.f}, av{0.f, 0.f}, aw{0.f, 0.f};
      int k0 = 0;
      const bool vec = (K & 3) == 0 &&
                       ((reinterpret_cast<uintptr_t>(UV) | reinterpret_cast<uintptr_t>(Om)) & 15) == 0;
      if (vec) {  // 16-byte loads: every row starts on a 16-byte boundary
        const float4* u4 = reinterpret_cast<const float4*>(ru);
        const float4* v4 = reinterpret_cast<const float4*>(rv);
        const float4* w4 = reinterpret_cast<const float4*>(rw);
        const float4* h4 = reinterpret_cast<const float4*>(bh);
        const float4* l4 = reinterpret_cast<const float4*>(bl);
        for (int j = lane; j < (K >> 2); j += 32) {
          const float4 uu = u4[j], vv = v4[j], ww = w4[j], hh = h4[j], ll = l4[j];
          add_prod(au, uu.x, hh.x, ll.x); add_prod(au, uu.y, hh.y, ll.y);
          add_prod(au, uu.z, hh.z, ll.z); add_prod(au, uu.w, hh.w, ll.w);
          add_prod(av, vv.x, hh.x, ll.x); add_prod(av, vv.y, hh.y, ll.y);
          add_prod(av, vv.z, hh.z, ll.z); add_prod(av, vv.w, hh.w, ll.w);
          add_prod(aw, ww.x, hh.x, ll.x); add_prod(aw, ww.y, hh.y, ll.y);
          add_prod(aw, ww.z, hh.z, ll.z); add_prod(aw, ww.w, hh.w, ll.w);
        }
        k0 = K;
      }
      for (int k = k0 + lane; k < K; k += 32) {
        const float h = bh[k], l = bl[k];
        add_prod(au, ru[k], h, l);
        add_prod(av, rv[k], h, l);
        add_prod(aw, rw[k], h, l);
      }
      au = warp_sum(au);
      av = warp_sum(av);
      aw = warp_sum(aw);
      u = (double)au.s + (double)au.c;
      v = (double)av.s + (double)av.c;
      w = (double)aw.s + (double)aw.c;
    } else {
      double su = 0, sv = 0, sw = 0;
      for (int k = lane; k < K; k += 32) {
        const double b = b64[k];
        su += ru[k] * b;
        sv += rv[k] * b;
        sw += rw[k] * b;
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        su += __shfl_xor_sync(0xffffffffu, su, o);
        sv += __shfl_xor_sync(0xffffffffu, sv, o);
        sw += __shfl_xor_sync(0xffffffffu, sw, o);
      }
      u = su;
      v = sv;
      w = sw;
    }
    if (lane == 0) {
      if (mode == 0) {
        const double q1 = weight * w * v, q2 = weight * w * u;
        q[p] = q1;
        q[n + p] = q2;
        if (qh) {
          split2(q1, qh[p], ql[p]);
          split2(q2, qh[n + p], ql[n + p]);
        }
      } else {
        q[p] = u;
        q[n + p] = v;
        q[2 * n + p] = w;
      }
    }
  }
}

// Pass 2: partial[chunk][k] = sum over the chunk's points of
// UV[p][0][k] q1[p] - UV[p][1][k] q2[p].  grid (K / 256, chunks).
template <typename T>
__global__ void __launch_bounds__(kColsPerBlock)
rollout_pass2(int64_t n, int K, int chunk, const T* __restrict__ UV, const double* __restrict__ q,
              const float* __restrict__ qh, const float* __restrict__ ql,
              double* __restrict__ partial) {
  __shared__ double s64[2][kChunkPts];
  __shared__ float sh[2][kChunkPts], sl[2][kChunkPts];
  const int k = blockIdx.x * kColsPerBlock + threadIdx.x;
  const int64_t p0 = (int64_t)blockIdx.y * chunk;
  const int np = (int)std::min<int64_t>(chunk, n - p0);
  for (int i = threadIdx.x; i < np; i += blockDim.x) {
    if constexpr (sizeof(T) == 4) {
      sh[0][i] = qh[p0 + i];
      sl[0][i] = ql[p0 + i];
      sh[1][i] = -qh[n + p0 + i];
      sl[1][i] = -ql[n + p0 + i];
    } else {
      s64[0][i] = q[p0 + i];
      s64[1][i] = -q[n + p0 + i];
    }
  }
  __syncthreads();
  if (k >= K) return;
  const T* base = UV + (p0 * 2) * K + k;
  double out;
  if constexpr (sizeof(T) == 4) {
    Acc2 a{0.f, 0.f};
    for (int i = 0; i < np; ++i) {
      add_prod(a, base[(int64_t)(2 * i) * K], sh[0][i], sl[0][i]);
      add_prod(a, base[(int64_t)(2 * i + 1) * K], sh[1][i], sl[1][i]);
    }
    out = (double)a.s + (double)a.c;
  } else {
    double a = 0.0;
    for (int i = 0; i < np; ++i)
      a += base[(int64_t)(2 * i) * K] * s64[0][i] + base[(int64_t)(2 * i + 1) * K] * s64[1][i];
    out = a;
  }
  partial[(int64_t)blockIdx.y * K + k] = out;
}

// y[k] = sum over chunks of partial[chunk][k] (fixed order): a block per 32
// columns, warp w summing chunks w, w + 16, ..., then the 16 warp sums.
constexpr int kReduceWarps = 16;
__global__ void __launch_bounds__(32 * kReduceWarps)
reduce_partials(int K, int chunks, const double* __restrict__ partial, double* __restrict__ y) {
  __shared__ double red[kReduceWarps][32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, k = blockIdx.x * 32 + lane;
  double s = 0.0;
  if (k < K)
    for (int c = w; c < chunks; c += kReduceWarps) s += partial[(int64_t)c * K + k];
  red[w][lane] = s;
  __syncthreads();
  if (w == 0 && k < K) {
    double t = 0.0;
    for (int j = 0; j < kReduceWarps; ++j) t += red[j][lane];
    y[k] = t;
  }
}

// r = R^T y, then the ETDRK4 stage (paper_rollout.py:65-72) at index k:
//   kind 0: nv = r, a = e2 c + q nv       kind 1: na = r, b = e2 c + q na
//   kind 2: nb = r, z = e2 a + q (2 nb - nv)
//   kind 3: c = e c + f1 nv + 2 f2 (na + nb) + f3 r
//   kind -1: out = r (a plain right-hand side / projection)
struct Stage {
  double *c, *a, *b, *z, *nv, *na, *nb, *out;
};
__global__ void rollout_finish(int kind, int K, const double* __restrict__ R,
                               const double* __restrict__ y, const double* __restrict__ coef,
                               Stage st) {
  const double* Rt = R + (int64_t)K * K;
  const int lane = threadIdx.x & 31;
  for (int k = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; k < K;
       k += (gridDim.x * blockDim.x) >> 5) {
    double r = 0.0;
    for (int i = lane; i < K; i += 32) r += Rt[(int64_t)k * K + i] * y[i];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) r += __shfl_xor_sync(0xffffffffu, r, o);
    if (lane != 0) continue;
    if (kind < 0) {
      st.out[k] = r;
      continue;
    }
    const double e = coef[k], e2 = coef[K + k], qq = coef[2 * K + k];
    if (kind == 0) {
      st.nv[k] = r;
      st.a[k] = e2 * st.c[k] + qq * r;
    } else if (kind == 1) {
      st.na[k] = r;
      st.b[k] = e2 * st.c[k] + qq * r;
    } else if (kind == 2) {
      st.nb[k] = r;
      st.z[k] = e2 * st.a[k] + qq * (2.0 * r - st.nv[k]);
    } else {
      const double f1 = coef[3 * K + k], f2 = coef[4 * K + k], f3 = coef[5 * K + k];
      st.c[k] = e * st.c[k] + f1 * st.nv[k] + 2.0 * f2 * (st.na[k] + st.nb[k]) + f3 * r;
    }
  }
}

// ------------------------------------------------------------ workspace
struct RollWs {
  size_t b64, bh, bl, q, qh, ql, partial, y, vec, vec_stride, total;
  int chunks, chunk;
};
// Points per block of the transposed pass: kChunkPts, fewer when the grid
// would otherwise hold less than about four blocks per SM.
int pass2_chunk(int64_t n, int K) {
  int dev = 0, sms = 148;
  if (cudaGetDevice(&dev) == cudaSuccess)
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int64_t cols = ceil_div(K, kColsPerBlock);
  int64_t c = n * cols / (4 * (int64_t)std::max(sms, 1));
  c = std::max<int64_t>(kMinChunkPts, std::min<int64_t>(kChunkPts, c));
  return (int)(c / kMinChunkPts * kMinChunkPts);
}
RollWs roll_ws(int64_t n, int K) {
  RollWs w{};
  w.chunk = pass2_chunk(n, K);
  w.chunks = (int)ceil_div(n, w.chunk);
  size_t o = 0;
  w.b64 = o; o += a256((size_t)K * 8);
  w.bh = o; o += a256((size_t)K * 4);
  w.bl = o; o += a256((size_t)K * 4);
  w.q = o; o += a256((size_t)3 * n * 8);
  w.qh = o; o += a256((size_t)2 * n * 4);
  w.ql = o; o += a256((size_t)2 * n * 4);
  w.partial = o; o += a256((size_t)ceil_div(n, kMinChunkPts) * K * 8);
  w.y = o; o += a256((size_t)K * 8);
  w.vec = o;  // the stage vectors a, b, z, nv, na, nb
  w.vec_stride = a256((size_t)K * 8);
  o += 6 * w.vec_stride;
  w.total = o;
  return w;
}

template <typename T>
int launch_pass1(int64_t n, int K, const void* UV, const void* Om, char* ws, const RollWs& w,
                 double weight, int mode, double* qout, cudaStream_t s) {
  KernelScope ks("rollout_pass1", s, 6.0 * n * K, 3.0 * n * K * sizeof(T));
  const int blocks = (int)std::min<int64_t>(ceil_div(n * 32, 256), 65535);
  rollout_pass1<T><<<blocks, 256, 0, s>>>(
      n, K, (const T*)UV, (const T*)Om, (const double*)(ws + w.b64), (const float*)(ws + w.bh),
      (const float*)(ws + w.bl), weight, mode, qout,
      sizeof(T) == 4 && mode == 0 ? (float*)(ws + w.qh) : nullptr, (float*)(ws + w.ql));
  NEB_LAUNCH_CHECK();
  return NEB_OK;
}

template <typename T>
int launch_pass2(int64_t n, int K, const void* UV, char* ws, const RollWs& w, cudaStream_t s) {
  {
    KernelScope ks("rollout_pass2", s, 4.0 * n * K, 2.0 * n * K * sizeof(T));
    dim3 grid((unsigned)ceil_div(K, kColsPerBlock), (unsigned)w.chunks);
    rollout_pass2<T><<<grid, kColsPerBlock, 0, s>>>(n, K, w.chunk, (const T*)UV,
                                                     (const double*)(ws + w.q),
                                                     (const float*)(ws + w.qh),
                                                     (const float*)(ws + w.ql),
                                                     (double*)(ws + w.partial));
    NEB_LAUNCH_CHECK();
  }
  KernelScope ks("reduce_partials", s, 0, 8.0 * w.chunks * K);
  reduce_partials<<<(unsigned)ceil_div(K, 32), 32 * kReduceWarps, 0, s>>>(
      K, w.chunks, (const double*)(ws + w.partial), (double*)(ws + w.y));
  NEB_LAUNCH_CHECK();
  return NEB_OK;
}

int launch_gemv(int K, const double* R, const double* x, char* ws, const RollWs& w,
                cudaStream_t s) {
  KernelScope ks("ritz_gemv", s, 2.0 * K * K, 8.0 * K * K);
  gemv_rows<<<grid_for((int64_t)K * 32), 256, 0, s>>>(K, R, x, (double*)(ws + w.b64),
                                                     (float*)(ws + w.bh), (float*)(ws + w.bl));
  NEB_LAUNCH_CHECK();
  return NEB_OK;
}

int launch_finish(int kind, int K, const double* R, const double* coef, const Stage& st,
                  char* ws, const RollWs& w, cudaStream_t s) {
  KernelScope ks("ritz_finish", s, 2.0 * K * K, 8.0 * K * K);
  rollout_finish<<<grid_for((int64_t)K * 32), 256, 0, s>>>(kind, K, R, (const double*)(ws + w.y),
                                                          coef, st);
  NEB_LAUNCH_CHECK();
  return NEB_OK;
}

// One right-hand side of the coefficient vector x, finished by stage kind.
template <typename T>
int rhs_stage(int64_t n, int K, const void* UV, const void* Om, const double* R, double weight,
              const double* x, int kind, const double* coef, const Stage& st, char* ws,
              const RollWs& w, cudaStream_t s) {
  if (int e = launch_gemv(K, R, x, ws, w, s)) return e;
  if (int e = launch_pass1<T>(n, K, UV, Om, ws, w, weight, 0, (double*)(ws + w.q), s)) return e;
  if (int e = launch_pass2<T>(n, K, UV, ws, w, s)) return e;
  return launch_finish(kind, K, R, coef, st, ws, w, s);
}

Stage stage_of(char* ws, const RollWs& w, double* c, double* out) {
  auto at = [&](int i) { return (double*)(ws + w.vec + (size_t)i * w.vec_stride); };
  return Stage{c, at(0), at(1), at(2), at(3), at(4), at(5), out};
}

// q[i] = +-weight q[i] (+ for i < half), and its float split.
__global__ void scale_split(int64_t total, int64_t half, double weight, double* __restrict__ q,
                            float* __restrict__ qh, float* __restrict__ ql) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total;
       i += (int64_t)gridDim.x * blockDim.x) {
    const double v = (i < half ? weight : -weight) * q[i];
    q[i] = v;
    split2(v, qh[i], ql[i]);
  }
}

int check_common(int precision, int64_t n, int K, const void* UV, size_t ws_bytes,
                 const void* ws) {
  NEB_REQUIRE(precision == NEB_PREC_FP32 || precision == NEB_PREC_FP64,
              "rollout: FP32 or FP64 fields");
  NEB_REQUIRE(n > 0 && n <= ((int64_t)1 << 31) && K > 0 && K <= (1 << 16) && UV,
              "rollout: bad sizes or fields");
  if (!ws || ws_bytes < roll_ws(n, K).total) {
    set_error("rollout: workspace %zu < %zu bytes", ws_bytes, roll_ws(n, K).total);
    return NEB_ERR_WORKSPACE;
  }
  return NEB_OK;
}

}  // namespace
}  // namespace neb

using namespace neb;

extern "C" int neb_periodic_features(int precision, int order, int n_freq, double length_x,
                                     double length_y, const double* points, int64_t n_points,
                                     void* features, neb_stream_t stream) {
  NEB_REQUIRE(precision == NEB_PREC_FP32 || precision == NEB_PREC_FP64,
              "neb_periodic_features: FP32 or FP64");
  NEB_REQUIRE(order >= 1 && order <= 3 && n_freq > 0 && length_x > 0 && length_y > 0 &&
                  points && features && n_points > 0,
              "neb_periodic_features: bad arguments");
  cudaStream_t s = (cudaStream_t)stream;
  const double kPi = 3.14159265358979323846;
  const int64_t total = n_points * 4 * n_freq;
  KernelScope ks("periodic_features", s, 0, (double)total * (order == 1 ? 3 : order == 2 ? 6 : 10) *
                                                 (precision == NEB_PREC_FP64 ? 8 : 4));
  if (precision == NEB_PREC_FP64)
    periodic_features_kernel<double><<<grid_for(total), 256, 0, s>>>(
        order, n_freq, 2 * kPi / length_x, 2 * kPi / length_y, points, n_points,
        (double*)features);
  else
    periodic_features_kernel<float><<<grid_for(total), 256, 0, s>>>(
        order, n_freq, 2 * kPi / length_x, 2 * kPi / length_y, points, n_points,
        (float*)features);
  NEB_LAUNCH_CHECK();
  return NEB_OK;
}

extern "C" int neb_stream_fields(int precision, int order, const void* out, int start, int stop,
                                 int64_t n_points, int n_modes, void* UV, void* Om, void* diag,
                                 neb_stream_t stream) {
  NEB_REQUIRE(precision == NEB_PREC_FP32 || precision == NEB_PREC_FP64,
              "neb_stream_fields: FP32 or FP64");
  NEB_REQUIRE(order == 2 || order == 3, "neb_stream_fields: jets of order 2 or 3");
  NEB_REQUIRE(out && UV && Om && 0 <= start && start < stop && stop <= n_modes && n_points > 0,
              "neb_stream_fields: bad arguments");
  NEB_REQUIRE(!diag || order == 3, "neb_stream_fields: diagnostic channels need order 3");
  cudaStream_t s = (cudaStream_t)stream;
  const int C = order == 2 ? 6 : 10, B = stop - start;
  const int64_t total = n_points * B;
  const size_t es = precision == NEB_PREC_FP64 ? 8 : 4;
  KernelScope ks("stream_fields", s, 0, (double)total * (C + (diag ? 6 : 3)) * es);
  if (precision == NEB_PREC_FP64)
    stream_fields_kernel<double><<<grid_for(total), 256, 0, s>>>(
        (const double*)out, C, start, B, n_points, n_modes, (double*)UV, (double*)Om,
        (double*)diag);
  else
    stream_fields_kernel<float><<<grid_for(total), 256, 0, s>>>(
        (const float*)out, C, start, B, n_points, n_modes, (float*)UV, (float*)Om, (float*)diag);
  NEB_LAUNCH_CHECK();
  return NEB_OK;
}

extern "C" int neb_normalize_pencil(int K, double* M, double* S, double* norm,
                                    neb_stream_t stream) {
  NEB_REQUIRE(K > 0 && M && S && norm, "neb_normalize_pencil: bad arguments");
  cudaStream_t s = (cudaStream_t)stream;
  KernelScope ks("normalize_pencil", s, 0, 32.0 * K * K);
  pencil_norms<<<grid_for(K), 256, 0, s>>>(K, M, norm);
  NEB_LAUNCH_CHECK();
  pencil_scale<<<grid_for((int64_t)K * K), 256, 0, s>>>(K, M, S, norm);
  NEB_LAUNCH_CHECK();
  return NEB_OK;
}

extern "C" int neb_ritz_transform(int K, const double* V, const double* norm, double* R,
                                  neb_stream_t stream) {
  NEB_REQUIRE(K > 0 && V && norm && R, "neb_ritz_transform: bad arguments");
  cudaStream_t s = (cudaStream_t)stream;
  KernelScope ks("ritz_transform", s, 0, 16.0 * K * K);
  ritz_transform<<<grid_for((int64_t)K * K), 256, 0, s>>>(K, V, norm, R);
  NEB_LAUNCH_CHECK();
  return NEB_OK;
}

extern "C" int neb_etdrk4_coefficients(int K, const double* lam, double nu, double h,
                                       double* coef, neb_stream_t stream) {
  NEB_REQUIRE(K > 0 && lam && coef && h > 0, "neb_etdrk4_coefficients: bad arguments");
  cudaStream_t s = (cudaStream_t)stream;
  KernelScope ks("etdrk4_coefficients", s, 0, 56.0 * K);
  etdrk4_coef_kernel<<<grid_for(K, 128), 128, 0, s>>>(K, lam, nu, h, coef);
  NEB_LAUNCH_CHECK();
  return NEB_OK;
}

extern "C" size_t neb_rollout_workspace_bytes(int64_t n_points, int K) {
  if (n_points <= 0 || K <= 0) return 0;
  return roll_ws(n_points, K).total;
}

extern "C" int neb_rollout_rhs(int precision, int64_t n_points, int K, const void* UV,
                               const void* Om, const double* R, double weight, const double* x,
                               double* out, void* workspace, size_t workspace_bytes,
                               neb_stream_t stream) {
  if (int e = check_common(precision, n_points, K, UV, workspace_bytes, workspace)) return e;
  NEB_REQUIRE(Om && R && x && out, "neb_rollout_rhs: bad arguments");
  cudaStream_t s = (cudaStream_t)stream;
  const RollWs w = roll_ws(n_points, K);
  char* ws = (char*)workspace;
  const Stage st = stage_of(ws, w, nullptr, out);
  return precision == NEB_PREC_FP64
             ? rhs_stage<double>(n_points, K, UV, Om, R, weight, x, -1, nullptr, st, ws, w, s)
             : rhs_stage<float>(n_points, K, UV, Om, R, weight, x, -1, nullptr, st, ws, w, s);
}

extern "C" int neb_etdrk4_step(int precision, int64_t n_points, int K, const void* UV,
                               const void* Om, const double* R, double weight,
                               const double* coef, double* c, void* workspace,
                               size_t workspace_bytes, neb_stream_t stream) {
  if (int e = check_common(precision, n_points, K, UV, workspace_bytes, workspace)) return e;
  NEB_REQUIRE(Om && R && coef && c, "neb_etdrk4_step: bad arguments");
  cudaStream_t s = (cudaStream_t)stream;
  const RollWs w = roll_ws(n_points, K);
  char* ws = (char*)workspace;
  const Stage st = stage_of(ws, w, c, nullptr);
  const double* inputs[4] = {c, st.a, st.b, st.z};
  for (int kind = 0; kind < 4; ++kind) {
    const int e = precision == NEB_PREC_FP64
                      ? rhs_stage<double>(n_points, K, UV, Om, R, weight, inputs[kind], kind,
                                          coef, st, ws, w, s)
                      : rhs_stage<float>(n_points, K, UV, Om, R, weight, inputs[kind], kind,
                                         coef, st, ws, w, s);
    if (e) return e;
  }
  return NEB_OK;
}

extern "C" int neb_rollout_project(int precision, int64_t n_points, int K, const void* UV,
                                   const double* R, const double* u0, const double* v0,
                                   double weight, double* c, void* workspace,
                                   size_t workspace_bytes, neb_stream_t stream) {
  if (int e = check_common(precision, n_points, K, UV, workspace_bytes, workspace)) return e;
  NEB_REQUIRE(R && u0 && v0 && c, "neb_rollout_project: bad arguments");
  cudaStream_t s = (cudaStream_t)stream;
  const RollWs w = roll_ws(n_points, K);
  char* ws = (char*)workspace;
  // q1 = w u0, q2 = -w v0, so that pass 2 forms w (U^T u0 + V^T v0)
  double* q = (double*)(ws + w.q);
  float* qh = (float*)(ws + w.qh);
  float* ql = (float*)(ws + w.ql);
  NEB_CUDA_CHECK(cudaMemcpyAsync(q, u0, n_points * 8, cudaMemcpyDeviceToDevice, s));
  NEB_CUDA_CHECK(cudaMemcpyAsync(q + n_points, v0, n_points * 8, cudaMemcpyDeviceToDevice, s));
  {
    KernelScope ks("scale_split", s, 0, 32.0 * n_points);
    scale_split<<<grid_for(2 * n_points), 256, 0, s>>>(2 * n_points, n_points, weight, q, qh, ql);
    NEB_LAUNCH_CHECK();
  }
  const int e = precision == NEB_PREC_FP64 ? launch_pass2<double>(n_points, K, UV, ws, w, s)
                                           : launch_pass2<float>(n_points, K, UV, ws, w, s);
  if (e) return e;
  return launch_finish(-1, K, R, nullptr, stage_of(ws, w, nullptr, c), ws, w, s);
}

extern "C" int neb_rollout_fields(int precision, int64_t n_points, int K, const void* UV,
                                  const void* Om, const double* R, const double* c,
                                  double* fields, void* workspace, size_t workspace_bytes,
                                  neb_stream_t stream) {
  if (int e = check_common(precision, n_points, K, UV, workspace_bytes, workspace)) return e;
  NEB_REQUIRE(Om && R && c && fields, "neb_rollout_fields: bad arguments");
  cudaStream_t s = (cudaStream_t)stream;
  const RollWs w = roll_ws(n_points, K);
  char* ws = (char*)workspace;
  if (int e = launch_gemv(K, R, c, ws, w, s)) return e;
  return precision == NEB_PREC_FP64
             ? launch_pass1<double>(n_points, K, UV, Om, ws, w, 1.0, 1, fields, s)
             : launch_pass1<float>(n_points, K, UV, Om, ws, w, 1.0, 1, fields, s);
}
