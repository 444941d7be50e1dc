// Mode-stacked SIREN networks: the reference's own per-mode architecture.
//
// K independent networks, one per mode, with weights stacked [K][out][in]
// and biases [K][out]: hidden layers y = sin(omega (W x + b)) (omega_first on
// the first layer, omega_hidden after), a linear output layer, and the output
// jet multiplied by an envelope jet (the reference's Model of
// experiments/metaball/_backend/flow/cases/metaball/native_cupy_core.py:
// 111-154 for first-order jets, velocity_trace_jet2.py:26-82 for second-order
// jets).  Jets carry C = 1 + dim (+ dim (dim + 1) / 2 Hessian entries for
// order 2) channels per point, laid out [n][C][width] per mode, modes
// outermost: [B][n][C][width] for a block of B modes.  The input features
// [n][C][F] are shared by every mode.
//
// Kernels (SIMT, FP32 or FP64 as the parameters):
//   mode_gemm<EPI>   per-mode jet GEMM over all channels, tiles of 8 points
//                    x 128 (FP32) or 64 (FP64) columns, the reduction staged
//                    through double-buffered shared memory by cp.async;
//   mode_output_narrow the output layer when it has at most 4 columns;
//                    epilogues: output layer (+ bias, x envelope), hidden
//                    layer (+ bias, x omega, sine jet, pre-activation kept),
//                    reverse data (sine-jet transpose of the layer below).
//   mode_wgrad       gW[k] = sum over points and channels of Abar (x) X,
//                    split over point ranges, FP64-free deterministic sum.
//   mode_bias        gb[k] = sum over points of the value-channel adjoint.
//   mode_envelope_reverse, velocity_fields, velocity_lift (3D curl fields of
//   a vector potential), and the per-mode Adam transaction.
#include <algorithm>
#include <math_constants.h>
#include "neb_common.cuh"
#include "elementwise.cuh"
#include "tc_blas.cuh"

namespace neb {
namespace {

// Compact Hessian pairs: 2D (xx, xy, yy), 3D (xx, xy, xz, yy, yz, zz).
__host__ __device__ constexpr int pair_i(int dim, int k) {
  return dim == 2 ? (k < 2 ? 0 : 1) : (k < 3 ? 0 : (k < 5 ? 1 : 2));
}
__host__ __device__ constexpr int pair_j(int dim, int k) {
  return dim == 2 ? (k == 0 ? 0 : 1) : (k < 3 ? k : (k == 3 ? 1 : 2));
}

// Channels of a jet: value, gradient, compact Hessian (order >= 2) and, for
// order 3 in 2D, the third derivatives (xxx, xxy, xyy, yyy) -- the layout of
// the reference's Jet3 (hardcoded_backend.py:58-152).  Order 3 is a forward
// (evaluation) jet only.
template <int DIM, int ORD> struct Jet {
  static_assert(ORD >= 1 && ORD <= 3 && (ORD < 3 || DIM == 2), "jet order");
  static constexpr int NH = ORD >= 2 ? DIM * (DIM + 1) / 2 : 0;
  static constexpr int NT = ORD == 3 ? 4 : 0;
  static constexpr int C = 1 + DIM + NH + NT;
};

// y = sin z, grad y = cos z grad z, H y = cos z H z - sin z grad z grad z^T,
// and in 2D to third order
//   y_ijk = cos z z_ijk - sin z (z_ij z_k + z_ik z_j + z_jk z_i) - cos z z_i z_j z_k.
template <int DIM, int ORD, typename T>
__device__ __forceinline__ void sine_jet(const T* z, T* y) {
  T s, c;
  if constexpr (sizeof(T) == 8) sincos(z[0], &s, &c); else sincosf(z[0], &s, &c);
  y[0] = s;
#pragma unroll
  for (int a = 0; a < DIM; ++a) y[1 + a] = c * z[1 + a];
#pragma unroll
  for (int k = 0; k < Jet<DIM, ORD>::NH; ++k)
    y[1 + DIM + k] = c * z[1 + DIM + k] - s * z[1 + pair_i(DIM, k)] * z[1 + pair_j(DIM, k)];
  if constexpr (ORD == 3) {
    const T zx = z[1], zy = z[2], hxx = z[3], hxy = z[4], hyy = z[5];
    y[6] = c * z[6] - s * (3 * hxx * zx) - c * zx * zx * zx;
    y[7] = c * z[7] - s * (hxx * zy + 2 * hxy * zx) - c * zx * zx * zy;
    y[8] = c * z[8] - s * (hyy * zx + 2 * hxy * zy) - c * zx * zy * zy;
    y[9] = c * z[9] - s * (3 * hyy * zy) - c * zy * zy * zy;
  }
}

// Transpose of sine_jet at z: adjoint a of y -> adjoint b of z.
template <int DIM, int ORD, typename T>
__device__ __forceinline__ void sine_jet_reverse(const T* z, const T* a, T* b) {
  T s, c;
  if constexpr (sizeof(T) == 8) sincos(z[0], &s, &c); else sincosf(z[0], &s, &c);
  T zb = c * a[0];
#pragma unroll
  for (int d = 0; d < DIM; ++d) {
    zb -= s * a[1 + d] * z[1 + d];
    b[1 + d] = c * a[1 + d];
  }
#pragma unroll
  for (int k = 0; k < Jet<DIM, ORD>::NH; ++k) {
    const int i = pair_i(DIM, k), j = pair_j(DIM, k), q = 1 + DIM + k;
    const T ah = a[q];
    zb += ah * (-s * z[q] - c * z[1 + i] * z[1 + j]);
    b[1 + i] -= s * ah * z[1 + j];
    b[1 + j] -= s * ah * z[1 + i];
    b[q] = c * ah;
  }
  b[0] = zb;
}

// Product of the envelope e with x (Leibniz rule on every channel).
template <int DIM, int ORD, typename T>
__device__ __forceinline__ void envelope_mul(const T* e, const T* x, T* y) {
  y[0] = e[0] * x[0];
#pragma unroll
  for (int a = 0; a < DIM; ++a) y[1 + a] = e[0] * x[1 + a] + e[1 + a] * x[0];
#pragma unroll
  for (int k = 0; k < Jet<DIM, ORD>::NH; ++k) {
    const int i = pair_i(DIM, k), j = pair_j(DIM, k), q = 1 + DIM + k;
    y[q] = e[0] * x[q] + e[q] * x[0] + e[1 + i] * x[1 + j] + e[1 + j] * x[1 + i];
  }
}

// Adjoint of x in envelope_mul: a (adjoint of y) -> b.
template <int DIM, int ORD, typename T>
__device__ __forceinline__ void envelope_mul_reverse(const T* e, const T* a, T* b) {
  T xb = e[0] * a[0];
#pragma unroll
  for (int d = 0; d < DIM; ++d) {
    xb += e[1 + d] * a[1 + d];
    b[1 + d] = e[0] * a[1 + d];
  }
#pragma unroll
  for (int k = 0; k < Jet<DIM, ORD>::NH; ++k) {
    const int i = pair_i(DIM, k), j = pair_j(DIM, k), q = 1 + DIM + k;
    xb += e[q] * a[q];
    b[1 + i] += e[1 + j] * a[q];
    b[1 + j] += e[1 + i] * a[q];
    b[q] = e[0] * a[q];
  }
  b[0] = xb;
}

constexpr int kTileK = 32;   // reduction chunk staged in shared memory
// output columns per thread: four in FP32, two in FP64.  A block of 128
// threads covers TC columns with TC / cols_per_thread column threads; the
// other factor of 128 are row threads of two points each.  Wide tiles (128
// FP32 / 64 FP64 columns, one row thread per warp, 8 points) serve layers
// wider than 32; narrow tiles (32 columns; 32 FP32 / 16 FP64 points) keep
// every lane busy on the 32-wide layers of the periodic networks.
template <typename T> constexpr int cols_per_thread() { return sizeof(T) == 4 ? 4 : 2; }
template <typename T> constexpr int tile_cols() { return 32 * cols_per_thread<T>(); }
constexpr int kNarrowTile = 32;
template <typename T, int TC> constexpr int col_threads() { return TC / cols_per_thread<T>(); }
template <typename T, int TC> constexpr int tile_pts() { return 2 * (128 / col_threads<T, TC>()); }

enum { EPI_OUTPUT = 0, EPI_HIDDEN = 1, EPI_REVERSE = 2 };

// Asynchronous global -> shared copy of one element (4 or 8 bytes); a copy
// with valid == false fills the destination with zeros and reads nothing.
template <typename T>
__device__ __forceinline__ void cp_async_elem(T* dst, const T* src, bool valid) {
  const uint32_t d = static_cast<uint32_t>(__cvta_generic_to_shared(dst));
  if constexpr (sizeof(T) == 4)
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;" ::"r"(d), "l"(src),
                 "r"(valid ? 4 : 0)
                 : "memory");
  else
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;" ::"r"(d), "l"(src),
                 "r"(valid ? 8 : 0)
                 : "memory");
}
__device__ __forceinline__ void cp_async_commit() {
  asm volatile("cp.async.commit_group;" ::: "memory");
}
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

// Shared memory of one pipeline stage of mode_gemm: B tile [kTileK][TC + 1]
// then A tile [points x C][kTileK + 1]; two stages.
template <typename T, int C, int TC> constexpr int mode_stage_elems() {
  return kTileK * (TC + 1) + tile_pts<T, TC>() * C * (kTileK + 1);
}
template <typename T, int C, int TC> constexpr int mode_gemm_smem() {
  return 2 * mode_stage_elems<T, C, TC>() * (int)sizeof(T);
}

// Per-mode jet GEMM.  blockIdx.x = tile of tile_pts points, blockIdx.y =
// tile of TC columns, blockIdx.z = mode b of the block; every pointer is
// already offset to the block's first mode and advanced by its *_mode stride.
//   EPI_OUTPUT : out = env * (A W^T + b on the value channel), W [N][Kd]
//   EPI_HIDDEN : pre = omega (A W^T + b), out = sine_jet(pre),   W [N][Kd]
//   EPI_REVERSE: out = omega sine_jet^T(pre_in, A W),            W [Kd][N]
// A: [n][C][Kd] (a_mode = 0 for the shared features); out, pre: [n][C][N].
// A thread holds 2 points x C channels x cols_per_thread columns: each
// shared-memory value it reads feeds cols_per_thread (A) or 2 C (B) FMAs.
// The next reduction chunk is copied into the other shared-memory stage by
// cp.async while the current one is consumed.  The A rows are padded to
// kTileK + 1 so the row threads of one warp read distinct banks.
template <typename T, int DIM, int ORD, int EPI, int TC>
__global__ void __launch_bounds__(128)
mode_gemm(const T* __restrict__ A, int64_t a_mode, const T* __restrict__ W, int64_t w_mode,
          const T* __restrict__ bias, int64_t b_mode, const T* __restrict__ env,
          const T* __restrict__ pre_in, T* __restrict__ pre_out, T* __restrict__ out,
          int64_t o_mode, int n, int Kd, int N, T omega) {
  constexpr int C = Jet<DIM, ORD>::C;
  constexpr int CPT = cols_per_thread<T>(), CT = col_threads<T, TC>(), PTS = tile_pts<T, TC>();
  constexpr int STAGE = mode_stage_elems<T, C, TC>(), LDA = kTileK + 1;
  extern __shared__ __align__(16) unsigned char mode_smem[];
  T* smem = reinterpret_cast<T*>(mode_smem);
  const int tid = threadIdx.x, tx = tid % CT, ty = tid / CT;
  const int mb = blockIdx.z;
  const int col0 = blockIdx.y * TC, p0 = blockIdx.x * PTS;
  A += mb * a_mode;
  W += mb * w_mode;
  // issue the copies of reduction chunk j0 into stage st
  auto stage_copy = [&](int j0, int st) {
    T* Bs = smem + st * STAGE;                 // [kTileK][TC + 1]
    T* As = Bs + kTileK * (TC + 1);            // [PTS C][kTileK + 1]
    for (int e = tid; e < kTileK * TC; e += 128) {
      int jj, col;
      if constexpr (EPI == EPI_REVERSE) {
        jj = e / TC;
        col = e % TC;
      } else {
        col = e / kTileK;
        jj = e % kTileK;
      }
      const int j = j0 + jj, o = col0 + col;
      const bool ok = j < Kd && o < N;
      const T* src = ok ? (EPI == EPI_REVERSE ? W + (int64_t)j * N + o : W + (int64_t)o * Kd + j) : W;
      cp_async_elem(&Bs[jj * (TC + 1) + col], src, ok);
    }
    for (int e = tid; e < PTS * C * kTileK; e += 128) {
      const int jj = e % kTileK, rc = e / kTileK;
      const int p = p0 + rc / C, c = rc % C, j = j0 + jj;
      const bool ok = p < n && j < Kd;
      cp_async_elem(&As[rc * LDA + jj], ok ? A + ((int64_t)p * C + c) * Kd + j : A, ok);
    }
    cp_async_commit();
  };
  T acc[2][C][CPT];
#pragma unroll
  for (int q = 0; q < 2; ++q)
#pragma unroll
    for (int c = 0; c < C; ++c)
#pragma unroll
      for (int u = 0; u < CPT; ++u) acc[q][c][u] = T(0);
  const int chunks = (Kd + kTileK - 1) / kTileK;
  stage_copy(0, 0);
  for (int ch = 0; ch < chunks; ++ch) {
    if (ch + 1 < chunks) {
      stage_copy((ch + 1) * kTileK, (ch + 1) & 1);
      cp_async_wait<1>();
    } else {
      cp_async_wait<0>();
    }
    __syncthreads();
    const T* Bs = smem + (ch & 1) * STAGE;
    const T* As = Bs + kTileK * (TC + 1);
#pragma unroll 4
    for (int jj = 0; jj < kTileK; ++jj) {
      T bv[CPT];
#pragma unroll
      for (int u = 0; u < CPT; ++u) bv[u] = Bs[jj * (TC + 1) + tx + CT * u];
#pragma unroll
      for (int q = 0; q < 2; ++q)
#pragma unroll
        for (int c = 0; c < C; ++c) {
          const T av = As[((ty * 2 + q) * C + c) * LDA + jj];
#pragma unroll
          for (int u = 0; u < CPT; ++u) acc[q][c][u] += av * bv[u];
        }
    }
    __syncthreads();  // the stage is refilled by the copies issued next
  }
  out += mb * o_mode;
#pragma unroll
  for (int u = 0; u < CPT; ++u) {
    const int o = col0 + tx + CT * u;
    if (o >= N) continue;
#pragma unroll
    for (int q = 0; q < 2; ++q) {
      const int p = p0 + ty * 2 + q;
      if (p >= n) continue;
      T z[C], y[C];
#pragma unroll
      for (int c = 0; c < C; ++c) z[c] = acc[q][c][u];
      const int64_t base = (int64_t)p * C * N + o;
      if constexpr (EPI == EPI_OUTPUT) {
        z[0] += bias[mb * b_mode + o];
        if (ORD < 3 && env) {  // third-order jets take the identity envelope
          T e[C];
#pragma unroll
          for (int c = 0; c < C; ++c) e[c] = env[(int64_t)p * C + c];
          envelope_mul<DIM, ORD>(e, z, y);
        } else {
#pragma unroll
          for (int c = 0; c < C; ++c) y[c] = z[c];
        }
      } else if constexpr (EPI == EPI_HIDDEN) {
        z[0] += bias[mb * b_mode + o];
#pragma unroll
        for (int c = 0; c < C; ++c) {
          z[c] *= omega;
          if (pre_out) pre_out[mb * o_mode + base + (int64_t)c * N] = z[c];
        }
        sine_jet<DIM, ORD>(z, y);
      } else {
        T pz[C];
#pragma unroll
        for (int c = 0; c < C; ++c) pz[c] = pre_in[mb * o_mode + base + (int64_t)c * N];
        sine_jet_reverse<DIM, ORD>(pz, z, y);
#pragma unroll
        for (int c = 0; c < C; ++c) y[c] *= omega;
      }
#pragma unroll
      for (int c = 0; c < C; ++c) out[base + (int64_t)c * N] = y[c];
    }
  }
}

// Output layer with few columns (N <= kNarrowCols, a vector potential's 3):
// a block takes 32 points of one mode; thread (u, p) = (tid / 32, tid % 32)
// holds column u of point p over all C channels.  The input rows are staged
// [C][32 points][33] through shared memory in coalesced 32-wide chunks, W_k
// (N x Kd) sits in shared memory; + bias on the value channel, x envelope.
// grid = (ceil(n / 32), B).
constexpr int kNarrowCols = 4, kNarrowPts = 32;
template <typename T, int C> constexpr int narrow_smem(int N, int Kd) {
  return (C * kNarrowPts * (kTileK + 1) + N * Kd) * (int)sizeof(T);
}
template <typename T, int DIM, int ORD>
__global__ void __launch_bounds__(128)
mode_output_narrow(const T* __restrict__ A, int64_t a_mode, const T* __restrict__ W,
                   int64_t w_mode, const T* __restrict__ bias, int64_t b_mode,
                   const T* __restrict__ env, T* __restrict__ out, int64_t o_mode, int n, int Kd,
                   int N) {
  constexpr int C = Jet<DIM, ORD>::C;
  extern __shared__ __align__(16) unsigned char narrow_smem_raw[];
  T* As = reinterpret_cast<T*>(narrow_smem_raw);        // [C][32][kTileK + 1]
  T* Ws = As + C * kNarrowPts * (kTileK + 1);           // [N][Kd]
  const int mb = blockIdx.y, p0 = blockIdx.x * kNarrowPts;
  const int tid = threadIdx.x, pl = tid % kNarrowPts, u = tid / kNarrowPts;
  A += mb * a_mode;
  W += mb * w_mode;
  for (int e = tid; e < N * Kd; e += blockDim.x) Ws[e] = W[e];
  T acc[C];
#pragma unroll
  for (int c = 0; c < C; ++c) acc[c] = T(0);
  for (int j0 = 0; j0 < Kd; j0 += kTileK) {
    __syncthreads();
    for (int e = tid; e < kNarrowPts * C * kTileK; e += blockDim.x) {
      const int jj = e % kTileK, rc = e / kTileK;  // rc = point * C + channel
      const int p = p0 + rc / C, c = rc % C, j = j0 + jj;
      As[(c * kNarrowPts + rc / C) * (kTileK + 1) + jj] =
          (p < n && j < Kd) ? A[((int64_t)p * C + c) * Kd + j] : T(0);
    }
    __syncthreads();
    if (u < N) {
      const int jn = min(kTileK, Kd - j0);
      for (int jj = 0; jj < jn; ++jj) {
        const T w = Ws[u * Kd + j0 + jj];
#pragma unroll
        for (int c = 0; c < C; ++c) acc[c] += As[(c * kNarrowPts + pl) * (kTileK + 1) + jj] * w;
      }
    }
  }
  const int p = p0 + pl;
  if (u >= N || p >= n) return;
  T e[C], y[C];
  acc[0] += bias[mb * b_mode + u];
  if constexpr (ORD == 3) {  // third-order jets take the identity envelope
#pragma unroll
    for (int c = 0; c < C; ++c) y[c] = acc[c];
  } else {
#pragma unroll
    for (int c = 0; c < C; ++c) e[c] = env ? env[(int64_t)p * C + c] : (c == 0 ? T(1) : T(0));
    envelope_mul<DIM, ORD>(e, acc, y);
  }
  T* o = out + mb * o_mode + (int64_t)p * C * N;
#pragma unroll
  for (int c = 0; c < C; ++c) o[(int64_t)c * N + u] = y[c];
}

// part[s][b][o][i] = sum over rows r in split s of Abar[b][r][o] X[b][r][i],
// rows r = (point, channel).  grid = (tiles of WT x WT, B, splits), threads
// (WT / 4)^2 (256 for 64-wide tiles, 64 for the 32-wide layers), 4 x 4
// outputs each; rows staged 32 at a time into double-buffered shared memory
// by cp.async.
constexpr int kWgRows = 32;
template <int WT> constexpr int wg_threads() { return (WT / 4) * (WT / 4); }
template <typename T, int WT> constexpr int mode_wgrad_smem() {
  return 2 * 2 * kWgRows * (WT + 4) * (int)sizeof(T);
}
template <typename T, int WT>
__global__ void __launch_bounds__(wg_threads<WT>())
mode_wgrad(const T* __restrict__ Abar, const T* __restrict__ X, int64_t x_mode, int64_t rows,
           int N, int Kin, int64_t rows_per_split, T* __restrict__ part) {
  constexpr int kWgTile = WT, kWgLd = WT + 4, NT = wg_threads<WT>(), TW = WT / 4;
  extern __shared__ __align__(16) unsigned char wg_smem[];
  T* smem = reinterpret_cast<T*>(wg_smem);  // [stage][A, X][kWgRows][kWgLd]
  const int tiles_i = (Kin + kWgTile - 1) / kWgTile;
  const int o0 = (blockIdx.x / tiles_i) * kWgTile, i0 = (blockIdx.x % tiles_i) * kWgTile;
  const int mb = blockIdx.y, s = blockIdx.z;
  const int tid = threadIdx.x, tx = tid % TW, ty = tid / TW;
  Abar += (int64_t)mb * rows * N;
  X += mb * x_mode;
  const int64_t r0 = (int64_t)s * rows_per_split;
  const int64_t r1 = r0 + rows_per_split < rows ? r0 + rows_per_split : rows;
  auto stage_copy = [&](int64_t rb, int st) {
    T* As = smem + st * 2 * kWgRows * kWgLd;
    T* Xs = As + kWgRows * kWgLd;
    for (int e = tid; e < kWgRows * kWgTile; e += NT) {
      const int rr = e / kWgTile, cc = e % kWgTile;
      const int64_t r = rb + rr;
      const bool ra = r < r1 && o0 + cc < N, rx = r < r1 && i0 + cc < Kin;
      cp_async_elem(&As[rr * kWgLd + cc], ra ? Abar + r * N + o0 + cc : Abar, ra);
      cp_async_elem(&Xs[rr * kWgLd + cc], rx ? X + r * Kin + i0 + cc : X, rx);
    }
    cp_async_commit();
  };
  T acc[4][4];
#pragma unroll
  for (int a = 0; a < 4; ++a)
#pragma unroll
    for (int c = 0; c < 4; ++c) acc[a][c] = T(0);
  const int64_t chunks = r1 > r0 ? (r1 - r0 + kWgRows - 1) / kWgRows : 0;
  if (chunks > 0) stage_copy(r0, 0);
  for (int64_t ch = 0; ch < chunks; ++ch) {
    if (ch + 1 < chunks) {
      stage_copy(r0 + (ch + 1) * kWgRows, (int)((ch + 1) & 1));
      cp_async_wait<1>();
    } else {
      cp_async_wait<0>();
    }
    __syncthreads();
    const T* As = smem + (ch & 1) * 2 * kWgRows * kWgLd;
    const T* Xs = As + kWgRows * kWgLd;
#pragma unroll 8
    for (int rr = 0; rr < kWgRows; ++rr) {
      T a[4], x[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        a[u] = As[rr * kWgLd + ty * 4 + u];
        x[u] = Xs[rr * kWgLd + tx * 4 + u];
      }
#pragma unroll
      for (int u = 0; u < 4; ++u)
#pragma unroll
        for (int v = 0; v < 4; ++v) acc[u][v] += a[u] * x[v];
    }
    __syncthreads();
  }
  T* dst = part + ((int64_t)s * gridDim.y + mb) * N * Kin;
#pragma unroll
  for (int u = 0; u < 4; ++u)
#pragma unroll
    for (int v = 0; v < 4; ++v) {
      const int o = o0 + ty * 4 + u, i = i0 + tx * 4 + v;
      if (o < N && i < Kin) dst[(int64_t)o * Kin + i] = acc[u][v];
    }
}

// gW[b][o][i] (+)= sum_s part[s][b][o][i]
template <typename T>
__global__ void mode_wgrad_reduce(const T* __restrict__ part, int splits, int64_t per_split,
                                  int accumulate, T* __restrict__ gW) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < per_split;
       i += (int64_t)gridDim.x * blockDim.x) {
    T s = T(0);
    for (int z = 0; z < splits; ++z) s += part[z * per_split + i];
    gW[i] = accumulate ? gW[i] + s : s;
  }
}

// gb[b][o] (+)= sum_p Abar[b][p][0][o].  One block of 16 warps per mode b:
// warp w sums points w, w + 16, ..., its lanes reading 32 consecutive
// columns of a point's value row; the partial sums are added in a fixed
// order.
constexpr int kBiasWarps = 16;
template <typename T, int C>
__global__ void __launch_bounds__(32 * kBiasWarps)
mode_bias(const T* __restrict__ Abar, int n, int N, int accumulate, T* __restrict__ gb) {
  __shared__ T red[kBiasWarps][32];
  const int mb = blockIdx.x, lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const T* a = Abar + (int64_t)mb * n * C * N;
  for (int o0 = 0; o0 < N; o0 += 32) {
    const int o = o0 + lane;
    T acc[4] = {T(0), T(0), T(0), T(0)};  // four independent chains hide the load latency
    if (o < N) {
      int p = w;
      for (; p + 3 * kBiasWarps < n; p += 4 * kBiasWarps)
#pragma unroll
        for (int k = 0; k < 4; ++k) acc[k] += a[(int64_t)(p + k * kBiasWarps) * C * N + o];
      for (; p < n; p += kBiasWarps) acc[0] += a[(int64_t)p * C * N + o];
    }
    red[w][lane] = (acc[0] + acc[1]) + (acc[2] + acc[3]);
    __syncthreads();
    if (w == 0 && o < N) {
      T s = T(0);
#pragma unroll
      for (int k = 0; k < kBiasWarps; ++k) s += red[k][lane];
      T* g = gb + (int64_t)mb * N + o;
      *g = accumulate ? *g + s : s;
    }
    __syncthreads();
  }
}

// adjoint of the raw output: b = envelope_mul_reverse(env, a), [B][n][C][N]
template <typename T, int DIM, int ORD>
__global__ void mode_envelope_reverse(const T* __restrict__ env, const T* __restrict__ a,
                                      int64_t total_pn, int n, int N, T* __restrict__ b) {
  constexpr int C = Jet<DIM, ORD>::C;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total_pn;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t row = i / N;  // (mode, point)
    const int o = (int)(i % N), p = (int)(row % n);
    const int64_t base = row * C * N + o;
    T e[C], av[C], bv[C];
#pragma unroll
    for (int c = 0; c < C; ++c) {
      e[c] = env ? env[(int64_t)p * C + c] : (c == 0 ? T(1) : T(0));
      av[c] = a[base + (int64_t)c * N];
    }
    envelope_mul_reverse<DIM, ORD>(e, av, bv);
#pragma unroll
    for (int c = 0; c < C; ++c) b[base + (int64_t)c * N] = bv[c];
  }
}

// 3D second-order vector potential A (3 outputs per mode) -> velocity
// u = curl A into U[(p*3 + a)][col] and its gradient d_j u_a into
// D[(p*9 + a*3 + j)][col], col = mode0 + b (velocity_trace_jet2.py:93-101).
template <typename T>
__global__ void velocity_fields(const T* __restrict__ out, int B, int n, int K, int mode0,
                                T* __restrict__ U, T* __restrict__ D) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= (int64_t)B * n) return;
  const int mb = (int)(i / n), p = (int)(i % n);
  const T* o = out + ((int64_t)mb * n + p) * 10 * 3;  // [10][3] of this point
  auto g = [&](int comp, int axis) { return o[(1 + axis) * 3 + comp]; };
  auto h = [&](int comp, int a, int b) { return o[(4 + hess_slot(a < b ? a : b, a < b ? b : a)) * 3 + comp]; };
  const int col = mode0 + mb;
  U[((int64_t)p * 3 + 0) * K + col] = g(2, 1) - g(1, 2);
  U[((int64_t)p * 3 + 1) * K + col] = g(0, 2) - g(2, 0);
  U[((int64_t)p * 3 + 2) * K + col] = g(1, 0) - g(0, 1);
#pragma unroll
  for (int a = 0; a < 3; ++a)
#pragma unroll
    for (int j = 0; j < 3; ++j)
      D[((int64_t)p * 9 + a * 3 + j) * K + col] =
          h((a + 2) % 3, j, (a + 1) % 3) - h((a + 1) % 3, j, (a + 2) % 3);
}

// Adjoint of velocity_fields: GU, GD (layouts of U, D) -> output adjoint
// [B][n][10][3] (velocity/core.py:32-38 lift).
template <typename T>
__global__ void velocity_lift(const T* __restrict__ GU, const T* __restrict__ GD, int B, int n,
                              int K, int mode0, T* __restrict__ adj) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= (int64_t)B * n) return;
  const int mb = (int)(i / n), p = (int)(i % n), col = mode0 + mb;
  T a[10][3];
#pragma unroll
  for (int c = 0; c < 10; ++c)
#pragma unroll
    for (int k = 0; k < 3; ++k) a[c][k] = T(0);
  const T u0 = GU[((int64_t)p * 3 + 0) * K + col], u1 = GU[((int64_t)p * 3 + 1) * K + col],
          u2 = GU[((int64_t)p * 3 + 2) * K + col];
  a[1 + 1][2] += u0; a[1 + 2][1] -= u0;
  a[1 + 2][0] += u1; a[1 + 0][2] -= u1;
  a[1 + 0][1] += u2; a[1 + 1][0] -= u2;
#pragma unroll
  for (int ax = 0; ax < 3; ++ax)
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      const T gd = GD[((int64_t)p * 9 + ax * 3 + j) * K + col];
      const int b1 = (ax + 1) % 3, b2 = (ax + 2) % 3;
      a[4 + hess_slot(j < b1 ? j : b1, j < b1 ? b1 : j)][b2] += gd;
      a[4 + hess_slot(j < b2 ? j : b2, j < b2 ? b2 : j)][b1] -= gd;
    }
  T* dst = adj + ((int64_t)mb * n + p) * 30;
#pragma unroll
  for (int c = 0; c < 10; ++c)
#pragma unroll
    for (int k = 0; k < 3; ++k) dst[c * 3 + k] = a[c][k];
}

// 2D scalar potential of one output per mode, first-order jets: the value
// into V[p][col] and the gradient into G[(p*2 + a)][col], col = mode0 + b
// (hardcoded_backend.py:3455-3460 raw_value / raw_gradient columns).
template <typename T>
__global__ void potential_fields(const T* __restrict__ out, int B, int n, int K, int mode0,
                                 T* __restrict__ V, T* __restrict__ G) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= (int64_t)B * n) return;
  const int mb = (int)(i / n), p = (int)(i % n), col = mode0 + mb;
  const T* o = out + ((int64_t)mb * n + p) * 3;  // [3][1] of this point
  V[(int64_t)p * K + col] = o[0];
  G[((int64_t)p * 2) * K + col] = o[1];
  G[((int64_t)p * 2 + 1) * K + col] = o[2];
}

// Adjoint of potential_fields: dV, dG -> output-jet adjoints [B][n][3][1].
template <typename T>
__global__ void potential_lift(const T* __restrict__ dV, const T* __restrict__ dG, int B, int n,
                               int K, int mode0, T* __restrict__ adj) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= (int64_t)B * n) return;
  const int mb = (int)(i / n), p = (int)(i % n), col = mode0 + mb;
  T* a = adj + ((int64_t)mb * n + p) * 3;
  a[0] = dV[(int64_t)p * K + col];
  a[1] = dG[((int64_t)p * 2) * K + col];
  a[2] = dG[((int64_t)p * 2 + 1) * K + col];
}

// A[r][k] -= mean over rows of column k (one block of 256 threads per
// column, FP64 sums): the sample-wise mean-zero gauge of the streamfunction
// (hardcoded_backend.py:3461-3465) and, applied to an adjoint, its transpose
// (:3579-3583).
template <typename T>
__global__ void column_center(T* __restrict__ A, int64_t rows, int K) {
  __shared__ double red[8];
  const int k = blockIdx.x;
  double s = 0.0;
  for (int64_t r = threadIdx.x; r < rows; r += blockDim.x) s += (double)A[r * K + k];
  for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  double tot = 0.0;
  for (int w = 0; w < (int)(blockDim.x >> 5); ++w) tot += red[w];
  const T mean = (T)(tot / (double)rows);
  for (int64_t r = threadIdx.x; r < rows; r += blockDim.x) A[r * K + k] -= mean;
}

// ------------------------------------------------------- per-mode Adam
// Tensors are stacked [K][...]; per_mode[t] elements of tensor t per mode.
struct ModeAdamTable {
  AdamTable t;
  int64_t per_mode[kMaxAdamTensors];
};

// norm2[k] = sum over tensors of |g_k|^2 (one block per mode); a non-finite
// gradient makes the mode's norm non-finite.
template <typename T>
__global__ void mode_adam_norms(ModeAdamTable mt, double* __restrict__ norm2) {
  __shared__ double red[32];
  const int k = blockIdx.x;
  double s = 0.0;
  bool nf = false;
  for (int ti = 0; ti < mt.t.n; ++ti) {
    const T* g = static_cast<const T*>(mt.t.g[ti]) + (int64_t)k * mt.per_mode[ti];
    for (int64_t i = threadIdx.x; i < mt.per_mode[ti]; i += blockDim.x) {
      const double v = (double)g[i];
      if (!isfinite(v)) nf = true;
      s += v * v;
    }
  }
  for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  nf = __any_sync(0xffffffffu, nf);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = nf ? CUDART_NAN : s;
  __syncthreads();
  if (threadIdx.x < 32) {
    double v = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.0;
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (threadIdx.x == 0) norm2[k] = v;
  }
}

// The transaction: commit when the objective's gate (if any) is 0 and
// every active mode's norm is finite and positive (native_cupy_core.py:
// 157-158; hardcoded_backend.py:2204-2212 with its active-mode mask).  Per
// mode: norms out, the clip scale (0 for a mode left unchanged) and the
// bias corrections of its step t = steps + 1, where steps is one shared
// count (per_mode = 0) or one count per mode; the counts of the updated
// modes advance.  par[k] = (scale, lr / (1 - 0.9^t), 1 / (1 - 0.999^t)).
__global__ void mode_adam_finalize(const double* __restrict__ norm2,
                                   const int* __restrict__ gate, const int* __restrict__ active,
                                   int K, double clip, double lr, int* __restrict__ steps,
                                   int per_mode, double* __restrict__ norms_out,
                                   int* __restrict__ committed, double* __restrict__ par) {
  __shared__ int ok_all;
  if (threadIdx.x == 0) ok_all = !gate || *gate == 0;
  __syncthreads();
  for (int k = threadIdx.x; k < K; k += blockDim.x) {
    const double nm = sqrt(norm2[k]);
    if (norms_out) norms_out[k] = nm;
    const bool act = !active || active[k] != 0;
    if (act && !(isfinite(nm) && nm > 0.0)) atomicAnd(&ok_all, 0);
  }
  __syncthreads();
  const bool ok = ok_all != 0;
  for (int k = threadIdx.x; k < K; k += blockDim.x) {
    const double nm = sqrt(norm2[k]);
    const bool upd = ok && (!active || active[k] != 0);
    const double t = (double)(per_mode ? steps[k] : steps[0]) + 1.0;
    par[3 * k] = upd ? fmin(1.0, clip / fmax(nm, 1e-30)) : 0.0;
    par[3 * k + 1] = lr / (1.0 - pow(0.9, t));
    par[3 * k + 2] = 1.0 / (1.0 - pow(0.999, t));
  }
  __syncthreads();  // every thread has read the step counts
  for (int k = threadIdx.x; k < K; k += blockDim.x)
    if (per_mode && ok && (!active || active[k] != 0)) steps[k] += 1;
  if (threadIdx.x == 0) {
    if (committed) *committed = ok;
    if (!per_mode && ok) steps[0] += 1;
  }
}

template <typename T>
__global__ void mode_adam_update(ModeAdamTable mt, const double* __restrict__ par) {
  const int64_t total = mt.t.off[mt.t.n];
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int ti = adam_find(mt.t, i);
    const int64_t j = i - mt.t.off[ti];
    const int k = (int)(j / mt.per_mode[ti]);
    const double sc = par[3 * k];
    if (sc == 0.0) continue;  // mode not updated
    const T lr_c1 = (T)par[3 * k + 1], inv_c2 = (T)par[3 * k + 2];
    T* p = static_cast<T*>(mt.t.p[ti]);
    T* m = static_cast<T*>(mt.t.m[ti]);
    T* v = static_cast<T*>(mt.t.v[ti]);
    const T g = static_cast<const T*>(mt.t.g[ti])[j] * (T)sc;
    const T mn = T(0.9) * m[j] + T(0.1) * g;
    const T vn = T(0.999) * v[j] + T(0.001) * g * g;
    m[j] = mn;
    v[j] = vn;
    p[j] -= lr_c1 * mn / (sqrt(vn * inv_c2) + T(1e-8));
  }
}

// ------------------------------------------------------------- host side
size_t a256(size_t x) { return (x + 255) & ~size_t(255); }

int mode_channels(const neb_modes* m) {
  return 1 + m->dim + (m->order >= 2 ? m->dim * (m->dim + 1) / 2 : 0) + (m->order == 3 ? 4 : 0);
}

int check_modes(const neb_modes* m) {
  NEB_REQUIRE(m != nullptr, "null neb_modes");
  NEB_REQUIRE(m->dim == 2 || m->dim == 3, "neb_modes.dim must be 2 or 3");
  NEB_REQUIRE(m->order == 1 || m->order == 2 || (m->order == 3 && m->dim == 2),
              "neb_modes.order must be 1 or 2 (or 3 in 2D)");
  NEB_REQUIRE(m->n_layers >= 1 && m->n_layers <= NEB_MAX_HIDDEN + 1,
              "neb_modes.n_layers must be in [1, %d]", NEB_MAX_HIDDEN + 1);
  for (int l = 0; l <= m->n_layers; ++l)
    NEB_REQUIRE(m->widths[l] > 0 && m->widths[l] <= 65536, "neb_modes.widths[%d] invalid", l);
  NEB_REQUIRE(m->precision == NEB_PREC_FP32 || m->precision == NEB_PREC_FP64 ||
                  m->precision == NEB_PREC_TF32 || m->precision == NEB_PREC_BF16X9,
              "neb_modes: FP32 (also with TF32 / BF16x9 tensor-core GEMMs) or FP64 parameters");
  NEB_REQUIRE(m->n_modes > 0, "neb_modes.n_modes must be positive");
  return NEB_OK;
}

size_t esize(const neb_modes* m) { return m->precision == NEB_PREC_FP64 ? 8 : 4; }

// Tape of a block of B modes: for hidden layer j (0..n_layers-2) the scaled
// pre-activation P_j and the output X_{j+1}, each [B][n][C][w_{j+1}].
struct ModeTape {
  size_t pre[NEB_MAX_HIDDEN + 1], x[NEB_MAX_HIDDEN + 2], total;
};

ModeTape mode_tape(const neb_modes* m, int B, int64_t n) {
  ModeTape t{};
  const size_t C = mode_channels(m), es = esize(m);
  size_t off = 0;
  for (int j = 0; j + 1 < m->n_layers; ++j) {
    const size_t sz = a256((size_t)B * n * C * m->widths[j + 1] * es);
    t.pre[j] = off;
    off += sz;
    t.x[j + 1] = off;
    off += sz;
  }
  t.total = off;
  return t;
}

int max_width(const neb_modes* m) {
  int w = 0;
  for (int l = 0; l <= m->n_layers; ++l) w = std::max(w, m->widths[l]);
  return w;
}

constexpr int kMaxWgradSplits = 32;

// Workspace of the reverse pass: two adjoint buffers [B][n][C][max w] and
// the weight-gradient split partials.
struct ModeWs {
  size_t a0, a1, part, total;
};

ModeWs mode_ws(const neb_modes* m, int B, int64_t n) {
  ModeWs w{};
  const size_t C = mode_channels(m), es = esize(m), mw = max_width(m);
  const size_t adj = a256((size_t)B * n * C * mw * es);
  w.a0 = 0;
  w.a1 = adj;
  w.part = 2 * adj;
  w.total = w.part + a256((size_t)kMaxWgradSplits * B * mw * mw * es);
  return w;
}

// Epilogue of a per-mode GEMM whose product Z is already in place (the
// tensor-core forms): EPI_HIDDEN: z = omega (Z + b on the value channel) ->
// pre (when kept), out = sine_jet(z); EPI_OUTPUT: out = env * (Z + b);
// EPI_REVERSE: out = omega sine_jet^T(pre_in, Z).  Z lives in pre (hidden
// layers with a tape) or in out; each thread owns one (mode, point, column).
template <int DIM, int ORD, int EPI>
__global__ void mode_epilogue(const float* __restrict__ Zsrc, const float* __restrict__ bias,
                              int64_t b_mode, const float* __restrict__ env,
                              const float* __restrict__ pre_in, float* __restrict__ pre_out,
                              float* __restrict__ out, int64_t o_mode, int B, int n, int N,
                              float omega) {
  constexpr int C = Jet<DIM, ORD>::C;
  const int64_t total = (int64_t)B * n * N;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int o = (int)(e % N);
    const int64_t bp = e / N;
    const int p = (int)(bp % n), mb = (int)(bp / n);
    const int64_t base = mb * o_mode + (int64_t)p * C * N + o;
    float z[C], y[C];
#pragma unroll
    for (int c = 0; c < C; ++c) z[c] = Zsrc[base + (int64_t)c * N];
    if constexpr (EPI == EPI_HIDDEN) {
      z[0] += bias[mb * b_mode + o];
#pragma unroll
      for (int c = 0; c < C; ++c) {
        z[c] *= omega;
        if (pre_out) pre_out[base + (int64_t)c * N] = z[c];
      }
      sine_jet<DIM, ORD>(z, y);
    } else if constexpr (EPI == EPI_OUTPUT) {
      z[0] += bias[mb * b_mode + o];
      if (ORD < 3 && env) {
        float ev[C];
#pragma unroll
        for (int c = 0; c < C; ++c) ev[c] = env[(int64_t)p * C + c];
        envelope_mul<DIM, ORD>(ev, z, y);
      } else {
#pragma unroll
        for (int c = 0; c < C; ++c) y[c] = z[c];
      }
    } else {
      float pz[C];
#pragma unroll
      for (int c = 0; c < C; ++c) pz[c] = pre_in[base + (int64_t)c * N];
      sine_jet_reverse<DIM, ORD>(pz, z, y);
#pragma unroll
      for (int c = 0; c < C; ++c) y[c] *= omega;
    }
#pragma unroll
    for (int c = 0; c < C; ++c) out[base + (int64_t)c * N] = y[c];
  }
}

// The per-mode GEMM of the tensor-core forms: one strided-batched cuBLAS
// GEMM over the block's modes (the shared features have stride 0), then the
// epilogue.  Rows are (point, channel) pairs: [n C][Kd] per mode.
template <int DIM, int ORD, int EPI>
int tc_mode_gemm(const float* A, int64_t a_mode, const float* W, int64_t w_mode,
                 const float* bias, int64_t b_mode, const float* env, const float* pre_in,
                 float* pre_out, float* out, int64_t o_mode, int B, int n, int Kd, int N,
                 double omega, cudaStream_t s, const char* name) {
  constexpr int C = Jet<DIM, ORD>::C;
  const int64_t R = (int64_t)n * C;
  float* Z = (EPI == EPI_HIDDEN && pre_out) ? pre_out : out;
  int st;
  if constexpr (EPI == EPI_REVERSE)  // [R][N] = A [R][Kd] W [Kd][N]
    st = tc_sgemm_batched(s, CUBLAS_OP_N, CUBLAS_OP_N, N, R, Kd, 1.f, W, N, w_mode, A, Kd,
                          a_mode, 0.f, Z, N, o_mode, B, name);
  else  // [R][N] = A [R][Kd] W^T, W [N][Kd]
    st = tc_sgemm_batched(s, CUBLAS_OP_T, CUBLAS_OP_N, N, R, Kd, 1.f, W, Kd, w_mode, A, Kd,
                          a_mode, 0.f, Z, N, o_mode, B, name);
  if (st) return st;
  const int64_t total = (int64_t)B * n * N;
  KernelScope ks("mode_epilogue", s, 0, (double)total * C * 4 * (EPI == EPI_REVERSE ? 3 : 2));
  mode_epilogue<DIM, ORD, EPI><<<(int)std::min<int64_t>(ceil_div(total, 256), 65535), 256, 0, s>>>(
      Z, bias, b_mode, env, pre_in, EPI == EPI_HIDDEN ? pre_out : nullptr, out, o_mode, B, n, N,
      (float)omega);
  NEB_LAUNCH_CHECK();
  return NEB_OK;
}

template <typename T, int DIM, int ORD, int EPI, int TC>
int run_mode_gemm(int dev, const T* A, int64_t a_mode, const T* W, int64_t w_mode,
                  const T* bias, int64_t b_mode, const T* env, const T* pre_in, T* pre_out,
                  T* out, int64_t o_mode, int B, int n, int Kd, int N, double omega,
                  cudaStream_t s) {
  constexpr int C = Jet<DIM, ORD>::C;
  static bool configured[kMaxDevices] = {};
  constexpr int smem = mode_gemm_smem<T, C, TC>();
  if (!configured[dev]) {
    NEB_CUDA_CHECK(cudaFuncSetAttribute(mode_gemm<T, DIM, ORD, EPI, TC>,
                                        cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
    configured[dev] = true;
  }
  NEB_REQUIRE(ceil_div(N, TC) <= 65535, "mode GEMM: width %d too large", N);
  dim3 grid((unsigned)ceil_div(n, tile_pts<T, TC>()), (unsigned)ceil_div(N, TC), (unsigned)B);
  mode_gemm<T, DIM, ORD, EPI, TC><<<grid, 128, smem, s>>>(A, a_mode, W, w_mode, bias, b_mode,
                                                          env, pre_in, pre_out, out, o_mode, n,
                                                          Kd, N, (T)omega);
  NEB_LAUNCH_CHECK();
  return NEB_OK;
}

template <typename T, int DIM, int ORD, int EPI>
int launch_mode_gemm(const T* A, int64_t a_mode, const T* W, int64_t w_mode, const T* bias,
                     int64_t b_mode, const T* env, const T* pre_in, T* pre_out, T* out,
                     int64_t o_mode, int B, int n, int Kd, int N, double omega, cudaStream_t s,
                     const char* name) {
  constexpr int C = Jet<DIM, ORD>::C;
  KernelScope ks(name, s, 2.0 * B * n * C * (double)Kd * N,
                 (double)B * n * C * (Kd + N * (EPI == EPI_OUTPUT ? 1 : 2)) * sizeof(T));
  int dev = 0, sms = 0;
  if (int st = device_sms(&dev, &sms)) return st;
  if constexpr (sizeof(T) == 4) {
    if (gemm_compute() && !(EPI == EPI_OUTPUT && N <= kNarrowCols))
      return tc_mode_gemm<DIM, ORD, EPI>(A, a_mode, W, w_mode, bias, b_mode, env, pre_in, pre_out,
                                         out, o_mode, B, n, Kd, N, omega, s, name);
  }
  if (EPI == EPI_OUTPUT && N <= kNarrowCols) {
    const int smem = narrow_smem<T, C>(N, Kd);
    NEB_REQUIRE(smem <= 200 * 1024, "mode output layer: %d inputs too many", Kd);
    static int configured_narrow[kMaxDevices] = {};
    if (configured_narrow[dev] < smem) {
      NEB_CUDA_CHECK(cudaFuncSetAttribute(mode_output_narrow<T, DIM, ORD>,
                                          cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
      configured_narrow[dev] = smem;
    }
    mode_output_narrow<T, DIM, ORD>
        <<<dim3((unsigned)ceil_div(n, kNarrowPts), (unsigned)B), 128, smem, s>>>(
            A, a_mode, W, w_mode, bias, b_mode, env, out, o_mode, n, Kd, N);
    NEB_LAUNCH_CHECK();
    return NEB_OK;
  }
  if (N <= kNarrowTile)
    return run_mode_gemm<T, DIM, ORD, EPI, kNarrowTile>(dev, A, a_mode, W, w_mode, bias, b_mode,
                                                        env, pre_in, pre_out, out, o_mode, B, n,
                                                        Kd, N, omega, s);
  return run_mode_gemm<T, DIM, ORD, EPI, tile_cols<T>()>(dev, A, a_mode, W, w_mode, bias, b_mode,
                                                         env, pre_in, pre_out, out, o_mode, B, n,
                                                         Kd, N, omega, s);
}

template <typename T, int DIM, int ORD>
int modes_forward_t(const neb_modes* m, int start, int B, const void* const* Wv,
                    const void* const* bv, const T* feats, const T* env, int64_t n, char* tape,
                    T* out, cudaStream_t s, bool eval = false) {
  constexpr int C = Jet<DIM, ORD>::C;
  ModeTape tl = mode_tape(m, B, n);
  // evaluation: no pre-activations, the layer outputs in two alternating buffers
  const size_t ping = a256((size_t)B * n * C * max_width(m) * sizeof(T));
  const T* x = feats;
  int64_t x_mode = 0;
  for (int j = 0; j < m->n_layers; ++j) {
    const int in = m->widths[j], o = m->widths[j + 1];
    const T* W = (const T*)Wv[j] + (int64_t)start * o * in;
    const T* b = (const T*)bv[j] + (int64_t)start * o;
    const int64_t o_mode = (int64_t)n * C * o;
    int st;
    if (j + 1 < m->n_layers) {
      T* pre = eval ? nullptr : (T*)(tape + tl.pre[j]);
      T* y = eval ? (T*)(tape + (j & 1) * ping) : (T*)(tape + tl.x[j + 1]);
      const double om = j == 0 ? m->omega_first : m->omega_hidden;
      st = launch_mode_gemm<T, DIM, ORD, EPI_HIDDEN>(x, x_mode, W, (int64_t)o * in, b, o, nullptr,
                                                     nullptr, pre, y, o_mode, B, (int)n, in, o, om,
                                                     s, "mode_layer_fwd");
      x = y;
      x_mode = o_mode;
    } else {
      st = launch_mode_gemm<T, DIM, ORD, EPI_OUTPUT>(x, x_mode, W, (int64_t)o * in, b, o, env,
                                                     nullptr, nullptr, out, o_mode, B, (int)n, in,
                                                     o, 1.0, s, "mode_output_fwd");
    }
    if (st) return st;
  }
  return NEB_OK;
}

template <typename T, int WT>
int run_mode_wgrad(int dev, dim3 grid, const T* Abar, const T* X, int64_t x_mode, int64_t rows,
                   int N, int Kin, int64_t per, T* part, cudaStream_t s) {
  static bool configured[kMaxDevices] = {};
  if (!configured[dev]) {
    NEB_CUDA_CHECK(cudaFuncSetAttribute(mode_wgrad<T, WT>,
                                        cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        mode_wgrad_smem<T, WT>()));
    configured[dev] = true;
  }
  mode_wgrad<T, WT><<<grid, wg_threads<WT>(), mode_wgrad_smem<T, WT>(), s>>>(Abar, X, x_mode,
                                                                             rows, N, Kin, per,
                                                                             part);
  NEB_LAUNCH_CHECK();
  return NEB_OK;
}

template <typename T, int DIM, int ORD>
int modes_backward_t(const neb_modes* m, int start, int B, const void* const* Wv, const T* feats,
                     const T* env, int64_t n, const char* tape, const T* adjoint,
                     void* const* gW, void* const* gb, int accumulate, char* ws, cudaStream_t s) {
  constexpr int C = Jet<DIM, ORD>::C;
  ModeTape tl = mode_tape(m, B, n);
  ModeWs wl = mode_ws(m, B, n);
  T* buf[2] = {(T*)(ws + wl.a0), (T*)(ws + wl.a1)};
  T* part = (T*)(ws + wl.part);
  const int L = m->n_layers;
  int dev = 0, sms = 0;
  if (int st = device_sms(&dev, &sms)) return st;
  {  // adjoint of the raw output
    const int No = m->widths[L];
    const int64_t total = (int64_t)B * n * No;
    KernelScope ks("mode_envelope_reverse", s, 0, 2.0 * total * C * sizeof(T));
    mode_envelope_reverse<T, DIM, ORD><<<(int)std::min<int64_t>(ceil_div(total, 256), 8192), 256, 0,
                                         s>>>(env, adjoint, total, (int)n, No, buf[0]);
    NEB_LAUNCH_CHECK();
  }
  int cur = 0;
  for (int j = L - 1; j >= 0; --j) {
    const int in = m->widths[j], o = m->widths[j + 1];
    const T* X = j == 0 ? feats : (const T*)(tape + tl.x[j]);
    const int64_t x_mode = j == 0 ? 0 : (int64_t)n * C * in;
    const int64_t rows = n * C;
    // weight gradient, split over row ranges so that B x tiles x splits
    // covers the SMs about twice (in 256-thread equivalents)
    const bool narrow = o <= 32 && in <= 32;
    const int wt = narrow ? 32 : 64;
    const int tiles = (int)(ceil_div(o, wt) * ceil_div(in, wt));
    const int64_t target = narrow ? 8 * sms : 2 * sms;
    int splits = (int)std::max<int64_t>(1, std::min<int64_t>(kMaxWgradSplits,
                                                             ceil_div(target, (int64_t)tiles * B)));
    splits = (int)std::min<int64_t>(splits, ceil_div(rows, kWgRows));
    const int64_t per = ceil_div(ceil_div(rows, splits), kWgRows) * kWgRows;
    splits = (int)ceil_div(rows, per);
    bool wg_done = false;
    if constexpr (sizeof(T) == 4) {
      if (gemm_compute()) {
        // gW[b] [o][in] = sum_r Abar_b[r][o] X_b[r][in]: column-major gW^T = X^T Abar
        int st = tc_sgemm_batched(s, CUBLAS_OP_N, CUBLAS_OP_T, in, o, rows, 1.f, X, in, x_mode,
                                  buf[cur], o, rows * o, accumulate ? 1.f : 0.f, (float*)gW[j],
                                  in, (int64_t)o * in, B, "tc_mode_weight_grad");
        if (st) return st;
        wg_done = true;
      }
    }
    if (!wg_done) {
      {
        KernelScope ks("mode_weight_grad", s, 2.0 * B * rows * (double)o * in,
                       (double)B * rows * (o + in) * sizeof(T));
        int st = narrow ? run_mode_wgrad<T, 32>(dev, dim3(tiles, B, splits), buf[cur], X, x_mode,
                                                  rows, o, in, per, part, s)
                        : run_mode_wgrad<T, 64>(dev, dim3(tiles, B, splits), buf[cur], X, x_mode,
                                                  rows, o, in, per, part, s);
        if (st) return st;
      }
      {
        const int64_t per_split = (int64_t)B * o * in;
        KernelScope ks("mode_weight_grad_reduce", s, 0, (double)splits * per_split * sizeof(T));
        mode_wgrad_reduce<T><<<(int)std::min<int64_t>(ceil_div(per_split, 256), 4096), 256, 0,
                               s>>>(part, splits, per_split, accumulate, (T*)gW[j]);
        NEB_LAUNCH_CHECK();
      }
    }
    {
      KernelScope ks("mode_bias_grad", s, 0, (double)B * n * o * sizeof(T));
      mode_bias<T, C><<<B, 32 * kBiasWarps, 0, s>>>(buf[cur], (int)n, o, accumulate,
                                                    (T*)gb[j]);
      NEB_LAUNCH_CHECK();
    }
    if (j == 0) break;
    // data gradient through W_j and the sine-jet transpose of layer j - 1
    const T* W = (const T*)Wv[j] + (int64_t)start * o * in;
    const T* pre = (const T*)(tape + tl.pre[j - 1]);
    const double om = j - 1 == 0 ? m->omega_first : m->omega_hidden;
    int st = launch_mode_gemm<T, DIM, ORD, EPI_REVERSE>(
        buf[cur], (int64_t)n * C * o, W, (int64_t)o * in, nullptr, 0, nullptr, pre, nullptr,
        buf[cur ^ 1], (int64_t)n * C * in, B, (int)n, o, in, om, s, "mode_layer_bwd_data");
    if (st) return st;
    cur ^= 1;
  }
  return NEB_OK;
}

#define NEB_MODES_DISPATCH(m, FN, ...)                                                  \
  ((m)->precision == NEB_PREC_FP64                                                     \
       ? ((m)->dim == 2 ? ((m)->order == 1 ? FN<double, 2, 1>(__VA_ARGS__)             \
                                           : FN<double, 2, 2>(__VA_ARGS__))            \
                        : ((m)->order == 1 ? FN<double, 3, 1>(__VA_ARGS__)             \
                                           : FN<double, 3, 2>(__VA_ARGS__)))           \
       : ((m)->dim == 2 ? ((m)->order == 1 ? FN<float, 2, 1>(__VA_ARGS__)              \
                                           : FN<float, 2, 2>(__VA_ARGS__))             \
                        : ((m)->order == 1 ? FN<float, 3, 1>(__VA_ARGS__)              \
                                           : FN<float, 3, 2>(__VA_ARGS__))))

template <typename T, int DIM, int ORD>
int modes_forward_d(const neb_modes* m, int start, int B, const void* const* W,
                    const void* const* b, const void* feats, const void* env, int64_t n,
                    void* tape, void* out, cudaStream_t s, bool eval = false) {
  return modes_forward_t<T, DIM, ORD>(m, start, B, W, b, (const T*)feats, (const T*)env, n,
                                      (char*)tape, (T*)out, s, eval);
}

size_t eval_scratch_bytes(const neb_modes* m, int B, int64_t n) {
  return 2 * a256((size_t)B * n * mode_channels(m) * max_width(m) * esize(m));
}

template <typename T, int DIM, int ORD>
int modes_backward_d(const neb_modes* m, int start, int B, const void* const* W, const void* feats,
                     const void* env, int64_t n, const void* tape, const void* adjoint,
                     void* const* gW, void* const* gb, int accumulate, void* ws, cudaStream_t s) {
  return modes_backward_t<T, DIM, ORD>(m, start, B, W, (const T*)feats, (const T*)env, n,
                                       (const char*)tape, (const T*)adjoint, gW, gb, accumulate,
                                       (char*)ws, s);
}

}  // namespace
}  // namespace neb

using namespace neb;

extern "C" size_t neb_modes_tape_bytes(const neb_modes* m, int n_block, int64_t n_points) {
  if (check_modes(m) || n_block <= 0 || n_points <= 0) return 0;
  return mode_tape(m, n_block, n_points).total;
}

extern "C" size_t neb_modes_workspace_bytes(const neb_modes* m, int n_block, int64_t n_points) {
  if (check_modes(m) || n_block <= 0 || n_points <= 0) return 0;
  return mode_ws(m, n_block, n_points).total;
}

extern "C" int neb_modes_forward(const neb_modes* m, int start, int stop, const void* const* W,
                                 const void* const* b, const void* features,
                                 const void* envelope, int64_t n_points, void* tape,
                                 size_t tape_bytes, void* out, neb_stream_t stream) {
  int st = check_modes(m);
  if (st) return st;
  GemmScope gemm(m->precision);
  NEB_REQUIRE(0 <= start && start < stop && stop <= m->n_modes,
              "neb_modes_forward: modes [%d, %d) outside [0, %d)", start, stop, m->n_modes);
  NEB_REQUIRE(n_points > 0 && n_points <= (1 << 30) && W && b && features && out,
              "neb_modes_forward: bad arguments");
  for (int j = 0; j < m->n_layers; ++j)
    NEB_REQUIRE(W[j] && b[j], "neb_modes_forward: null parameters of layer %d", j);
  const int B = stop - start;
  NEB_REQUIRE(B <= 65535, "neb_modes_forward: at most 65535 modes per call");
  if (mode_tape(m, B, n_points).total > 0 && (!tape || tape_bytes < mode_tape(m, B, n_points).total)) {
    set_error("neb_modes_forward: tape smaller than neb_modes_tape_bytes");
    return NEB_ERR_WORKSPACE;
  }
  if (m->order == 3) {
    NEB_REQUIRE(!envelope, "neb_modes_forward: third-order jets take the identity envelope");
    return m->precision == NEB_PREC_FP64
               ? modes_forward_d<double, 2, 3>(m, start, B, W, b, features, envelope, n_points,
                                               tape, out, (cudaStream_t)stream)
               : modes_forward_d<float, 2, 3>(m, start, B, W, b, features, envelope, n_points,
                                              tape, out, (cudaStream_t)stream);
  }
  return NEB_MODES_DISPATCH(m, modes_forward_d, m, start, B, W, b, features, envelope, n_points,
                            tape, out, (cudaStream_t)stream);
}

extern "C" size_t neb_modes_eval_scratch_bytes(const neb_modes* m, int n_block,
                                               int64_t n_points) {
  if (check_modes(m) || n_block <= 0 || n_points <= 0) return 0;
  return eval_scratch_bytes(m, n_block, n_points);
}

extern "C" int neb_modes_forward_eval(const neb_modes* m, int start, int stop,
                                      const void* const* W, const void* const* b,
                                      const void* features, const void* envelope,
                                      int64_t n_points, void* scratch, size_t scratch_bytes,
                                      void* out, neb_stream_t stream) {
  int st = check_modes(m);
  if (st) return st;
  GemmScope gemm(m->precision);
  NEB_REQUIRE(0 <= start && start < stop && stop <= m->n_modes,
              "neb_modes_forward_eval: modes [%d, %d) outside [0, %d)", start, stop, m->n_modes);
  NEB_REQUIRE(n_points > 0 && n_points <= (1 << 30) && W && b && features && out,
              "neb_modes_forward_eval: bad arguments");
  for (int j = 0; j < m->n_layers; ++j)
    NEB_REQUIRE(W[j] && b[j], "neb_modes_forward_eval: null parameters of layer %d", j);
  const int B = stop - start;
  NEB_REQUIRE(B <= 65535, "neb_modes_forward_eval: at most 65535 modes per call");
  if (!scratch || scratch_bytes < eval_scratch_bytes(m, B, n_points)) {
    set_error("neb_modes_forward_eval: scratch smaller than neb_modes_eval_scratch_bytes");
    return NEB_ERR_WORKSPACE;
  }
  cudaStream_t s = (cudaStream_t)stream;
  if (m->order == 3) {
    NEB_REQUIRE(!envelope, "neb_modes_forward_eval: third-order jets take the identity envelope");
    return m->precision == NEB_PREC_FP64
               ? modes_forward_d<double, 2, 3>(m, start, B, W, b, features, envelope, n_points,
                                               scratch, out, s, true)
               : modes_forward_d<float, 2, 3>(m, start, B, W, b, features, envelope, n_points,
                                              scratch, out, s, true);
  }
  return NEB_MODES_DISPATCH(m, modes_forward_d, m, start, B, W, b, features, envelope, n_points,
                            scratch, out, s, true);
}

extern "C" int neb_modes_backward(const neb_modes* m, int start, int stop, const void* const* W,
                                  const void* features, const void* envelope, int64_t n_points,
                                  const void* tape, const void* adjoint, void* const* gW,
                                  void* const* gb, int accumulate, void* workspace,
                                  size_t workspace_bytes, neb_stream_t stream) {
  int st = check_modes(m);
  if (st) return st;
  GemmScope gemm(m->precision);
  NEB_REQUIRE(0 <= start && start < stop && stop <= m->n_modes,
              "neb_modes_backward: modes [%d, %d) outside [0, %d)", start, stop, m->n_modes);
  NEB_REQUIRE(n_points > 0 && n_points <= (1 << 30) && W && features && adjoint && gW && gb,
              "neb_modes_backward: bad arguments");
  NEB_REQUIRE(m->n_layers == 1 || tape, "neb_modes_backward: null tape");
  for (int j = 0; j < m->n_layers; ++j)
    NEB_REQUIRE(W[j] && gW[j] && gb[j], "neb_modes_backward: null pointer at layer %d", j);
  const int B = stop - start;
  NEB_REQUIRE(B <= 65535, "neb_modes_backward: at most 65535 modes per call");
  if (!workspace || workspace_bytes < mode_ws(m, B, n_points).total) {
    set_error("neb_modes_backward: workspace smaller than neb_modes_workspace_bytes");
    return NEB_ERR_WORKSPACE;
  }
  NEB_REQUIRE(m->order <= 2, "neb_modes_backward: third-order jets are forward only");
  return NEB_MODES_DISPATCH(m, modes_backward_d, m, start, B, W, features, envelope, n_points,
                            tape, adjoint, gW, gb, accumulate, workspace, (cudaStream_t)stream);
}

extern "C" int neb_velocity_fields(int precision, const void* out, int start, int stop,
                                   int64_t n_points, int n_modes, void* U, void* D,
                                   neb_stream_t stream) {
  NEB_REQUIRE(precision == NEB_PREC_FP32 || precision == NEB_PREC_FP64,
              "neb_velocity_fields: FP32 or FP64");
  NEB_REQUIRE(out && U && D && n_points > 0 && 0 <= start && start < stop && stop <= n_modes,
              "neb_velocity_fields: bad arguments");
  const int B = stop - start;
  const int64_t total = (int64_t)B * n_points;
  cudaStream_t s = (cudaStream_t)stream;
  const size_t es = precision == NEB_PREC_FP64 ? 8 : 4;
  KernelScope ks("velocity_fields", s, 0, (double)total * (30 + 12) * es);
  if (precision == NEB_PREC_FP64)
    velocity_fields<double><<<(int)ceil_div(total, 256), 256, 0, s>>>(
        (const double*)out, B, (int)n_points, n_modes, start, (double*)U, (double*)D);
  else
    velocity_fields<float><<<(int)ceil_div(total, 256), 256, 0, s>>>(
        (const float*)out, B, (int)n_points, n_modes, start, (float*)U, (float*)D);
  NEB_LAUNCH_CHECK();
  return NEB_OK;
}

extern "C" int neb_velocity_lift(int precision, const void* GU, const void* GD, int start,
                                 int stop, int64_t n_points, int n_modes, void* adjoint,
                                 neb_stream_t stream) {
  NEB_REQUIRE(precision == NEB_PREC_FP32 || precision == NEB_PREC_FP64,
              "neb_velocity_lift: FP32 or FP64");
  NEB_REQUIRE(GU && GD && adjoint && n_points > 0 && 0 <= start && start < stop &&
                  stop <= n_modes,
              "neb_velocity_lift: bad arguments");
  const int B = stop - start;
  const int64_t total = (int64_t)B * n_points;
  cudaStream_t s = (cudaStream_t)stream;
  const size_t es = precision == NEB_PREC_FP64 ? 8 : 4;
  KernelScope ks("velocity_lift", s, 0, (double)total * (30 + 12) * es);
  if (precision == NEB_PREC_FP64)
    velocity_lift<double><<<(int)ceil_div(total, 256), 256, 0, s>>>(
        (const double*)GU, (const double*)GD, B, (int)n_points, n_modes, start, (double*)adjoint);
  else
    velocity_lift<float><<<(int)ceil_div(total, 256), 256, 0, s>>>(
        (const float*)GU, (const float*)GD, B, (int)n_points, n_modes, start, (float*)adjoint);
  NEB_LAUNCH_CHECK();
  return NEB_OK;
}

extern "C" int neb_potential_fields(int precision, const void* out, int start, int stop,
                                    int64_t n_points, int n_modes, void* V, void* G,
                                    neb_stream_t stream) {
  NEB_REQUIRE(precision == NEB_PREC_FP32 || precision == NEB_PREC_FP64,
              "neb_potential_fields: FP32 or FP64");
  NEB_REQUIRE(out && V && G && n_points > 0 && 0 <= start && start < stop && stop <= n_modes,
              "neb_potential_fields: bad arguments");
  const int B = stop - start;
  const int64_t total = (int64_t)B * n_points;
  cudaStream_t s = (cudaStream_t)stream;
  const size_t es = precision == NEB_PREC_FP64 ? 8 : 4;
  KernelScope ks("potential_fields", s, 0, (double)total * 6 * es);
  if (precision == NEB_PREC_FP64)
    potential_fields<double><<<(int)ceil_div(total, 256), 256, 0, s>>>(
        (const double*)out, B, (int)n_points, n_modes, start, (double*)V, (double*)G);
  else
    potential_fields<float><<<(int)ceil_div(total, 256), 256, 0, s>>>(
        (const float*)out, B, (int)n_points, n_modes, start, (float*)V, (float*)G);
  NEB_LAUNCH_CHECK();
  return NEB_OK;
}

extern "C" int neb_potential_lift(int precision, const void* dV, const void* dG, int start,
                                  int stop, int64_t n_points, int n_modes, void* adjoint,
                                  neb_stream_t stream) {
  NEB_REQUIRE(precision == NEB_PREC_FP32 || precision == NEB_PREC_FP64,
              "neb_potential_lift: FP32 or FP64");
  NEB_REQUIRE(dV && dG && adjoint && n_points > 0 && 0 <= start && start < stop &&
                  stop <= n_modes,
              "neb_potential_lift: bad arguments");
  const int B = stop - start;
  const int64_t total = (int64_t)B * n_points;
  cudaStream_t s = (cudaStream_t)stream;
  const size_t es = precision == NEB_PREC_FP64 ? 8 : 4;
  KernelScope ks("potential_lift", s, 0, (double)total * 6 * es);
  if (precision == NEB_PREC_FP64)
    potential_lift<double><<<(int)ceil_div(total, 256), 256, 0, s>>>(
        (const double*)dV, (const double*)dG, B, (int)n_points, n_modes, start, (double*)adjoint);
  else
    potential_lift<float><<<(int)ceil_div(total, 256), 256, 0, s>>>(
        (const float*)dV, (const float*)dG, B, (int)n_points, n_modes, start, (float*)adjoint);
  NEB_LAUNCH_CHECK();
  return NEB_OK;
}

extern "C" int neb_column_center(int precision, int64_t rows, int K, void* A,
                                 neb_stream_t stream) {
  NEB_REQUIRE(precision == NEB_PREC_FP32 || precision == NEB_PREC_FP64,
              "neb_column_center: FP32 or FP64");
  NEB_REQUIRE(A && rows > 0 && K > 0, "neb_column_center: bad arguments");
  cudaStream_t s = (cudaStream_t)stream;
  KernelScope ks("column_center", s, 0, 2.0 * rows * K * (precision == NEB_PREC_FP64 ? 8 : 4));
  if (precision == NEB_PREC_FP64) column_center<double><<<K, 256, 0, s>>>((double*)A, rows, K);
  else column_center<float><<<K, 256, 0, s>>>((float*)A, rows, K);
  NEB_LAUNCH_CHECK();
  return NEB_OK;
}

extern "C" size_t neb_modes_adam_workspace_bytes(int n_modes) {
  return n_modes <= 0 ? 0 : a256((size_t)n_modes * sizeof(double)) +
                                a256((size_t)3 * n_modes * sizeof(double));
}

extern "C" int neb_modes_adam(int dtype, int n_modes, int n_tensors, void* const* params,
                              void* const* exp_avg, void* const* exp_avg_sq,
                              const void* const* grads, const int64_t* sizes, int* step_counter,
                              int steps_per_mode, const int* active, const int* gate, double lr,
                              double clip, double* norms_out, int* committed_out, void* workspace,
                              size_t workspace_bytes, neb_stream_t stream) {
  NEB_REQUIRE(dtype == 0 || dtype == 1, "neb_modes_adam: dtype must be 0 (float) or 1 (double)");
  NEB_REQUIRE(n_modes > 0 && n_tensors > 0 && n_tensors <= kMaxAdamTensors,
              "neb_modes_adam: 1..%d tensors of at least one mode", kMaxAdamTensors);
  NEB_REQUIRE(params && exp_avg && exp_avg_sq && grads && sizes && step_counter,
              "neb_modes_adam: bad arguments");
  if (!workspace || workspace_bytes < neb_modes_adam_workspace_bytes(n_modes)) {
    set_error("neb_modes_adam: workspace too small");
    return NEB_ERR_WORKSPACE;
  }
  ModeAdamTable mt{};
  mt.t.n = n_tensors;
  mt.t.off[0] = 0;
  for (int i = 0; i < n_tensors; ++i) {
    NEB_REQUIRE(params[i] && exp_avg[i] && exp_avg_sq[i] && grads[i] && sizes[i] > 0 &&
                    sizes[i] % n_modes == 0,
                "neb_modes_adam: tensor %d must hold a whole number of modes", i);
    mt.t.p[i] = params[i];
    mt.t.m[i] = exp_avg[i];
    mt.t.v[i] = exp_avg_sq[i];
    mt.t.g[i] = grads[i];
    mt.t.off[i + 1] = mt.t.off[i] + sizes[i];
    mt.per_mode[i] = sizes[i] / n_modes;
  }
  cudaStream_t s = (cudaStream_t)stream;
  char* ws = (char*)workspace;
  double* norm2 = (double*)ws;
  double* par = (double*)(ws + a256((size_t)n_modes * sizeof(double)));
  const int64_t total = mt.t.off[n_tensors];
  const double es = dtype == 0 ? 4.0 : 8.0;
  {
    KernelScope ks("mode_adam_norms", s, 0, total * es);
    if (dtype == 0) mode_adam_norms<float><<<n_modes, 256, 0, s>>>(mt, norm2);
    else mode_adam_norms<double><<<n_modes, 256, 0, s>>>(mt, norm2);
    NEB_LAUNCH_CHECK();
  }
  {
    KernelScope ks("mode_adam_update", s, 0, total * es * 7, 2);
    mode_adam_finalize<<<1, 256, 0, s>>>(norm2, gate, active, n_modes, clip, lr, step_counter,
                                         steps_per_mode ? 1 : 0, norms_out, committed_out, par);
    NEB_LAUNCH_CHECK();
    const int blocks = (int)std::min<int64_t>(std::max<int64_t>(ceil_div(total, 256), 1), 2048);
    if (dtype == 0) mode_adam_update<float><<<blocks, 256, 0, s>>>(mt, par);
    else mode_adam_update<double><<<blocks, 256, 0, s>>>(mt, par);
    NEB_LAUNCH_CHECK();
  }
  return NEB_OK;
}
