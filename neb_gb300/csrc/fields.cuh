// Velocity / vorticity fields of the output jets and their transpose (the
// direct route: K x K Grams assembled from the fields of every mode).
//
// Field layout F: [n][C][K], the jet channel count C of the network, so the
// jet GEMM and row-sum kernels take it unchanged.
//   2D (C = 4), psi_k scalar:      F1 = u_x = d_y psi, F2 = u_y = -d_x psi,
//                                  F3 = omega = -lap psi, F0 = 0.
//   3D (C = 10), A_k = (psi_3k, psi_3k+1, psi_3k+2):
//                                  F1..F3 = u = curl A,
//                                  F4..F6 = omega = curl u = grad div A - lap A,
//                                  F0, F7..F9 = 0.
// (velocity_trace_jet2.py:93-98 velocity / vorticity; velocity/core.py:32-38
// lift; the 2D sign convention of evaluate_large_comparison.py:35-38.)
#pragma once
#include "neb_common.cuh"

namespace neb {

// Output jets Psi [n][C][Ko] -> fields F [n][C][K]; one thread per (point, mode).
template <typename T, int C>
__global__ void fields_extract(const T* __restrict__ psi, T* __restrict__ F, int64_t n, int K,
                               int Ko) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n * K) return;
  const int64_t p = i / K;
  const int k = (int)(i % K);
  const T* ps = psi + p * C * (int64_t)Ko;
  T* f = F + p * C * (int64_t)K + k;
  if constexpr (C == 4) {
    f[0] = T(0);
    f[K] = ps[2 * (int64_t)Ko + k];
    f[2 * K] = -ps[(int64_t)Ko + k];
    f[3 * K] = -ps[3 * (int64_t)Ko + k];
  } else {
    // g(comp, axis) = d_axis A_comp; h(comp, a, b) = d_a d_b A_comp
    auto g = [&](int comp, int axis) { return ps[(1 + axis) * (int64_t)Ko + 3 * k + comp]; };
    auto h = [&](int comp, int a, int b) {
      int s = a <= b ? hess_slot(a, b) : hess_slot(b, a);
      return ps[(4 + s) * (int64_t)Ko + 3 * k + comp];
    };
    f[0] = T(0);
    f[K] = g(2, 1) - g(1, 2);
    f[2 * K] = g(0, 2) - g(2, 0);
    f[3 * K] = g(1, 0) - g(0, 1);
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      T w = T(0);
#pragma unroll
      for (int b = 0; b < 3; ++b) w += h(b, a, b) - h(a, b, b);
      f[(4 + a) * K] = w;
    }
    f[7 * K] = T(0);
    f[8 * K] = T(0);
    f[9 * K] = T(0);
  }
}

// Transpose of fields_extract: field adjoints Fb [n][C][K] -> output-jet
// adjoints Pb [n][C][Ko] (every entry written; the value channel is zero).
template <typename T, int C>
__global__ void fields_adjoint(const T* __restrict__ Fb, T* __restrict__ Pb, int64_t n, int K,
                               int Ko) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n * K) return;
  const int64_t p = i / K;
  const int k = (int)(i % K);
  const T* fb = Fb + p * C * (int64_t)K + k;
  T* pb = Pb + p * C * (int64_t)Ko;
  if constexpr (C == 4) {
    pb[k] = T(0);
    pb[(int64_t)Ko + k] = -fb[2 * K];
    pb[2 * (int64_t)Ko + k] = fb[K];
    pb[3 * (int64_t)Ko + k] = -fb[3 * K];
  } else {
    T a[C][3];
#pragma unroll
    for (int c = 0; c < C; ++c)
#pragma unroll
      for (int j = 0; j < 3; ++j) a[c][j] = T(0);
    const T u0 = fb[K], u1 = fb[2 * K], u2 = fb[3 * K];
    // velocity: u0 = g(2,1) - g(1,2), u1 = g(0,2) - g(2,0), u2 = g(1,0) - g(0,1)
    a[1 + 1][2] += u0;
    a[1 + 2][1] -= u0;
    a[1 + 2][0] += u1;
    a[1 + 0][2] -= u1;
    a[1 + 0][1] += u2;
    a[1 + 1][0] -= u2;
    // vorticity: omega_a = sum_b h(b, a, b) - h(a, b, b)
#pragma unroll
    for (int ax = 0; ax < 3; ++ax) {
      const T w = fb[(4 + ax) * K];
#pragma unroll
      for (int b = 0; b < 3; ++b) {
        int s1 = ax <= b ? hess_slot(ax, b) : hess_slot(b, ax);
        a[4 + s1][b] += w;
        a[4 + hess_slot(b, b)][ax] -= w;
      }
    }
#pragma unroll
    for (int c = 0; c < C; ++c)
#pragma unroll
      for (int j = 0; j < 3; ++j) pb[c * (int64_t)Ko + 3 * k + j] = a[c][j];
  }
}

}  // namespace neb

namespace neb {

// Envelope product of the output jets of the shared network (Leibniz rule
// on the jet channels; reference: native_cupy_core.py product1,
// velocity_trace_jet2.py product).  e: [n][C] one scalar jet per point;
// x, y: [n][C][W].  2D (C = 4, value / d_x / d_y / Laplacian):
//   lap(e x) = e lap x + x lap e + 2 grad e . grad x;
// 3D (C = 10, value / gradient / Hessian xx xy xz yy yz zz):
//   H(e x) = e H x + x H e + grad e grad x^T + grad x grad e^T.
// REVERSE: y = adjoint of x given the adjoint x of the product.
template <typename T, int C, bool REVERSE>
__global__ void envelope_jets(const T* __restrict__ e, const T* __restrict__ x,
                              T* __restrict__ y, int64_t n, int W) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n * W) return;
  const int64_t p = i / W;
  const int k = (int)(i % W);
  T ev[C], a[C], b[C];
#pragma unroll
  for (int c = 0; c < C; ++c) {
    ev[c] = e[p * C + c];
    a[c] = x[(p * C + c) * W + k];
  }
  if constexpr (C == 4) {
    if constexpr (!REVERSE) {
      b[0] = ev[0] * a[0];
      b[1] = ev[0] * a[1] + ev[1] * a[0];
      b[2] = ev[0] * a[2] + ev[2] * a[0];
      b[3] = ev[0] * a[3] + ev[3] * a[0] + T(2) * (ev[1] * a[1] + ev[2] * a[2]);
    } else {
      b[0] = ev[0] * a[0] + ev[1] * a[1] + ev[2] * a[2] + ev[3] * a[3];
      b[1] = ev[0] * a[1] + T(2) * ev[1] * a[3];
      b[2] = ev[0] * a[2] + T(2) * ev[2] * a[3];
      b[3] = ev[0] * a[3];
    }
  } else {
    if constexpr (!REVERSE) {
      b[0] = ev[0] * a[0];
#pragma unroll
      for (int d = 0; d < 3; ++d) b[1 + d] = ev[0] * a[1 + d] + ev[1 + d] * a[0];
#pragma unroll
      for (int i2 = 0; i2 < 3; ++i2)
#pragma unroll
        for (int j2 = i2; j2 < 3; ++j2) {
          const int q = 4 + hess_slot(i2, j2);
          b[q] = ev[0] * a[q] + ev[q] * a[0] + ev[1 + i2] * a[1 + j2] + ev[1 + j2] * a[1 + i2];
        }
    } else {
      b[0] = ev[0] * a[0];
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        b[0] += ev[1 + d] * a[1 + d];
        b[1 + d] = ev[0] * a[1 + d];
      }
#pragma unroll
      for (int i2 = 0; i2 < 3; ++i2)
#pragma unroll
        for (int j2 = i2; j2 < 3; ++j2) {
          const int q = 4 + hess_slot(i2, j2);
          b[0] += ev[q] * a[q];
          b[1 + i2] += ev[1 + j2] * a[q];
          b[1 + j2] += ev[1 + i2] * a[q];
          b[q] = ev[0] * a[q];
        }
    }
  }
#pragma unroll
  for (int c = 0; c < C; ++c) y[(p * C + c) * W + k] = b[c];
}

}  // namespace neb
