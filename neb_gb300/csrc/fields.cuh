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
