// Shared definitions of the neb_gb300 CUDA library: status handling, the
// tanh derivative ladder and the jet chain rule / transpose used by every
// kernel epilogue.
//
// Jet layout in device memory: one row per (point, channel), rows of a point
// adjacent, i.e. a [n_points][C][width] row-major array.  2D: C = 4 channels
// (value, d/dx, d/dy, Laplacian).  3D: C = 10 channels (value, d/dx, d/dy,
// d/dz, Hessian xx, xy, xz, yy, yz, zz).
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include <cstdio>
#include <cmath>
#include "neb_gb300.h"

namespace neb {

void set_error(const char* fmt, ...);

#define NEB_CUDA_CHECK(expr)                                                   \
  do {                                                                         \
    cudaError_t _e = (expr);                                                   \
    if (_e != cudaSuccess) {                                                   \
      ::neb::set_error("%s:%d %s: %s", __FILE__, __LINE__, #expr,              \
                       cudaGetErrorString(_e));                                \
      return NEB_ERR_CUDA;                                                     \
    }                                                                          \
  } while (0)

#define NEB_LAUNCH_CHECK()                                                     \
  do {                                                                         \
    cudaError_t _e = cudaGetLastError();                                       \
    if (_e != cudaSuccess) {                                                   \
      ::neb::set_error("%s:%d kernel launch: %s", __FILE__, __LINE__,          \
                       cudaGetErrorString(_e));                                \
      return NEB_ERR_CUDA;                                                     \
    }                                                                          \
  } while (0)

#define NEB_REQUIRE(cond, ...)                                                 \
  do {                                                                         \
    if (!(cond)) {                                                             \
      ::neb::set_error(__VA_ARGS__);                                           \
      return NEB_ERR_ARG;                                                      \
    }                                                                          \
  } while (0)

// Hessian slot of the ordered pair (i, j), i <= j, in (xx, xy, xz, yy, yz, zz).
__host__ __device__ constexpr int hess_slot(int i, int j) {
  return i == 0 ? j : (i == 1 ? 2 + j : 5);
}

// tanh and its first three derivatives, written through e = exp(-2|z|) so that
// s1 = sech^2 z keeps full relative accuracy when |t| is close to 1:
//   t  = sign(z) (1 - e) / (1 + e),   s1 = 4 e / (1 + e)^2,
//   s2 = -2 t s1,                      s3 = -2 s1 (s1 - 2 t^2).
template <typename T>
__device__ __forceinline__ void tanh_ladder(T z, T& t, T& s1, T& s2, T& s3) {
  T a = z < T(0) ? -z : z;
  T e;
  if constexpr (sizeof(T) == 8) e = exp(-2.0 * a); else e = expf(-2.0f * a);
  T inv = T(1) / (T(1) + e);
  T tt = (T(1) - e) * inv;
  t = z < T(0) ? -tt : tt;
  s1 = T(4) * e * inv * inv;
  s2 = T(-2) * t * s1;
  s3 = T(-2) * s1 * (s1 - T(2) * t * t);
}

// Jet chain rule through tanh, in place: z[C] -> y[C].
template <int C, typename T>
__device__ __forceinline__ void jet_act_forward(T* z) {
  T t, s1, s2, s3;
  tanh_ladder(z[0], t, s1, s2, s3);
  if constexpr (C == 4) {
    T g2 = z[1] * z[1] + z[2] * z[2];
    z[0] = t;
    z[3] = s1 * z[3] + s2 * g2;
    z[1] *= s1;
    z[2] *= s1;
  } else {
    T g[3] = {z[1], z[2], z[3]};
    z[0] = t;
#pragma unroll
    for (int a = 0; a < 3; ++a) z[1 + a] = s1 * g[a];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = i; j < 3; ++j) {
        int k = 4 + hess_slot(i, j);
        z[k] = s1 * z[k] + s2 * g[i] * g[j];
      }
  }
}

// Transpose of jet_act_forward: given the pre-activation jet z[C] and the
// adjoint yb[C] of the activation, overwrite yb with the adjoint of z.
template <int C, typename T>
__device__ __forceinline__ void jet_act_backward(const T* z, T* yb) {
  T t, s1, s2, s3;
  tanh_ladder(z[0], t, s1, s2, s3);
  if constexpr (C == 4) {
    T g2 = z[1] * z[1] + z[2] * z[2];
    T zb = yb[0] * s1 + (yb[1] * z[1] + yb[2] * z[2]) * s2 + yb[3] * (s2 * z[3] + s3 * g2);
    T l2 = T(2) * s2 * yb[3];
    yb[0] = zb;
    yb[1] = s1 * yb[1] + l2 * z[1];
    yb[2] = s1 * yb[2] + l2 * z[2];
    yb[3] = s1 * yb[3];
  } else {
    T zb = yb[0] * s1;
    T gb[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      zb += yb[1 + a] * z[1 + a] * s2;
      gb[a] = s1 * yb[1 + a];
    }
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = i; j < 3; ++j) {
        int k = 4 + hess_slot(i, j);
        T hb = yb[k];
        zb += hb * (s2 * z[k] + s3 * z[1 + i] * z[1 + j]);
        gb[i] += s2 * hb * z[1 + j];
        gb[j] += s2 * hb * z[1 + i];
        yb[k] = s1 * hb;
      }
    yb[0] = zb;
#pragma unroll
    for (int a = 0; a < 3; ++a) yb[1 + a] = gb[a];
  }
}

inline int64_t ceil_div(int64_t a, int64_t b) { return (a + b - 1) / b; }

// Kernel instrumentation: every launch of this library goes through a
// KernelScope, which counts it and, while timing is enabled
// (neb_timing_begin / neb_timing_end), brackets it with CUDA events on the
// launching stream and records its algorithmic flops and bytes.
// Per-device caches (function attributes set, SM counts, side streams) are
// arrays indexed by the device ordinal.
constexpr int kMaxDevices = 64;

// The current device and its SM count (cached per device).
inline int device_sms(int* dev, int* sms) {
  static int count[kMaxDevices] = {};
  NEB_CUDA_CHECK(cudaGetDevice(dev));
  NEB_REQUIRE(*dev >= 0 && *dev < kMaxDevices, "device index %d", *dev);
  if (!count[*dev])
    NEB_CUDA_CHECK(cudaDeviceGetAttribute(&count[*dev], cudaDevAttrMultiProcessorCount, *dev));
  *sms = count[*dev];
  return NEB_OK;
}

// Joins a side stream back into the main stream when it leaves scope, so an
// early error return still leaves the side work ordered before whatever the
// caller enqueues next on the main stream.  Disarmed once the normal path
// has joined explicitly.
struct SideStreamJoin {
  cudaStream_t main, side;
  cudaEvent_t ev;
  bool armed;
  ~SideStreamJoin() {
    if (armed && cudaEventRecord(ev, side) == cudaSuccess) cudaStreamWaitEvent(main, ev, 0);
  }
};

void timing_record(const char* name, cudaStream_t s, double flops, double bytes, bool begin);
void count_launch(int n = 1);

struct KernelScope {
  const char* name;
  cudaStream_t stream;
  double flops, bytes;
  int launches;
  KernelScope(const char* n, cudaStream_t s, double f = 0, double b = 0, int nl = 1)
      : name(n), stream(s), flops(f), bytes(b), launches(nl) {
    timing_record(name, stream, flops, bytes, true);
  }
  ~KernelScope() {
    count_launch(launches);
    timing_record(name, stream, flops, bytes, false);
  }
};

}  // namespace neb
