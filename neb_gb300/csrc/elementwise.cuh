// Elementwise kernels: input features with jets, the Adam transaction, and
// small helpers of the spectral stage.
#pragma once
#include "neb_common.cuh"

namespace neb {

// Feature parameters passed by value (hole centres of the multihole domain).
struct FeatureParams {
  int n;
  double v[64];
};

// One thread per (point, feature): writes the C jet channels of the feature.
// Periodic features with FP32 outputs reduce the phase in turns in FP64
// (t = k s / period, t - rint(t): four FP64 operations, exact to ~1e-16
// turns) and evaluate sin / cos (pi * 2 (t - rint t)) in FP32; inv_period =
// 1 / period comes from the host, so no FP64 division runs per element.
template <typename T, int C>
__global__ void features_kernel(int kind, int n_freq, double period, double inv_period,
                                FeatureParams prm, const double* __restrict__ pts, int64_t n,
                                int F, T* __restrict__ X0) {
  const int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int64_t total = n * F;
  if (idx >= total) return;
  int64_t p;
  int f;
  if (total < ((int64_t)1 << 31)) {
    const int i32 = (int)idx;
    p = i32 / F;
    f = i32 - (int)p * F;
  } else {
    p = idx / F;
    f = (int)(idx % F);
  }
  if constexpr (sizeof(T) == 4 && C == 4) {
    if (kind == NEB_FEAT_PERIODIC) {
      // for axis in (x, y), for k = 1..n_freq, (sin, cos) of 2 pi k s / period
      const int axis = f / (2 * n_freq), r = f % (2 * n_freq), k = r / 2 + 1;
      const double t = (double)k * (pts[p * 2 + axis] * inv_period);
      const float red2 = 2.f * (float)(t - rint(t));  // in [-1, 1]
      float sn, cs;
      sincospif(red2, &sn, &cs);
      const float w = (float)(6.283185307179586 * inv_period) * (float)k;
      const float v = (r & 1) ? cs : sn;
      float* o = X0 + (p * C) * (int64_t)F + f;
      o[0] = v;
      o[(int64_t)(1 + axis) * F] = (r & 1) ? -w * sn : w * cs;
      o[(int64_t)(2 - axis) * F] = 0.f;
      o[(int64_t)3 * F] = -w * w * v;
      return;
    }
  }
  double out[C];
#pragma unroll
  for (int c = 0; c < C; ++c) out[c] = 0.0;
  if (kind == NEB_FEAT_PERIODIC) {
    int axis = f / (2 * n_freq), r = f % (2 * n_freq), k = r / 2 + 1;
    double w = 2.0 * 3.14159265358979323846 * k / period;
    double sn, cs;
    sincos(w * pts[p * 2 + axis], &sn, &cs);
    double v = (r & 1) ? cs : sn;
    out[0] = v;
    out[1 + axis] = (r & 1) ? -w * sn : w * cs;
    out[3] = -w * w * v;
  } else if (kind == NEB_FEAT_MULTIHOLE) {
    double x = pts[p * 2], y = pts[p * 2 + 1];
    if (f < 2) {
      out[0] = f == 0 ? x : y;
      out[1 + f] = 1.0;
    } else {
      double dx = x - prm.v[2 * (f - 2)], dy = y - prm.v[2 * (f - 2) + 1];
      double r2 = dx * dx + dy * dy;
      out[0] = atan2(dy, dx);
      out[1] = -dy / r2;
      out[2] = dx / r2;
    }
  } else {  // raw coordinates
    out[0] = pts[p * 3 + f];
    out[1 + f] = 1.0;
  }
#pragma unroll
  for (int c = 0; c < C; ++c) X0[(p * C + c) * (int64_t)F + f] = (T)out[c];
}

constexpr int kMaxAdamTensors = 40;
struct AdamTable {
  int n;
  void* p[kMaxAdamTensors];
  void* m[kMaxAdamTensors];
  void* v[kMaxAdamTensors];
  const void* g[kMaxAdamTensors];
  int64_t off[kMaxAdamTensors + 1];
};

__device__ __forceinline__ int adam_find(const AdamTable& t, int64_t i) {
  int k = 0;
  while (k + 1 < t.n && i >= t.off[k + 1]) ++k;
  return k;
}

// acc[0] += sum g^2 (double), flag[0] |= any non-finite.  Zeroed by the host.
template <typename T>
__global__ void adam_norm(AdamTable t, double* __restrict__ acc, int* __restrict__ flag) {
  __shared__ double red[32];
  double s = 0.0;
  int bad = 0;
  const int64_t total = t.off[t.n];
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total;
       i += (int64_t)gridDim.x * blockDim.x) {
    int k = adam_find(t, i);
    double g = (double)static_cast<const T*>(t.g[k])[i - t.off[k]];
    if (!isfinite(g)) bad = 1;
    s += g * g;
  }
  for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  bad = __any_sync(0xffffffffu, bad);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  if (bad && (threadIdx.x & 31) == 0) atomicOr(flag, 1);
  __syncthreads();
  if (threadIdx.x < 32) {
    double v = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.0;
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (threadIdx.x == 0) atomicAdd(acc, v);
  }
}

// The transaction's scalars, once: global norm, commit decision (finite
// gradients, a positive norm and, when given, a zero status word of the
// objective -- the physical-validity gate of hardcoded_backend.py:2184-2277,
// 3677-3721), the clip
// scale min(1, clip / norm) (scal[0] = 0 means "do not commit") and the bias
// corrections of step t = committed steps + 1 (scal[1] = lr / (1 - beta1^t),
// scal[2] = 1 / (1 - beta2^t)).  The committed-step count comes from the
// device counter *steps when given (advanced here only on commit, as the
// reference advances its epoch only after a committed update,
// native_cupy_core.py:157-170), else from the host argument.
static __global__ void adam_finalize(const double* __restrict__ acc, const int* __restrict__ flag,
                                     double clip, int host_steps, int* __restrict__ steps,
                                     const int* __restrict__ gate, double lr, double beta1,
                                     double beta2, double* __restrict__ norm_out,
                                     int* __restrict__ committed_out, double* __restrict__ scal) {
  const double norm = sqrt(acc[0]);
  const bool ok = (flag[0] == 0) && isfinite(norm) && norm > 0.0 && (!gate || *gate == 0);
  if (norm_out) *norm_out = norm;
  if (committed_out) *committed_out = ok ? 1 : 0;
  const double t = (double)(steps ? *steps : host_steps) + 1.0;
  scal[0] = ok ? fmin(1.0, clip / fmax(norm, 1e-30)) : 0.0;
  scal[1] = lr / (1.0 - pow(beta1, t));
  scal[2] = 1.0 / (1.0 - pow(beta2, t));
  if (steps && ok) *steps += 1;
}

// Masked Adam update with the scalars of adam_finalize (the bias
// corrections are formed once there, so no per-element double-precision
// work remains for the FP32 form).
template <typename T>
__global__ void adam_update(AdamTable t, const double* __restrict__ scal, T b1, T b2, T eps) {
  const double sc = scal[0];
  if (sc == 0.0) return;
  const T scale = (T)sc, lr_c1 = (T)scal[1], inv_c2 = (T)scal[2];
  const T ob1 = T(1) - b1, ob2 = T(1) - b2;
  const int64_t total = t.off[t.n];
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total;
       i += (int64_t)gridDim.x * blockDim.x) {
    int k = adam_find(t, i);
    int64_t j = i - t.off[k];
    T* p = static_cast<T*>(t.p[k]);
    T* m = static_cast<T*>(t.m[k]);
    T* v = static_cast<T*>(t.v[k]);
    T g = static_cast<const T*>(t.g[k])[j] * scale;
    T mn = b1 * m[j] + ob1 * g;
    T vn = b2 * v[j] + ob2 * g * g;
    m[j] = mn;
    v[j] = vn;
    p[j] -= lr_c1 * mn / (sqrt(vn * inv_c2) + eps);
  }
}

// Objective weights applied to eigenvector columns (column-major V, m x m):
// out[i + j m] = V[i + j m] * f_j with f = c (G_S) or f = c * lam (G_M).
static __global__ void scale_columns(const double* __restrict__ V, const double* __restrict__ c,
                              const double* __restrict__ lam, int m, double* __restrict__ out) {
  int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (idx >= (int64_t)m * m) return;
  int j = (int)(idx / m);
  double f = c[j] * (lam ? lam[j] : 1.0);
  out[idx] = V[idx] * f;
}

// loss = sum_k c_k lam_k; also flags a non-finite loss into info when the
// solver reported success.
static __global__ void weighted_sum(const double* __restrict__ c, const double* __restrict__ lam, int m,
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
    if (info && *info == 0 && !isfinite(v)) *info = -1;
  }
}

template <typename S, typename D>
__global__ void convert_kernel(const S* __restrict__ src, D* __restrict__ dst, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    dst[i] = (D)src[i];
}

}  // namespace neb
