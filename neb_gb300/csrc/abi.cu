// extern "C" entry points of the jet MLP, the Grams and the reverse pass.
// Precision dispatch: NEB_PREC_FP32 / NEB_PREC_FP64 run the SIMT kernels;
// NEB_PREC_BF16X3 runs the tcgen05 kernels of tc_path.cu; NEB_PREC_TF32 /
// NEB_PREC_BF16X9 run the FP32 SIMT path with its layer GEMMs on the tensor
// cores through cuBLAS (plain GEMMs; the jet epilogues stay ours).
#include <cublas_v2.h>
#include <cmath>
#include <cstdarg>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>
#include "simt_kernels.cuh"
#include "elementwise.cuh"
#include "tc_path.cuh"
#include "tc_blas.cuh"
#include "fields.cuh"

namespace neb {

int& gemm_compute() {
  thread_local int compute = 0;
  return compute;
}

thread_local std::string g_last_error;

// ---------------------------------------------------------------- timing
namespace {
struct TimingEntry {
  const char* name;
  cudaEvent_t a, b;
  double flops, bytes;
};
struct TimingState {
  bool enabled = false;
  std::vector<TimingEntry> entries;
  std::vector<size_t> open;  // entries whose scope has not ended (scopes nest)
  std::vector<cudaEvent_t> pool;
  size_t used = 0;
  cudaEvent_t get() {
    if (used == pool.size()) {
      cudaEvent_t e;
      cudaEventCreate(&e);
      pool.push_back(e);
    }
    return pool[used++];
  }
};
TimingState g_timing;
unsigned long long g_launches = 0;
}  // namespace

void count_launch(int n) { __atomic_add_fetch(&g_launches, (unsigned long long)n, __ATOMIC_RELAXED); }

void timing_record(const char* name, cudaStream_t s, double flops, double bytes, bool begin) {
  if (!g_timing.enabled) return;
  cudaEvent_t e = g_timing.get();
  cudaEventRecord(e, s);
  if (begin) {
    g_timing.open.push_back(g_timing.entries.size());
    g_timing.entries.push_back({name, e, nullptr, flops, bytes});
  } else if (!g_timing.open.empty()) {
    g_timing.entries[g_timing.open.back()].b = e;
    g_timing.open.pop_back();
  }
}

void set_error(const char* fmt, ...) {
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_last_error = buf;
}

namespace {

size_t a256(size_t x) { return (x + 255) & ~size_t(255); }

// ------------------------------------------------ tensor-core layer GEMMs
cublasHandle_t g_layer_blas[kMaxDevices] = {};
std::mutex g_layer_blas_mutex;

int layer_blas(cudaStream_t s, cublasHandle_t* h) {
  int dev = 0;
  NEB_CUDA_CHECK(cudaGetDevice(&dev));
  NEB_REQUIRE(dev >= 0 && dev < kMaxDevices, "device index %d", dev);
  {
    std::lock_guard<std::mutex> lock(g_layer_blas_mutex);
    if (!g_layer_blas[dev] && cublasCreate(&g_layer_blas[dev]) != CUBLAS_STATUS_SUCCESS) {
      set_error("cublasCreate failed");
      return NEB_ERR_CUDA;
    }
  }
  *h = g_layer_blas[dev];
  if (cublasSetStream(*h, s) != CUBLAS_STATUS_SUCCESS) {
    set_error("cublasSetStream failed");
    return NEB_ERR_CUDA;
  }
  return NEB_OK;
}

// Row-major C [rows][ldc] = alpha op(A) op(B) + beta C through cublasGemmEx
// in FP32 storage with the scope's tensor-core compute type, expressed in
// cuBLAS's column-major terms by the caller.
int tc_sgemm(cudaStream_t s, cublasOperation_t ta, cublasOperation_t tb, int m, int64_t n,
             int64_t k, float alpha, const float* A, int lda, const float* B, int ldb, float beta,
             float* C, int ldc, const char* name) {
  return tc_sgemm_batched(s, ta, tb, m, n, k, alpha, A, lda, 0, B, ldb, 0, beta, C, ldc, 0, 1,
                          name);
}

// Bias on the value channel and the tanh jet of a pre-activation Z already
// formed by a GEMM: Z [n*C][ldo] (updated in place), Y [n*C][ldo].
template <int C>
__global__ void jet_act_epilogue(float* __restrict__ Z, const float* __restrict__ bias,
                                 float* __restrict__ Y, int64_t n, int N, int ldo) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n * N;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t p = e / N;
    const int o = (int)(e % N);
    float z[C];
#pragma unroll
    for (int c = 0; c < C; ++c) z[c] = Z[(p * C + c) * ldo + o];
    if (bias) {
      z[0] += bias[o];
      Z[p * C * ldo + o] = z[0];
    }
    if (Y) {
      jet_act_forward<C>(z);
#pragma unroll
      for (int c = 0; c < C; ++c) Y[(p * C + c) * ldo + o] = z[c];
    }
  }
}

// The tanh-jet transpose with the pre-activation Zprev, in place on
// Out [n*C][N].
template <int C>
__global__ void jet_act_transpose(const float* __restrict__ Zprev, float* __restrict__ Out,
                                  int64_t n, int N) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n * N;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t p = e / N;
    const int i = (int)(e % N);
    float z[C], yb[C];
#pragma unroll
    for (int c = 0; c < C; ++c) {
      z[c] = Zprev[(p * C + c) * N + i];
      yb[c] = Out[(p * C + c) * N + i];
    }
    jet_act_backward<C>(z, yb);
#pragma unroll
    for (int c = 0; c < C; ++c) Out[(p * C + c) * N + i] = yb[c];
  }
}

int ew_grid(int64_t n) { return (int)std::min<int64_t>(std::max<int64_t>(ceil_div(n, 256), 1), 65535); }

int net_channels(const neb_net* net) { return net->dim == 2 ? 4 : 10; }

int check_net(const neb_net* net) {
  NEB_REQUIRE(net != nullptr, "null neb_net");
  NEB_REQUIRE(net->dim == 2 || net->dim == 3, "neb_net.dim must be 2 or 3 (got %d)", net->dim);
  NEB_REQUIRE(net->n_hidden >= 1 && net->n_hidden <= NEB_MAX_HIDDEN,
              "neb_net.n_hidden must be in [1, %d] (got %d)", NEB_MAX_HIDDEN, net->n_hidden);
  for (int l = 0; l <= net->n_hidden + 1; ++l)
    NEB_REQUIRE(net->widths[l] > 0 && net->widths[l] <= 65536, "neb_net.widths[%d] = %d invalid", l,
                net->widths[l]);
  NEB_REQUIRE(net->precision == NEB_PREC_FP32 || net->precision == NEB_PREC_FP64 ||
                  net->precision == NEB_PREC_BF16X3 || net->precision == NEB_PREC_TF32 ||
                  net->precision == NEB_PREC_BF16X9,
              "unknown precision %d", net->precision);
  NEB_REQUIRE(net->gram == NEB_GRAM_PLAIN || net->gram == NEB_GRAM_COMPENSATED,
              "unknown Gram accumulation %d", net->gram);
  if (net->dim == 3) NEB_REQUIRE(net->widths[net->n_hidden + 1] % 3 == 0,
                                 "3D output width must be 3 K");
  return NEB_OK;
}

size_t master_size(const neb_net* net) { return net->precision == NEB_PREC_FP64 ? 8 : 4; }

// Tape: X_0 | Z_1 | X_1 | ... | Z_L | X_L, each [n][C][w] in storage format.
// X_l storage: FP32 -> float, FP64 -> double, BF16X3 -> hi and lo bf16 planes.
// Z_l storage: master type.
struct TapeLayout {
  size_t x_off[NEB_MAX_HIDDEN + 1];
  size_t z_off[NEB_MAX_HIDDEN + 1];
  size_t total;
};

TapeLayout tape_layout(const neb_net* net, int64_t n) {
  TapeLayout t{};
  if (net->precision == NEB_PREC_BF16X3) {
    t.total = tc_tape_bytes(net, n, t.x_off, t.z_off);
    return t;
  }
  const int C = net_channels(net);
  const size_t es = master_size(net);
  size_t off = 0;
  for (int l = 0; l <= net->n_hidden; ++l) {
    size_t elems = (size_t)n * C * net->widths[l];
    if (l > 0) {
      t.z_off[l] = off;
      off += a256(elems * es);
    }
    t.x_off[l] = off;
    off += a256(elems * es);  // bf16 hi + lo planes = 4 bytes per element
  }
  t.total = off;
  return t;
}

int64_t chunk_points(int64_t n) {
  int64_t c = ceil_div(n, 32);
  if (c < 256) c = 256;
  return c;
}

int max_width(const neb_net* net) {
  int m = 0;
  for (int l = 0; l <= net->n_hidden + 1; ++l) m = m > net->widths[l] ? m : net->widths[l];
  return m;
}

// Workspace: [Zbar ping][Zbar pong][partials][bias partials][G casts][tc scratch]
struct WsLayout {
  size_t zb0, zb1, part, partb, gcast, fld, psib, tc, total;
};

// Modes of the output layer: K = widths[L+1] scalar potentials in 2D,
// widths[L+1] / 3 vector potentials in 3D.
int n_modes(const neb_net* net) {
  const int Ko = net->widths[net->n_hidden + 1];
  return net->dim == 2 ? Ko : Ko / 3;
}

WsLayout ws_layout(const neb_net* net, int64_t n) {
  WsLayout w{};
  if (net->precision == NEB_PREC_BF16X3) {
    w.total = a256(tc_workspace_bytes(net, n));
    return w;
  }
  const int C = net_channels(net);
  const size_t es = master_size(net);
  const int mw = max_width(net);
  const int64_t chunks = ceil_div(n, chunk_points(n));
  size_t zb = a256((size_t)n * C * mw * es);
  size_t part = a256((size_t)chunks * mw * mw * sizeof(double));
  size_t partb = a256((size_t)chunks * mw * sizeof(double));
  size_t gcast = a256((size_t)2 * mw * mw * es);
  // direct route: fields F [n][C][K] and output-jet adjoints [n][C][Ko]
  size_t fld = a256((size_t)n * C * n_modes(net) * es);
  size_t psib = a256((size_t)n * C * net->widths[net->n_hidden + 1] * es);
  w.zb0 = 0;
  w.zb1 = zb;
  w.part = 2 * zb;
  w.partb = w.part + part;
  w.gcast = w.partb + partb;
  w.fld = w.gcast + gcast;
  w.psib = w.fld + fld;
  w.tc = w.psib + psib;
  w.total = w.tc;
  return w;
}

template <typename T, int C>
int launch_fwd(const T* X, const T* W, const T* b, T* Z, T* Y, int64_t n, int K, int N, int ldo,
               cudaStream_t s) {
  if constexpr (sizeof(T) == 4) {
    if (gemm_compute()) {
      // row-major Z [n C][ldo] = X [n C][K] W^T: column-major Z^T = W^T(K x N)^T X^T
      int st = tc_sgemm(s, CUBLAS_OP_T, CUBLAS_OP_N, N, n * C, K, 1.f, W, K, X, K, 0.f, Z, ldo,
                        Y ? "tc_layer_fwd" : "tc_output_fwd");
      if (st) return st;
      if (b || Y) {
        KernelScope ks("jet_act_epilogue", s, 0, (double)n * C * N * (Y ? 12 : 8));
        jet_act_epilogue<C><<<ew_grid(n * N), 256, 0, s>>>(Z, b, Y, n, N, ldo);
        NEB_LAUNCH_CHECK();
      }
      return NEB_OK;
    }
  }
  using Tl = simt::Tile<C>;
  dim3 grid((unsigned)ceil_div(N, simt::kBN), (unsigned)ceil_div(n * C, Tl::BM));
  KernelScope ks(Y ? "simt_jet_layer_fwd" : "simt_jet_output_fwd", s, 2.0 * n * C * K * N,
                 (double)n * C * (K + (Y ? 2 : 1) * N) * sizeof(T));
  if (Y)
    simt::jet_gemm_fwd<T, C, true><<<grid, simt::kThreads, 0, s>>>(X, W, b, Z, Y, n, K, N, ldo);
  else
    simt::jet_gemm_fwd<T, C, false><<<grid, simt::kThreads, 0, s>>>(X, W, b, Z, Y, n, K, N, ldo);
  NEB_LAUNCH_CHECK();
  return NEB_OK;
}

template <typename T, int C, int MAP>
int launch_bwd(const T* A, const T* B0, const T* B1, const T* rowscale, T scale, const T* Zprev,
               T* Out, int64_t n, int K, int N, cudaStream_t s) {
  if constexpr (sizeof(T) == 4 && MAP == 0) {
    if (gemm_compute() && !rowscale) {
      // row-major Out [n C][N] = scale A [n C][K] B0 [K][N]
      int st = tc_sgemm(s, CUBLAS_OP_N, CUBLAS_OP_N, N, n * C, K, (float)scale, B0, N, A, K, 0.f,
                        Out, N, "tc_layer_bwd_data");
      if (st) return st;
      if (Zprev) {
        KernelScope ks("jet_act_transpose", s, 0, (double)n * C * N * 12);
        jet_act_transpose<C><<<ew_grid(n * N), 256, 0, s>>>(Zprev, Out, n, N);
        NEB_LAUNCH_CHECK();
      }
      return NEB_OK;
    }
  }
  using Tl = simt::Tile<C>;
  dim3 grid((unsigned)ceil_div(N, simt::kBN), (unsigned)ceil_div(n * C, Tl::BM));
  KernelScope ks(MAP ? "simt_gram_adjoint_bwd" : "simt_jet_layer_bwd_data", s,
                 2.0 * n * (MAP == 0 ? C : (MAP == 1 ? 3 : 6)) * K * N,
                 (double)n * C * (K + (Zprev ? 2 : 1) * N) * sizeof(T));
  if (Zprev)
    simt::jet_gemm_bwd<T, C, MAP, true>
        <<<grid, simt::kThreads, 0, s>>>(A, B0, B1, rowscale, scale, Zprev, Out, n, K, N);
  else
    simt::jet_gemm_bwd<T, C, MAP, false>
        <<<grid, simt::kThreads, 0, s>>>(A, B0, B1, rowscale, scale, Zprev, Out, n, K, N);
  NEB_LAUNCH_CHECK();
  return NEB_OK;
}

// Out[m][n] = scale * sum_{p, c in chans} w_p P[r][m] Q[r][n] -> OutT
template <typename T, int C, typename OutT>
int launch_rowsum(const T* P, int ldp, const T* Q, int ldq, const T* w, simt::ChanSet chans,
                  int64_t n, int M, int N, bool sym, double scale, double* part, OutT* out,
                  cudaStream_t s, int accumulate = 0, bool comp = false) {
  if constexpr (sizeof(T) == 4 && sizeof(OutT) == 4) {
    if (gemm_compute() && !sym && !w && chans.n == C) {
      // every channel row of every point: row-major out [M][N] = scale sum_r P[r][M]^T Q[r][N]
      return tc_sgemm(s, CUBLAS_OP_N, CUBLAS_OP_T, N, M, n * C, (float)scale, Q, ldq, P, ldp,
                      accumulate ? 1.f : 0.f, (float*)out, N, "tc_weight_grad");
    }
  }
  const int64_t cp = chunk_points(n);
  const int chunks = (int)ceil_div(n, cp);
  const int mt = (int)ceil_div(M, 128), nt = (int)ceil_div(N, simt::kBN);
  const int tiles = sym ? nt * (nt + 1) / 2 : mt * nt;
  if (sym) NEB_REQUIRE(M == N, "symmetric rowsum needs M == N");
  dim3 grid(tiles, chunks);
  {
    const bool c32 = comp && sizeof(T) == 4;
    KernelScope ks(sym ? (c32 ? "simt_gram_compensated" : "simt_gram") : "simt_weight_grad", s,
                   (sym ? 1.0 : 2.0) * n * chans.n * (double)M * N,
                   (double)n * chans.n * (M + N) * sizeof(T));
    if constexpr (sizeof(T) == 4) {
      if (c32)
        simt::rowsum_gemm<T, C, true><<<grid, simt::kThreads, 0, s>>>(
            P, ldp, Q, ldq, w, chans, n, cp, M, N, sym ? 1 : 0, part);
    }
    if (!c32)
      simt::rowsum_gemm<T, C><<<grid, simt::kThreads, 0, s>>>(P, ldp, Q, ldq, w, chans, n, cp, M,
                                                              N, sym ? 1 : 0, part);
    NEB_LAUNCH_CHECK();
  }
  int64_t total = (int64_t)M * N;
  int blocks = (int)std::min<int64_t>(ceil_div(total, 256), 4096);
  {
    KernelScope ks("reduce_chunks", s, 0, (double)chunks * total * 8);
    simt::reduce_chunks<OutT><<<blocks, 256, 0, s>>>(part, chunks, M, N, sym ? 1 : 0, scale,
                                                      accumulate, out);
    NEB_LAUNCH_CHECK();
  }
  return NEB_OK;
}

template <typename T, int C, typename OutT>
int launch_bias(const T* Zb, int64_t n, int N, double* partb, OutT* out, cudaStream_t s,
                int accumulate = 0) {
  const int64_t cp = chunk_points(n);
  const int chunks = (int)ceil_div(n, cp);
  dim3 grid((unsigned)ceil_div(N, 128), chunks);
  {
    KernelScope ks("bias_grad", s, 0, (double)n * N * sizeof(T));
    simt::bias_partial<T, C><<<grid, 128, 0, s>>>(Zb, n, cp, N, partb);
    NEB_LAUNCH_CHECK();
  }
  int blocks = (int)ceil_div(N, 256);
  {
    KernelScope ks("reduce_chunks", s, 0, (double)chunks * N * 8);
    simt::reduce_chunks<OutT><<<blocks, 256, 0, s>>>(partb, chunks, 1, N, 0, 1.0, accumulate, out);
    NEB_LAUNCH_CHECK();
  }
  return NEB_OK;
}

// ---------------------------------------------------------------- forward
template <typename T, int C>
int forward_simt(const neb_net* net, const void* const* W, const void* const* b,
                 const void* feats, int64_t n, void* tape, cudaStream_t s) {
  TapeLayout tl = tape_layout(net, n);
  char* tp = (char*)tape;
  NEB_CUDA_CHECK(cudaMemcpyAsync(tp + tl.x_off[0], feats,
                                 (size_t)n * C * net->widths[0] * sizeof(T),
                                 cudaMemcpyDeviceToDevice, s));
  for (int l = 1; l <= net->n_hidden; ++l) {
    const T* X = (const T*)(tp + tl.x_off[l - 1]);
    T* Z = (T*)(tp + tl.z_off[l]);
    T* Y = (T*)(tp + tl.x_off[l]);
    int st = launch_fwd<T, C>(X, (const T*)W[l - 1], (const T*)b[l - 1], Z, Y, n,
                              net->widths[l - 1], net->widths[l], net->widths[l], s);
    if (st) return st;
  }
  return NEB_OK;
}

// ------------------------------------------------------- hidden backward
// Zbar of layer `l` is in `zb`; walk down to layer 1, writing gW/gb.
template <typename T, int C>
int backward_layers(const neb_net* net, const void* const* W, int top, T* zb, T* zb_other,
                    const char* tp, const TapeLayout& tl, void* const* gW, void* const* gb,
                    double* part, double* partb, int64_t n, cudaStream_t s, int accumulate = 0) {
  simt::ChanSet all{C, {0, 1, 2, 3, 4, 5, 6, 7, 8, 9}};
  for (int l = top; l >= 1; --l) {
    const int in = net->widths[l - 1], out = net->widths[l];
    const T* X = (const T*)(tp + tl.x_off[l - 1]);
    // gW_l[o][i] = sum_r zb[r][o] X[r][i];  gb_l[o] = sum_p zb[p, value][o]
    int st = launch_rowsum<T, C, T>(zb, out, X, in, nullptr, all, n, out, in, false, 1.0, part,
                                    (T*)gW[l - 1], s, accumulate);
    if (st) return st;
    st = launch_bias<T, C, T>(zb, n, out, partb, (T*)gb[l - 1], s, accumulate);
    if (st) return st;
    if (l > 1) {
      const T* Zp = (const T*)(tp + tl.z_off[l - 1]);
      st = launch_bwd<T, C, 0>(zb, (const T*)W[l - 1], nullptr, nullptr, T(1), Zp, zb_other, n, out,
                               in, s);
      if (st) return st;
      T* t = zb;
      zb = zb_other;
      zb_other = t;
    }
  }
  return NEB_OK;
}

template <typename T, int C>
int backward_hidden_simt(const neb_net* net, const void* const* W, const double* GMh,
                         const double* GSh, const void* qw, int64_t n, const void* tape,
                         void* const* gW, void* const* gb, void* ws, cudaStream_t s,
                         int accumulate) {
  const int L = net->n_hidden, H = net->widths[L];
  TapeLayout tl = tape_layout(net, n);
  WsLayout wl = ws_layout(net, n);
  char* w = (char*)ws;
  const char* tp = (const char*)tape;
  T* zb0 = (T*)(w + wl.zb0);
  T* zb1 = (T*)(w + wl.zb1);
  T* gM = (T*)(w + wl.gcast);
  T* gS = gM + (size_t)H * H;
  int64_t hh = (int64_t)H * H;
  int blocks = (int)std::min<int64_t>(ceil_div(hh, 256), 4096);
  {
    KernelScope ks("convert", s, 0, (double)hh * 2 * (8 + sizeof(T)));
    convert_kernel<double, T><<<blocks, 256, 0, s>>>(GMh, gM, hh);
    NEB_LAUNCH_CHECK();
  }
  {
    KernelScope ks("convert", s, 0, (double)hh * (8 + sizeof(T)));
    convert_kernel<double, T><<<blocks, 256, 0, s>>>(GSh, gS, hh);
    NEB_LAUNCH_CHECK();
  }
  // hbar = 2 w (h G) per channel, then the tanh-jet transpose of layer L
  const T* HL = (const T*)(tp + tl.x_off[L]);
  const T* ZL = (const T*)(tp + tl.z_off[L]);
  int st = launch_bwd<T, C, 1>(HL, gM, gS, (const T*)qw, T(2), ZL, zb0, n, H, H, s);
  if (st) return st;
  return backward_layers<T, C>(net, W, L, zb0, zb1, tp, tl, gW, gb, (double*)(w + wl.part),
                               (double*)(w + wl.partb), n, s, accumulate);
}

template <typename T, int C>
int backward_output_simt(const neb_net* net, const void* const* W, int start, int stop,
                         const void* psibar, int64_t n, const void* tape, void* const* gW,
                         void* const* gb, void* ws, cudaStream_t s, int accumulate) {
  const int L = net->n_hidden, H = net->widths[L], Ko = stop - start;
  TapeLayout tl = tape_layout(net, n);
  WsLayout wl = ws_layout(net, n);
  char* w = (char*)ws;
  const char* tp = (const char*)tape;
  T* zb0 = (T*)(w + wl.zb0);
  T* zb1 = (T*)(w + wl.zb1);
  double* part = (double*)(w + wl.part);
  double* partb = (double*)(w + wl.partb);
  simt::ChanSet all{C, {0, 1, 2, 3, 4, 5, 6, 7, 8, 9}};
  const T* PB = (const T*)psibar;
  const T* HL = (const T*)(tp + tl.x_off[L]);
  const T* Wout = (const T*)W[L] + (size_t)start * H;
  // output layer gradients for rows [start, stop)
  int st = launch_rowsum<T, C, T>(PB, Ko, HL, H, nullptr, all, n, Ko, H, false, 1.0, part,
                                  (T*)gW[L] + (size_t)start * H, s, accumulate);
  if (st) return st;
  st = launch_bias<T, C, T>(PB, n, Ko, partb, (T*)gb[L] + start, s, accumulate);
  if (st) return st;
  // hbar = psibar W_out[start:stop], then tanh-jet transpose of layer L
  const T* ZL = (const T*)(tp + tl.z_off[L]);
  st = launch_bwd<T, C, 0>(PB, Wout, nullptr, nullptr, T(1), ZL, zb0, n, Ko, H, s);
  if (st) return st;
  return backward_layers<T, C>(net, W, L, zb0, zb1, tp, tl, gW, gb, part, partb, n, s,
                               accumulate);
}

template <typename T, int C>
int hidden_gram_simt(const neb_net* net, const void* qw, int64_t n, const void* tape, double* AM,
                     double* AS, void* ws, cudaStream_t s, int accumulate = 0) {
  const int L = net->n_hidden, H = net->widths[L];
  TapeLayout tl = tape_layout(net, n);
  WsLayout wl = ws_layout(net, n);
  const T* HL = (const T*)((const char*)tape + tl.x_off[L]);
  double* part = (double*)((char*)ws + wl.part);
  simt::ChanSet grad{2, {1, 2}};
  simt::ChanSet lap{1, {3}};
  const bool comp = net->gram == NEB_GRAM_COMPENSATED;
  int st = launch_rowsum<T, C, double>(HL, H, HL, H, (const T*)qw, grad, n, H, H, true, 1.0, part,
                                       AM, s, accumulate, comp);
  if (st) return st;
  return launch_rowsum<T, C, double>(HL, H, HL, H, (const T*)qw, lap, n, H, H, true, 1.0, part, AS,
                                     s, accumulate, comp);
}

// ------------------------------------------------------ direct route
// Output jets Psi = W_out h (no bias: the fields use derivative channels
// only) into psi, then the fields F of every mode.
template <typename T, int C>
int fields_forward_simt(const neb_net* net, const void* Wout, int64_t n, const void* tape,
                        T* psi, T* F, cudaStream_t s) {
  const int L = net->n_hidden, H = net->widths[L], Ko = net->widths[L + 1];
  const int K = n_modes(net);
  TapeLayout tl = tape_layout(net, n);
  const T* HL = (const T*)((const char*)tape + tl.x_off[L]);
  int st = launch_fwd<T, C>(HL, (const T*)Wout, nullptr, psi, nullptr, n, H, Ko, Ko, s);
  if (st) return st;
  const int64_t total = n * K;
  KernelScope ks("fields_extract", s, 0, (double)n * C * (Ko + K) * sizeof(T));
  fields_extract<T, C><<<(unsigned)ceil_div(total, 256), 256, 0, s>>>(psi, F, n, K, Ko);
  NEB_LAUNCH_CHECK();
  return NEB_OK;
}

// M (+)= sum_p w_p u_i . u_j, S (+)= sum_p w_p omega_i . omega_j over the
// modes i, j (K x K, FP64).
template <typename T, int C>
int fields_gram_simt(const neb_net* net, const void* Wout, const void* qw, int64_t n,
                     const void* tape, double* M, double* S, int accumulate, void* ws,
                     cudaStream_t s) {
  WsLayout wl = ws_layout(net, n);
  char* w = (char*)ws;
  T* psi = (T*)(w + wl.zb0);
  T* F = (T*)(w + wl.fld);
  double* part = (double*)(w + wl.part);
  const int K = n_modes(net);
  int st = fields_forward_simt<T, C>(net, Wout, n, tape, psi, F, s);
  if (st) return st;
  simt::ChanSet vel = C == 4 ? simt::ChanSet{2, {1, 2}} : simt::ChanSet{3, {1, 2, 3}};
  simt::ChanSet vor = C == 4 ? simt::ChanSet{1, {3}} : simt::ChanSet{3, {4, 5, 6}};
  const bool comp = net->gram == NEB_GRAM_COMPENSATED;
  st = launch_rowsum<T, C, double>(F, K, F, K, (const T*)qw, vel, n, K, K, true, 1.0, part, M, s,
                                   accumulate, comp);
  if (st) return st;
  return launch_rowsum<T, C, double>(F, K, F, K, (const T*)qw, vor, n, K, K, true, 1.0, part, S,
                                     s, accumulate, comp);
}

// Reverse of fields_gram + objective adjoints G_M, G_S: field adjoints
// Fbar = 2 w F G (velocity rows with G_M, vorticity rows with G_S), their
// transpose to output-jet adjoints, then the output and hidden layers.
template <typename T, int C>
int backward_fields_simt(const neb_net* net, const void* const* W, const double* GM,
                         const double* GS, const void* qw, int64_t n, const void* tape,
                         void* const* gW, void* const* gb, int accumulate, void* ws,
                         cudaStream_t s) {
  const int L = net->n_hidden, Ko = net->widths[L + 1];
  const int K = n_modes(net);
  WsLayout wl = ws_layout(net, n);
  char* w = (char*)ws;
  T* psi = (T*)(w + wl.zb0);
  T* Fb = (T*)(w + wl.zb1);
  T* F = (T*)(w + wl.fld);
  T* Pb = (T*)(w + wl.psib);
  T* gM = (T*)(w + wl.gcast);
  T* gS = gM + (size_t)K * K;
  int st = fields_forward_simt<T, C>(net, W[L], n, tape, psi, F, s);
  if (st) return st;
  const int64_t kk = (int64_t)K * K;
  const int blocks = (int)std::min<int64_t>(ceil_div(kk, 256), 4096);
  {
    KernelScope ks("convert", s, 0, (double)kk * 2 * (8 + sizeof(T)), 2);
    convert_kernel<double, T><<<blocks, 256, 0, s>>>(GM, gM, kk);
    NEB_LAUNCH_CHECK();
    convert_kernel<double, T><<<blocks, 256, 0, s>>>(GS, gS, kk);
    NEB_LAUNCH_CHECK();
  }
  constexpr int MAP = C == 4 ? 1 : 2;
  st = launch_bwd<T, C, MAP>(F, gM, gS, (const T*)qw, T(2), nullptr, Fb, n, K, K, s);
  if (st) return st;
  {
    const int64_t total = n * K;
    KernelScope ks("fields_adjoint", s, 0, (double)n * C * (Ko + K) * sizeof(T));
    fields_adjoint<T, C><<<(unsigned)ceil_div(total, 256), 256, 0, s>>>(Fb, Pb, n, K, Ko);
    NEB_LAUNCH_CHECK();
  }
  return backward_output_simt<T, C>(net, W, 0, Ko, Pb, n, tape, gW, gb, ws, s, accumulate);
}

}  // namespace

int tc_sgemm_batched(cudaStream_t s, cublasOperation_t ta, cublasOperation_t tb, int m,
                     int64_t n, int64_t k, float alpha, const float* A, int lda, int64_t sa,
                     const float* B, int ldb, int64_t sb, float beta, float* C, int ldc,
                     int64_t sc, int batch, const char* name) {
  NEB_REQUIRE(n <= INT32_MAX && k <= INT32_MAX, "%s: %lld x %lld too large for one GEMM", name,
              (long long)n, (long long)k);
  cublasHandle_t h;
  if (int st = layer_blas(s, &h)) return st;
  KernelScope ks(name, s, 2.0 * batch * m * (double)n * k,
                 4.0 * batch * ((double)m * k + (double)n * k + (double)m * n));
  const cublasComputeType_t ct = (cublasComputeType_t)gemm_compute();
  const cublasStatus_t r =
      batch == 1 ? cublasGemmEx(h, ta, tb, m, (int)n, (int)k, &alpha, A, CUDA_R_32F, lda, B,
                                CUDA_R_32F, ldb, &beta, C, CUDA_R_32F, ldc, ct,
                                CUBLAS_GEMM_DEFAULT)
                 : cublasGemmStridedBatchedEx(h, ta, tb, m, (int)n, (int)k, &alpha, A, CUDA_R_32F,
                                              lda, sa, B, CUDA_R_32F, ldb, sb, &beta, C,
                                              CUDA_R_32F, ldc, sc, batch, ct, CUBLAS_GEMM_DEFAULT);
  if (r != CUBLAS_STATUS_SUCCESS) {
    set_error("%s: cuBLAS GEMM failed (status %d)", name, (int)r);
    return NEB_ERR_CUDA;
  }
  return NEB_OK;
}

}  // namespace neb

using namespace neb;

#define NEB_DISPATCH(net, FN, ...)                                                 \
  ((net)->precision == NEB_PREC_FP64                                               \
       ? ((net)->dim == 2 ? FN<double, 4>(__VA_ARGS__) : FN<double, 10>(__VA_ARGS__)) \
       : ((net)->dim == 2 ? FN<float, 4>(__VA_ARGS__) : FN<float, 10>(__VA_ARGS__)))

extern "C" const char* neb_last_error(void) { return g_last_error.c_str(); }

extern "C" unsigned long long neb_kernel_launches(void) {
  return __atomic_load_n(&g_launches, __ATOMIC_RELAXED);
}

extern "C" int neb_timing_begin(void) {
  g_timing.entries.clear();
  g_timing.open.clear();
  g_timing.used = 0;
  g_timing.enabled = true;
  return NEB_OK;
}

extern "C" int neb_timing_end(int max_kernels, char* names, int name_len, int* launches,
                              double* total_ms, double* flops, double* bytes, int* n_kernels) {
  g_timing.enabled = false;
  std::vector<std::string> keys;
  std::vector<int> cnt;
  std::vector<double> ms, fl, by;
  for (auto& e : g_timing.entries) {
    if (!e.b) continue;
    NEB_CUDA_CHECK(cudaEventSynchronize(e.b));
    float t = 0.f;
    NEB_CUDA_CHECK(cudaEventElapsedTime(&t, e.a, e.b));
    size_t k = 0;
    while (k < keys.size() && keys[k] != e.name) ++k;
    if (k == keys.size()) {
      keys.push_back(e.name);
      cnt.push_back(0);
      ms.push_back(0);
      fl.push_back(0);
      by.push_back(0);
    }
    cnt[k] += 1;
    ms[k] += t;
    fl[k] += e.flops;
    by[k] += e.bytes;
  }
  int n = (int)keys.size() < max_kernels ? (int)keys.size() : max_kernels;
  for (int k = 0; k < n; ++k) {
    snprintf(names + (size_t)k * name_len, name_len, "%s", keys[k].c_str());
    launches[k] = cnt[k];
    total_ms[k] = ms[k];
    flops[k] = fl[k];
    bytes[k] = by[k];
  }
  *n_kernels = n;
  g_timing.entries.clear();
  g_timing.open.clear();
  g_timing.used = 0;
  return NEB_OK;
}

extern "C" size_t neb_tape_bytes(const neb_net* net, int64_t n) {
  if (check_net(net) != NEB_OK || n <= 0) return 0;
  return tape_layout(net, n).total;
}

extern "C" size_t neb_workspace_bytes(const neb_net* net, int64_t n) {
  if (check_net(net) != NEB_OK || n <= 0) return 0;
  return ws_layout(net, n).total;
}

extern "C" int neb_features(const neb_net* net, int kind, int n_freq, const double* params,
                            int n_params, const double* points, int64_t n, void* feats,
                            neb_stream_t stream) {
  int st = check_net(net);
  if (st) return st;
  NEB_REQUIRE(n > 0 && points && feats, "neb_features: bad arguments");
  const int F = net->widths[0];
  double period = 0.0;
  if (kind == NEB_FEAT_PERIODIC) {
    NEB_REQUIRE(net->dim == 2 && n_freq > 0 && F == 4 * n_freq && n_params >= 1 && params,
                "periodic features need dim 2, widths[0] == 4 n_freq and params[0] = period");
    // the period is read on the host: params is a host array here
    period = params[0];
    NEB_REQUIRE(period > 0, "period must be positive");
  } else if (kind == NEB_FEAT_MULTIHOLE) {
    NEB_REQUIRE(net->dim == 2 && n_params % 2 == 0 && F == 2 + n_params / 2,
                "multihole features need widths[0] == 2 + holes and 2 params per hole");
  } else if (kind == NEB_FEAT_RAW3D) {
    NEB_REQUIRE(net->dim == 3 && F == 3, "raw 3D features need dim 3 and widths[0] == 3");
  } else {
    NEB_REQUIRE(false, "unknown feature kind %d", kind);
  }
  cudaStream_t s = (cudaStream_t)stream;
  // hole centres (host array) travel to the kernel by value
  FeatureParams dprm{};
  if (kind == NEB_FEAT_MULTIHOLE) {
    NEB_REQUIRE(n_params <= 64, "at most 32 holes");
    dprm.n = n_params;
    for (int i = 0; i < n_params; ++i) dprm.v[i] = params[i];
  }
  const double inv_period = kind == NEB_FEAT_PERIODIC ? 1.0 / period : 0.0;
  int64_t total = n * F;
  int blocks = (int)ceil_div(total, 256);
  KernelScope ks("features", s, 0, (double)total * net_channels(net) * master_size(net));
  if (net->precision == NEB_PREC_FP64) {
    if (net->dim == 2)
      features_kernel<double, 4><<<blocks, 256, 0, s>>>(
          kind, n_freq, period, inv_period, dprm, points, n, F, (double*)feats);
    else
      features_kernel<double, 10><<<blocks, 256, 0, s>>>(
          kind, n_freq, period, inv_period, dprm, points, n, F, (double*)feats);
  } else {
    if (net->dim == 2)
      features_kernel<float, 4><<<blocks, 256, 0, s>>>(
          kind, n_freq, period, inv_period, dprm, points, n, F, (float*)feats);
    else
      features_kernel<float, 10><<<blocks, 256, 0, s>>>(
          kind, n_freq, period, inv_period, dprm, points, n, F, (float*)feats);
  }
  NEB_LAUNCH_CHECK();
  return NEB_OK;
}

extern "C" int neb_forward(const neb_net* net, const void* const* W, const void* const* b,
                           const void* feats, int64_t n, void* tape, void* ws, size_t ws_bytes,
                           neb_stream_t stream) {
  int st = check_net(net);
  if (st) return st;
  GemmScope gemm(net->precision);
  NEB_REQUIRE(n > 0 && W && b && feats && tape, "neb_forward: bad arguments");
  for (int l = 0; l < net->n_hidden; ++l) NEB_REQUIRE(W[l] && b[l], "neb_forward: null W/b[%d]", l);
  cudaStream_t s = (cudaStream_t)stream;
  if (net->precision == NEB_PREC_BF16X3) {
    if (ws_bytes < ws_layout(net, n).total || !ws) {
      set_error("neb_forward: workspace too small");
      return NEB_ERR_WORKSPACE;
    }
    WsLayout wl = ws_layout(net, n);
    TapeLayout tl = tape_layout(net, n);
    TcTape tt;
    for (int l = 0; l <= net->n_hidden; ++l) {
      tt.x[l] = (char*)tape + tl.x_off[l];
      tt.z[l] = (char*)tape + tl.z_off[l];
    }
    return tc_forward(net, (const float* const*)W, (const float* const*)b, (const float*)feats, n,
                      tt, (char*)ws + wl.tc, s);
  }
  return NEB_DISPATCH(net, forward_simt, net, W, b, feats, n, tape, s);
}

template <typename T, int C>
static int output_simt(const neb_net* net, const void* Wout, const void* bout, int start, int stop,
                       int64_t n, const void* tape, void* psi, cudaStream_t s) {
  const int L = net->n_hidden, H = net->widths[L];
  TapeLayout tl = tape_layout(net, n);
  const T* HL = (const T*)((const char*)tape + tl.x_off[L]);
  return launch_fwd<T, C>(HL, (const T*)Wout + (size_t)start * H,
                          bout ? (const T*)bout + start : nullptr, (T*)psi, nullptr, n, H,
                          stop - start, stop - start, s);
}

extern "C" int neb_output(const neb_net* net, const void* Wout, const void* bout, int start,
                          int stop, int64_t n, const void* tape, void* psi, neb_stream_t stream) {
  int st = check_net(net);
  if (st) return st;
  GemmScope gemm(net->precision);
  const int K = net->widths[net->n_hidden + 1];
  NEB_REQUIRE(n > 0 && Wout && tape && psi && 0 <= start && start < stop && stop <= K,
              "neb_output: bad arguments");
  if (net->precision == NEB_PREC_BF16X3)
    return tc_output(net, (const float*)Wout, (const float*)bout, start, stop, n, tape, psi,
                     (cudaStream_t)stream);
  return NEB_DISPATCH(net, output_simt, net, Wout, bout, start, stop, n, tape, psi,
                      (cudaStream_t)stream);
}

namespace neb {
namespace {
template <typename T, int C>
int envelope_simt(const void* e, const void* x, void* y, int64_t n, int W, int reverse,
                  cudaStream_t s) {
  const int64_t total = n * W;
  KernelScope ks("envelope_jets", s, 0, 2.0 * total * C * sizeof(T));
  if (reverse)
    envelope_jets<T, C, true><<<(unsigned)ceil_div(total, 256), 256, 0, s>>>(
        (const T*)e, (const T*)x, (T*)y, n, W);
  else
    envelope_jets<T, C, false><<<(unsigned)ceil_div(total, 256), 256, 0, s>>>(
        (const T*)e, (const T*)x, (T*)y, n, W);
  NEB_LAUNCH_CHECK();
  return NEB_OK;
}
}  // namespace
}  // namespace neb

extern "C" int neb_envelope_product(const neb_net* net, const void* envelope, int64_t n, int width,
                                    const void* x, void* y, int reverse, neb_stream_t stream) {
  int st = check_net(net);
  if (st) return st;
  NEB_REQUIRE(envelope && x && y && n > 0 && width > 0, "neb_envelope_product: bad arguments");
  NEB_REQUIRE(net->precision != NEB_PREC_BF16X3,
              "neb_envelope_product: output jets are FP32 or FP64 (the evaluation network)");
  return NEB_DISPATCH(net, envelope_simt, envelope, x, y, n, width, reverse, (cudaStream_t)stream);
}

extern "C" int neb_hidden_gram(const neb_net* net, const void* qw, int64_t n, const void* tape,
                               double* AM, double* AS, int accumulate, void* ws, size_t ws_bytes,
                               neb_stream_t stream) {
  int st = check_net(net);
  if (st) return st;
  GemmScope gemm(net->precision);
  NEB_REQUIRE(net->dim == 2, "neb_hidden_gram: 2D scalar potential only");
  NEB_REQUIRE(n > 0 && qw && tape && AM && AS, "neb_hidden_gram: bad arguments");
  if (ws_bytes < ws_layout(net, n).total || !ws) {
    set_error("neb_hidden_gram: workspace too small");
    return NEB_ERR_WORKSPACE;
  }
  cudaStream_t s = (cudaStream_t)stream;
  if (net->precision == NEB_PREC_BF16X3) {
    TapeLayout tl = tape_layout(net, n);
    WsLayout wl = ws_layout(net, n);
    return tc_hidden_gram(net, (const float*)qw, n, (const char*)tape + tl.x_off[net->n_hidden],
                          AM, AS, accumulate, (char*)ws + wl.tc, s);
  }
  if (net->precision == NEB_PREC_FP64)
    return hidden_gram_simt<double, 4>(net, qw, n, tape, AM, AS, ws, s, accumulate);
  return hidden_gram_simt<float, 4>(net, qw, n, tape, AM, AS, ws, s, accumulate);
}

extern "C" int neb_backward_hidden(const neb_net* net, const void* const* W, const double* GMh,
                                   const double* GSh, const void* qw, int64_t n, const void* tape,
                                   void* const* gW, void* const* gb, int accumulate, void* ws,
                                   size_t ws_bytes, neb_stream_t stream) {
  int st = check_net(net);
  if (st) return st;
  GemmScope gemm(net->precision);
  NEB_REQUIRE(net->dim == 2, "neb_backward_hidden: 2D scalar potential only");
  NEB_REQUIRE(n > 0 && W && GMh && GSh && qw && tape && gW && gb, "neb_backward_hidden: bad arguments");
  for (int l = 0; l < net->n_hidden; ++l)
    NEB_REQUIRE(W[l] && gW[l] && gb[l], "neb_backward_hidden: null pointer at layer %d", l);
  if (ws_bytes < ws_layout(net, n).total || !ws) {
    set_error("neb_backward_hidden: workspace too small");
    return NEB_ERR_WORKSPACE;
  }
  cudaStream_t s = (cudaStream_t)stream;
  if (net->precision == NEB_PREC_BF16X3) {
    TapeLayout tl = tape_layout(net, n);
    WsLayout wl = ws_layout(net, n);
    TcTape tt;
    for (int l = 0; l <= net->n_hidden; ++l) {
      tt.x[l] = (char*)tape + tl.x_off[l];
      tt.z[l] = (char*)tape + tl.z_off[l];
    }
    return tc_backward_hidden(net, GMh, GSh, (const float*)qw, n, tt, (float* const*)gW,
                              (float* const*)gb, accumulate, (char*)ws + wl.tc, s);
  }
  if (net->precision == NEB_PREC_FP64)
    return backward_hidden_simt<double, 4>(net, W, GMh, GSh, qw, n, tape, gW, gb, ws, s,
                                           accumulate);
  return backward_hidden_simt<float, 4>(net, W, GMh, GSh, qw, n, tape, gW, gb, ws, s,
                                        accumulate);
}

extern "C" int neb_backward_output(const neb_net* net, const void* const* W, int start, int stop,
                                   const void* psibar, int64_t n, const void* tape,
                                   void* const* gW, void* const* gb, int accumulate, void* ws,
                                   size_t ws_bytes, neb_stream_t stream) {
  int st = check_net(net);
  if (st) return st;
  GemmScope gemm(net->precision);
  const int K = net->widths[net->n_hidden + 1];
  NEB_REQUIRE(n > 0 && W && psibar && tape && gW && gb && 0 <= start && start < stop && stop <= K,
              "neb_backward_output: bad arguments");
  for (int l = 0; l <= net->n_hidden; ++l)
    NEB_REQUIRE(W[l] && gW[l] && gb[l], "neb_backward_output: null pointer at layer %d", l);
  if (ws_bytes < ws_layout(net, n).total || !ws) {
    set_error("neb_backward_output: workspace too small");
    return NEB_ERR_WORKSPACE;
  }
  NEB_REQUIRE(net->precision != NEB_PREC_BF16X3,
              "neb_backward_output: use NEB_PREC_FP32 or NEB_PREC_FP64 for output-jet adjoints");
  return NEB_DISPATCH(net, backward_output_simt, net, W, start, stop, psibar, n, tape, gW, gb, ws,
                      (cudaStream_t)stream, accumulate);
}

extern "C" int neb_fields_gram(const neb_net* net, const void* Wout, const void* qw, int64_t n,
                               const void* tape, double* M, double* S, int accumulate, void* ws,
                               size_t ws_bytes, neb_stream_t stream) {
  int st = check_net(net);
  if (st) return st;
  GemmScope gemm(net->precision);
  NEB_REQUIRE(n > 0 && Wout && qw && tape && M && S, "neb_fields_gram: bad arguments");
  NEB_REQUIRE(net->precision != NEB_PREC_BF16X3,
              "neb_fields_gram: the direct route runs in NEB_PREC_FP32 or NEB_PREC_FP64");
  if (ws_bytes < ws_layout(net, n).total || !ws) {
    set_error("neb_fields_gram: workspace too small");
    return NEB_ERR_WORKSPACE;
  }
  return NEB_DISPATCH(net, fields_gram_simt, net, Wout, qw, n, tape, M, S, accumulate, ws,
                      (cudaStream_t)stream);
}

extern "C" int neb_backward_fields(const neb_net* net, const void* const* W, const double* GM,
                                   const double* GS, const void* qw, int64_t n, const void* tape,
                                   void* const* gW, void* const* gb, int accumulate, void* ws,
                                   size_t ws_bytes, neb_stream_t stream) {
  int st = check_net(net);
  if (st) return st;
  GemmScope gemm(net->precision);
  NEB_REQUIRE(n > 0 && W && GM && GS && qw && tape && gW && gb,
              "neb_backward_fields: bad arguments");
  for (int l = 0; l <= net->n_hidden; ++l)
    NEB_REQUIRE(W[l] && gW[l] && gb[l], "neb_backward_fields: null pointer at layer %d", l);
  NEB_REQUIRE(net->precision != NEB_PREC_BF16X3,
              "neb_backward_fields: the direct route runs in NEB_PREC_FP32 or NEB_PREC_FP64");
  if (ws_bytes < ws_layout(net, n).total || !ws) {
    set_error("neb_backward_fields: workspace too small");
    return NEB_ERR_WORKSPACE;
  }
  return NEB_DISPATCH(net, backward_fields_simt, net, W, GM, GS, qw, n, tape, gW, gb, accumulate,
                      ws, (cudaStream_t)stream);
}

extern "C" int neb_check_status(const neb_net* net, int64_t n, void* ws, size_t ws_bytes,
                                neb_stream_t stream) {
  int st = check_net(net);
  if (st) return st;
  if (net->precision != NEB_PREC_BF16X3) return NEB_OK;
  if (ws_bytes < ws_layout(net, n).total || !ws) {
    set_error("neb_check_status: workspace too small");
    return NEB_ERR_WORKSPACE;
  }
  int code = 0;
  st = tc_read_status(net, n, (char*)ws + ws_layout(net, n).tc, (cudaStream_t)stream, &code);
  if (st) return st;
  if (code) {
    set_error("a bounded device-side wait gave up (status %d); results of this step are invalid",
              code);
    return NEB_ERR_TIMEOUT;
  }
  return NEB_OK;
}

extern "C" size_t neb_column_gram_workspace_bytes(int64_t rows, int K) {
  if (rows <= 0 || K <= 0) return 0;
  return a256((size_t)ceil_div(rows, chunk_points(rows)) * K * K * sizeof(double));
}

extern "C" int neb_column_gram(int precision, int64_t rows, int K, const void* A, double scale,
                               int compensated, double* G, void* ws, size_t ws_bytes,
                               neb_stream_t stream) {
  NEB_REQUIRE(precision == NEB_PREC_FP32 || precision == NEB_PREC_FP64,
              "neb_column_gram: FP32 or FP64");
  NEB_REQUIRE(rows > 0 && K > 0 && A && G, "neb_column_gram: bad arguments");
  if (!ws || ws_bytes < neb_column_gram_workspace_bytes(rows, K)) {
    set_error("neb_column_gram: workspace too small");
    return NEB_ERR_WORKSPACE;
  }
  simt::ChanSet one{1, {0}};
  cudaStream_t s = (cudaStream_t)stream;
  if (precision == NEB_PREC_FP64)
    return launch_rowsum<double, 1, double>((const double*)A, K, (const double*)A, K, nullptr,
                                            one, rows, K, K, true, scale, (double*)ws, G, s);
  return launch_rowsum<float, 1, double>((const float*)A, K, (const float*)A, K, nullptr, one,
                                         rows, K, K, true, scale, (double*)ws, G, s, 0,
                                         compensated != 0);
}

extern "C" int neb_wait_selftest(int arrive, uint32_t spin_limit, int* status,
                                 neb_stream_t stream) {
  NEB_REQUIRE(status != nullptr, "neb_wait_selftest: null status");
  NEB_REQUIRE(spin_limit >= 1024 && spin_limit <= (1u << 24),
              "neb_wait_selftest: spin_limit must be in [1024, 2^24]");
  int code = 0;
  int st = tc_wait_selftest(arrive, spin_limit, status, (cudaStream_t)stream, &code);
  if (st) return st;
  if (code) {
    set_error("a bounded device-side wait gave up (status %d)", code);
    return NEB_ERR_TIMEOUT;
  }
  return NEB_OK;
}

extern "C" size_t neb_adam_workspace_bytes(void) { return 256; }

extern "C" int neb_adam(int dtype, int n_tensors, void* const* params, void* const* m,
                        void* const* v, const void* const* grads, const int64_t* sizes, int step,
                        int* step_counter, const int* gate, double lr, double clip,
                        double beta1, double beta2,
                        double eps,
                        double* norm_out, int* committed_out, void* ws, size_t ws_bytes,
                        neb_stream_t stream) {
  NEB_REQUIRE(dtype == 0 || dtype == 1, "neb_adam: dtype must be 0 (float) or 1 (double)");
  NEB_REQUIRE(n_tensors > 0 && n_tensors <= kMaxAdamTensors, "neb_adam: 1..%d tensors",
              kMaxAdamTensors);
  NEB_REQUIRE(params && m && v && grads && sizes && step >= 0, "neb_adam: bad arguments");
  if (ws_bytes < neb_adam_workspace_bytes() || !ws) {
    set_error("neb_adam: workspace too small");
    return NEB_ERR_WORKSPACE;
  }
  AdamTable t{};
  t.n = n_tensors;
  t.off[0] = 0;
  for (int i = 0; i < n_tensors; ++i) {
    NEB_REQUIRE(params[i] && m[i] && v[i] && grads[i] && sizes[i] >= 0,
                "neb_adam: bad tensor %d", i);
    t.p[i] = params[i];
    t.m[i] = m[i];
    t.v[i] = v[i];
    t.g[i] = grads[i];
    t.off[i + 1] = t.off[i] + sizes[i];
  }
  cudaStream_t s = (cudaStream_t)stream;
  double* acc = (double*)ws;
  int* flag = (int*)((char*)ws + 64);
  NEB_CUDA_CHECK(cudaMemsetAsync(ws, 0, 128, s));
  int64_t total = t.off[n_tensors];
  int blocks = (int)std::min<int64_t>(std::max<int64_t>(ceil_div(total, 256), 1), 1184);
  const double es = dtype == 0 ? 4.0 : 8.0;
  {
    KernelScope ks("adam_norm", s, 0, total * es);
    if (dtype == 0) adam_norm<float><<<blocks, 256, 0, s>>>(t, acc, flag);
    else adam_norm<double><<<blocks, 256, 0, s>>>(t, acc, flag);
    NEB_LAUNCH_CHECK();
  }
  double* scal = (double*)((char*)ws + 128);
  {
    KernelScope ks("adam_update", s, 0, total * es * 7, 2);
    adam_finalize<<<1, 1, 0, s>>>(acc, flag, clip, step, step_counter, gate, lr, beta1, beta2,
                                  norm_out, committed_out, scal);
    NEB_LAUNCH_CHECK();
    if (dtype == 0)
      adam_update<float><<<blocks, 256, 0, s>>>(t, scal, (float)beta1, (float)beta2, (float)eps);
    else
      adam_update<double><<<blocks, 256, 0, s>>>(t, scal, beta1, beta2, eps);
    NEB_LAUNCH_CHECK();
  }
  return NEB_OK;
}

// ------------------------------------------- allocation-free hidden Grams
// neb_hidden_gram_static computes what neb_hidden_gram computes for the
// FP32 and FP64 networks, but takes no workspace: its per-chunk FP64
// partial Grams live in the fixed device array below, so the call allocates
// no device memory at all.  It exists for callers that cannot hand the
// library a workspace: a plain C or ctypes host with no PyTorch or CuPy
// memory pool to carve one from, for which a cudaMalloc / cudaFree pair per
// call would also synchronise the whole device.
//
// The array holds at most kStaticScratchBytes (8 MiB):
// chunks x H x H doubles with chunks = ceil(n / max(256, ceil(n / 32))),
// i.e. H <= 128 at any n, H = 256 up to n = 4096.  Larger requests are
// rejected with NEB_ERR_ARG before anything is launched.  Nothing in the
// array needs to start at zero: every partial the reduction reads is
// written by the chunk kernel of the same call.
//
// The first call on each device looks up the array's device address with
// cudaGetSymbolAddress (with that device current) and caches it; make that
// first call before any stream capture begins.  There is one array per
// device, so calls that overlap in time on one device (two streams, two
// host threads) race on it: serialise them, e.g. on one stream.
static __device__ __align__(256) unsigned char g_gram_scratch[8u << 20];

namespace neb {
namespace {
constexpr size_t kStaticScratchBytes = sizeof(g_gram_scratch);
constexpr int kMaxScratchDevices = 64;
std::mutex g_scratch_mutex;
void* g_scratch_ptr[kMaxScratchDevices] = {};

int static_scratch(void** out) {
  int dev = -1;
  NEB_CUDA_CHECK(cudaGetDevice(&dev));
  NEB_REQUIRE(dev >= 0 && dev < kMaxScratchDevices,
              "neb_hidden_gram_static: device ordinal %d beyond %d", dev, kMaxScratchDevices);
  std::lock_guard<std::mutex> lock(g_scratch_mutex);
  if (!g_scratch_ptr[dev]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_gram_scratch);
    if (e != cudaSuccess || !p) {
      set_error("neb_hidden_gram_static: cudaGetSymbolAddress on device %d: %s", dev,
                cudaGetErrorString(e));
      return NEB_ERR_CUDA;
    }
    g_scratch_ptr[dev] = p;
  }
  *out = g_scratch_ptr[dev];
  return NEB_OK;
}

template <typename T>
int hidden_gram_fixed(const neb_net* net, const void* qw, int64_t n, const void* tape,
                      double* AM, double* AS, double* part, cudaStream_t s) {
  const int L = net->n_hidden, H = net->widths[L];
  TapeLayout tl = tape_layout(net, n);
  const T* HL = (const T*)((const char*)tape + tl.x_off[L]);
  simt::ChanSet grad{2, {1, 2}};
  simt::ChanSet lap{1, {3}};
  int st = launch_rowsum<T, 4, double>(HL, H, HL, H, (const T*)qw, grad, n, H, H, true, 1.0, part,
                                       AM, s);
  if (st) return st;
  return launch_rowsum<T, 4, double>(HL, H, HL, H, (const T*)qw, lap, n, H, H, true, 1.0, part,
                                     AS, s);
}
}  // namespace
}  // namespace neb

extern "C" int neb_hidden_gram_static(const neb_net* net, const void* qw, int64_t n,
                                      const void* tape, double* AM, double* AS,
                                      neb_stream_t stream) {
  int st = check_net(net);
  if (st) return st;
  NEB_REQUIRE(net->dim == 2, "neb_hidden_gram_static: 2D scalar potential only");
  NEB_REQUIRE(net->precision == NEB_PREC_FP32 || net->precision == NEB_PREC_FP64,
              "neb_hidden_gram_static: FP32 or FP64 networks only");
  NEB_REQUIRE(n > 0 && qw && tape && AM && AS, "neb_hidden_gram_static: bad arguments");
  const int H = net->widths[net->n_hidden];
  const int64_t chunks = ceil_div(n, chunk_points(n));
  const size_t need = (size_t)chunks * H * H * sizeof(double);
  NEB_REQUIRE(need <= kStaticScratchBytes,
              "neb_hidden_gram_static: %lld points x width %d need %zu bytes of scratch "
              "(%lld chunks x %d x %d doubles); the fixed array holds %zu",
              (long long)n, H, need, (long long)chunks, H, H, kStaticScratchBytes);
  void* part = nullptr;
  st = static_scratch(&part);
  if (st) return st;
  cudaStream_t s = (cudaStream_t)stream;
  if (net->precision == NEB_PREC_FP64)
    return hidden_gram_fixed<double>(net, qw, n, tape, AM, AS, (double*)part, s);
  return hidden_gram_fixed<float>(net, qw, n, tape, AM, AS, (double*)part, s);
}
