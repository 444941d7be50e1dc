// Tensor-core path of the jet MLP (NEB_PREC_BF16X3) on sm_103a.
//
// Every GEMM runs on tcgen05 with split-BF16 operands: a value x is stored as
// hi = bf16(x), lo = bf16(x - hi) (16 significant bits), and a product is
// accumulated in FP32 tensor memory as A_hi B_hi + A_lo B_hi + A_hi B_lo
// (+ A_lo B_lo for the Grams, where the dropped term would bias every
// diagonal the same way).
// Operands arrive by TMA (128-byte swizzle) through an mbarrier ring; one
// thread issues the MMAs, and the epilogue reads the accumulators from TMEM
// (sixteen warps in the jet GEMM, eight in the row sums).  The jet GEMM is
// persistent (one CTA per SM, tiles dealt round-robin): 128 points x 128
// outputs for the layer GEMMs (4 channels fill all 512 TMEM columns, so the
// epilogue of a tile and the MMAs of the next take turns), 128 x 64 with
// double-buffered accumulators for the Gram adjoint (epilogue and MMAs
// overlap).
//
// Device layouts (n_pad = n rounded up to 128 points; "planar" = one matrix
// per jet channel c in 0..3 = value, d/dx, d/dy, Laplacian), points
// contiguous so that a warp (32 TMEM lanes = 32 points) stores whole
// 128-byte lines:
//   X_l   [2 planes hi/lo][C][w_pad][n_pad]  layer output: MN-major A operand
//                                            of the next layer, K-major
//                                            (over points) for the weight
//                                            gradient and the Grams
//   Z_l   [C][w][n_pad]  float               pre-activation, for the reverse pass
// Kernels:
//   tc_jet_gemm<0>  forward layer:  Z = X W^T + b (value channel), X' = tanh-jet(Z)
//   tc_jet_gemm<1>  reverse data:   Zbar' = tanh-jet^T(Z', Zbar W)
//   tc_jet_gemm<2>  Gram adjoint:   Zbar_L = tanh-jet^T(Z_L, 2 w [0, h_x G_M, h_y G_M, h_lap G_S])
//   tc_rowsum       sum over points of A[m][p] B[n][p] (Grams, weight gradients),
//                   split over point ranges, FP32 chunk partials reduced
//                   afterwards with compensation (reduce_parts).
#include <cudaTypedefs.h>
#include "tc_path.cuh"
#include "tc_ptx.cuh"

namespace neb {

namespace {

constexpr int C = 4;              // 2D jet channels
constexpr int kTileBytes = 128 * 128;  // 128 rows x 64 bf16

int64_t round_up(int64_t a, int64_t b) { return (a + b - 1) / b * b; }

// ------------------------------------------------------------ host: maps
PFN_cuTensorMapEncodeTiled_v12000 g_encode = nullptr;

int get_encode() {
  if (g_encode) return NEB_OK;
  cudaDriverEntryPointQueryResult q;
  void* fn = nullptr;
  cudaError_t e = cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000,
                                                   cudaEnableDefault, &q);
  if (e != cudaSuccess || q != cudaDriverEntryPointSuccess || !fn) {
    set_error("cuTensorMapEncodeTiled unavailable");
    return NEB_ERR_CUDA;
  }
  g_encode = (PFN_cuTensorMapEncodeTiled_v12000)fn;
  return NEB_OK;
}

// 2D bf16 map over a row-major [rows][cols] array, box {64 cols, box_rows}.
int make_map(CUtensorMap* m, const void* base, int64_t rows, int64_t cols, int box_rows) {
  int st = get_encode();
  if (st) return st;
  if ((reinterpret_cast<uintptr_t>(base) & 15) || (cols * 2) % 16) {
    set_error("tensor map: base or row stride not 16-byte aligned");
    return NEB_ERR_ARG;
  }
  cuuint64_t dims[2] = {(cuuint64_t)cols, (cuuint64_t)rows};
  cuuint64_t strides[1] = {(cuuint64_t)cols * 2};
  cuuint32_t box[2] = {64, (cuuint32_t)box_rows};
  cuuint32_t estr[2] = {1, 1};
  CUresult r = g_encode(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(base), dims,
                        strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                        CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                        CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) {
    set_error("cuTensorMapEncodeTiled failed (%d) rows=%lld cols=%lld", (int)r, (long long)rows,
              (long long)cols);
    return NEB_ERR_CUDA;
  }
  return NEB_OK;
}

__device__ __forceinline__ uint8_t* align1024(uint8_t* p) {
  uintptr_t a = reinterpret_cast<uintptr_t>(p);
  return reinterpret_cast<uint8_t*>((a + 1023) & ~uintptr_t(1023));
}

// -------------------------------------------------------- jet GEMM kernel
struct JetGemmArgs {
  int n_points, n_pad, K, N;
  const float* bias;   // EPI 0: [N]
  const float* zprev;  // EPI 1, 2: [C][N][n_pad] pre-activation of the target layer
  const float* qw;     // EPI 2: [n_points] quadrature weights
  float* z_out;        // EPI 0: [C][N][n_pad]
  __nv_bfloat16* yt_out;  // [2][C][N][n_pad] split output
  int* status;
};

// epilogue warps of the jet GEMM (four per TMEM lane quarter) and the
// accumulator columns each reads per TMEM load
constexpr int kJetEpiWarps = 16;
constexpr int kJetEpiCols = 8;
constexpr int kJetThreads = 64 + 32 * kJetEpiWarps;

template <int EPI> struct JetCfg {
  // output columns per tile: 128 for the layer GEMMs (single accumulator
  // buffer, wider MMAs); 64 for the Gram adjoint (three channels, so two
  // buffers fit and its epilogue overlaps the next tile's MMAs)
  static constexpr int BN = EPI == 2 ? 64 : 128;
  static constexpr int NB = EPI == 2 ? 2 : 1;    // distinct B matrices
  static constexpr int NCH = EPI == 2 ? 3 : 4;   // accumulated channels
  static constexpr int CH0 = EPI == 2 ? 1 : 0;
  // accumulator buffers in the 512 TMEM columns (double-buffered when they fit)
  static constexpr int NBUF = 2 * NCH * BN <= 512 ? 2 : 1;
  static constexpr int TBUF = 512 / NBUF;        // TMEM columns per accumulator buffer
  // planes of B: the weights are split in two (hi, lo); the Gram adjoints
  // G_M, G_S in three (24 significant bits), because h G cancels in the
  // directions where G is large, so an independent rounding of G's entries
  // to 16 bits would show up in the gradient amplified by that cancellation
  static constexpr int NPL = EPI == 2 ? 3 : 2;
  static constexpr int A_ST = EPI == 2 ? 4 : 5;  // shared memory holds 4 A stages with 3 B planes
  static constexpr int B_ST = 2;
  static constexpr int B_TILE = BN * 128;        // BN rows x 64 bf16
  static constexpr int B_BYTES = NPL * NB * B_TILE;
  static constexpr int SMEM = 1024 + A_ST * 2 * kTileBytes + B_ST * B_BYTES + 256;
};


// Tile schedule of the persistent jet GEMM: whole rounds of 128 x BN tiles
// dealt round-robin to the CTAs, then, for the forward layer, the R tiles left
// over as 2R half tiles of BN / 2 outputs, one per CTA, when 2R fits the
// grid (512 tiles on 152 CTAs: three rounds, then 112 half tiles instead of
// a fourth round of 56 full ones while 96 CTAs wait).  A half tile loads the
// same operand stages (the B box from its first output row) and multiplies
// with N = BN / 2.
struct TileSched {
  int n_tiles, full_end, halves;  // halves: 0, or 2R half tiles after full_end
};

__device__ __forceinline__ TileSched make_sched(int total, int n_tiles, bool split) {
  TileSched s{n_tiles, total, 0};
  if (split) {
    const int G = gridDim.x, full = total / G * G, R = total - full;
    if (R > 0 && 2 * R <= G) {
      s.full_end = full;
      s.halves = 2 * R;
    }
  }
  return s;
}

// The i-th tile of this CTA (false: none): first output n0, first point p0,
// half = 1 for a half tile.
__device__ __forceinline__ bool tile_of(const TileSched& s, int i, int BN, int& n0, int& p0,
                                        int& half) {
  const int t = blockIdx.x + i * gridDim.x;
  if (t < s.full_end) {
    n0 = (t % s.n_tiles) * BN;
    p0 = (t / s.n_tiles) * 128;
    half = 0;
    return true;
  }
  if (s.halves == 0 || (int)blockIdx.x >= s.halves || i != s.full_end / (int)gridDim.x)
    return false;
  const int tf = s.full_end + blockIdx.x / 2;
  n0 = (tf % s.n_tiles) * BN + (blockIdx.x & 1) * (BN / 2);
  p0 = (tf / s.n_tiles) * 128;
  half = 1;
  return true;
}

// Persistent tcgen05 jet GEMM: tiles of 128 points x BN outputs (all jet
// channels) are dealt round-robin to the CTAs (one per SM).  The producer
// keeps loading operand stages across tile boundaries; the accumulators are
// double-buffered in tensor memory when 2 x NCH x BN columns fit in 512, so
// the epilogue of one tile can overlap the MMAs of the next.  Roles: warp 0 lane 0 issues TMA
// loads, warp 1 lane 0 issues MMAs, warps 2-17 run the epilogue (lane quarter
// w % 4, column quarter (w - 2) / 4 of the tile, in chunks of kJetEpiCols).
template <int EPI>
__global__ void __launch_bounds__(kJetThreads, 1)
tc_jet_gemm(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB,
            JetGemmArgs g) {
  using Cfg = JetCfg<EPI>;
  constexpr int BN = Cfg::BN, NB = Cfg::NB, NCH = Cfg::NCH, CH0 = Cfg::CH0, A_ST = Cfg::A_ST,
                B_ST = Cfg::B_ST, NPL = Cfg::NPL;
  static_assert(Cfg::SMEM <= 232448, "jet GEMM shared memory above the 227 KB per block");
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = align1024(smem_raw);
  uint8_t* a_smem = smem;
  uint8_t* b_smem = smem + A_ST * 2 * kTileBytes;
  uint64_t* bars = reinterpret_cast<uint64_t*>(b_smem + B_ST * Cfg::B_BYTES);
  uint64_t* a_full = bars;
  uint64_t* a_empty = bars + A_ST;
  uint64_t* b_full = bars + 2 * A_ST;
  uint64_t* b_empty = bars + 2 * A_ST + B_ST;
  uint64_t* acc_full = bars + 2 * A_ST + 2 * B_ST;   // [2]
  uint64_t* acc_empty = acc_full + 2;                // [2]
  uint64_t* mma_done = acc_empty + 2;                // every MMA of this CTA completed
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(mma_done + 1);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int KC = g.K / 64;
  const int n_tiles = g.N / BN;
  const int total = n_tiles * (g.n_pad / 128);
  // the forward layer runs alone on the GPU; the reverse-data GEMM shares it
  // with the weight-gradient GEMM on a side stream, so its CTAs do not all
  // start together and a last round of half tiles would not shorten it
  const TileSched sched = make_sched(total, n_tiles, EPI == 0);

  if (threadIdx.x == 0) {
    for (int i = 0; i < A_ST; ++i) {
      tc::mbar_init(&a_full[i], 1);
      tc::mbar_init(&a_empty[i], 1);
    }
    for (int i = 0; i < B_ST; ++i) {
      tc::mbar_init(&b_full[i], 1);
      tc::mbar_init(&b_empty[i], 1);
    }
    for (int i = 0; i < 2; ++i) {
      tc::mbar_init(&acc_full[i], 1);
      tc::mbar_init(&acc_empty[i], kJetEpiWarps);  // one arrival per epilogue warp
    }
    tc::mbar_init(mma_done, 1);
    tc::fence_mbar_init();
  }
  if (warp == 1) {
    tc::tmem_alloc(tmem_slot, 512);
    tc::tmem_relinquish();
  }
  tc::tc_fence_before();
  __syncthreads();
  tc::tc_fence_after();
  const uint32_t tmem = *tmem_slot;

  if (warp == 0 && lane == 0) {
    // ---------------- TMA producer.  A wait that gives up ends the issue
    // before the stage's expect_tx, so every stage is either fully issued or
    // untouched; the copies already issued are drained before the CTA exits.
    int ai = 0, bi = 0;
    bool ok = true;
    for (int i = 0; ok; ++i) {
      int n0, p0, half;
      if (!tile_of(sched, i, BN, n0, p0, half)) break;
      for (int kc = 0; ok && kc < KC; ++kc) {
        const int bs = bi % B_ST;
        if (!tc::mbar_wait(&b_empty[bs], ((bi / B_ST) & 1) ^ 1, g.status)) {
          ok = false;
          break;
        }
        tc::mbar_expect_tx(&b_full[bs], Cfg::B_BYTES);
        for (int b = 0; b < NB; ++b)
          for (int pl = 0; pl < NPL; ++pl)
            tc::tma_load_2d(b_smem + bs * Cfg::B_BYTES + (b * NPL + pl) * Cfg::B_TILE, &tmB,
                            &b_full[bs], kc * 64, (pl * NB + b) * g.N + n0);
        ++bi;
        for (int ci = 0; ci < NCH; ++ci) {
          const int as = ai % A_ST, c = CH0 + ci;
          if (!tc::mbar_wait(&a_empty[as], ((ai / A_ST) & 1) ^ 1, g.status)) {
            ok = false;
            break;
          }
          tc::mbar_expect_tx(&a_full[as], 2 * kTileBytes);
          // A is MN-major: [plane][channel][k][point]; a tile is two boxes of
          // 64 points x 64 k rows
          for (int pl = 0; pl < 2; ++pl)
            for (int hb = 0; hb < 2; ++hb)
              tc::tma_load_2d(a_smem + (as * 2 + pl) * kTileBytes + hb * (kTileBytes / 2), &tmA,
                              &a_full[as], p0 + hb * 64, (pl * C + c) * g.K + kc * 64);
          ++ai;
        }
      }
    }
    tc::drain_ring(b_full, B_ST, bi, g.status);
    tc::drain_ring(a_full, A_ST, ai, g.status);
  } else if (warp == 1 && lane == 0) {
    // ---------------- MMA issuer (stops at the first wait that gives up)
    constexpr uint32_t idesc_full = tc::idesc_bf16(128, BN, true);
    constexpr uint32_t idesc_half = tc::idesc_bf16(128, BN / 2, true);
    int ai = 0, bi = 0;
    bool ok = true;
    for (int it = 0; ok; ++it) {
      int n0, p0, half;
      if (!tile_of(sched, it, BN, n0, p0, half)) break;
      const uint32_t idesc = half ? idesc_half : idesc_full;
      const int buf = it % Cfg::NBUF, use = it / Cfg::NBUF;
      if (!tc::mbar_wait(&acc_empty[buf], (use & 1) ^ 1, g.status)) break;
      tc::tc_fence_after();
      for (int kc = 0; ok && kc < KC; ++kc) {
        const int bs = bi % B_ST;
        if (!tc::mbar_wait(&b_full[bs], (bi / B_ST) & 1, g.status)) {
          ok = false;
          break;
        }
        tc::tc_fence_after();
        for (int ci = 0; ci < NCH; ++ci) {
          const int as = ai % A_ST, c = CH0 + ci;
          if (!tc::mbar_wait(&a_full[as], (ai / A_ST) & 1, g.status)) {
            ok = false;
            break;
          }
          tc::tc_fence_after();
          const int bsel = (EPI == 2 && c == 3) ? 1 : 0;
          const uint32_t a_hi = tc::smem_u32(a_smem + (as * 2) * kTileBytes);
          const uint32_t a_lo = a_hi + kTileBytes;
          const uint32_t b_hi =
              tc::smem_u32(b_smem + bs * Cfg::B_BYTES + (bsel * NPL) * Cfg::B_TILE);
          const uint32_t b_lo = b_hi + Cfg::B_TILE;
          const uint32_t d = tmem + buf * Cfg::TBUF + ci * BN;
#pragma unroll
          for (int kk = 0; kk < 4; ++kk) {
            // K step of 16: 16 rows of the MN-major A tile, 32 bytes of the K-major B rows
            const uint32_t aoff = kk * 2048, boff = kk * 32;
            const uint64_t dah = tc::desc_mn_sw128(a_hi + aoff, kTileBytes / 2);
            const uint64_t dal = tc::desc_mn_sw128(a_lo + aoff, kTileBytes / 2);
            const uint64_t dbh = tc::desc_sw128(b_hi + boff), dbl = tc::desc_sw128(b_lo + boff);
            tc::mma_bf16(d, dah, dbh, idesc, (kc | kk) != 0);
            tc::mma_bf16(d, dal, dbh, idesc, 1);
            tc::mma_bf16(d, dah, dbl, idesc, 1);
            if constexpr (NPL == 3) {  // B = b1 + b2 + b3: add lo.b2 and hi.b3
              const uint64_t db3 = tc::desc_sw128(b_hi + 2 * Cfg::B_TILE + boff);
              tc::mma_bf16(d, dal, dbl, idesc, 1);
              tc::mma_bf16(d, dah, db3, idesc, 1);
            }
          }
          tc::mma_commit(&a_empty[as]);
          ++ai;
        }
        if (!ok) break;
        tc::mma_commit(&b_empty[bs]);
        ++bi;
      }
      if (!ok) break;
      tc::mma_commit(&acc_full[buf]);
    }
    // the MMAs issued so far must complete before the tensor memory is freed
    tc::mma_commit(mma_done);
    tc::mbar_wait_drain(mma_done, 0, g.status);
  } else if (warp >= 2) {
    // ---------------- epilogue: kJetEpiWarps warps, one thread per point
    // (TMEM lane): warp w reads lane quarter w % 4, column slice (w - 2) / 4
    const int q = warp & 3, slice = (warp - 2) >> 2;
    const int row = q * 32 + lane;
    const size_t plane = (size_t)C * g.n_pad * g.N;  // elements of one hi or lo plane
    bool ok = true;
    for (int it = 0; ok; ++it) {
      int n0, p0, half;
      if (!tile_of(sched, it, BN, n0, p0, half)) break;
      const int p = p0 + row;
      const int buf = it % Cfg::NBUF, use = it / Cfg::NBUF;
      float w2 = 0.f;
      if constexpr (EPI == 2) w2 = p < g.n_points ? 2.f * g.qw[p] : 0.f;
      // columns per TMEM load: the reverse transposes hold more live values
      constexpr int kW = EPI == 0 ? kJetEpiCols : kJetEpiCols / 2;
      constexpr int kSlice = BN / (kJetEpiWarps / 4);  // columns of this warp
      constexpr int kChunks = kSlice / kW;
      // a half tile: half the columns per warp, every warp still drains (and
      // releases) its share of the accumulator buffer
      const int slice_w = half ? kSlice / 2 : kSlice, nchunks = half ? kChunks / 2 : kChunks;
      for (int jc = 0; jc < nchunks; ++jc) {
        const int j0 = slice * slice_w + jc * kW;
        const int col = n0 + j0;
        // global operands first (bias, or the pre-activations of the target
        // layer), so their latency overlaps the accumulator wait and loads
        float out[C][kW];
        float bias_c[kW];
        if constexpr (EPI == 0) {
#pragma unroll
          for (int j = 0; j < kW; ++j) bias_c[j] = __ldg(g.bias + col + j);
        } else {
#pragma unroll
          for (int c = 0; c < C; ++c)
#pragma unroll
            for (int j = 0; j < kW; ++j)
              out[c][j] = __ldg(g.zprev + ((size_t)c * g.N + col + j) * g.n_pad + p);
        }
        if (jc == 0) {
          // the TMEM loads below are warp-collective: the whole warp goes on
          // only when every lane saw the accumulators complete
          ok = __all_sync(0xffffffffu, tc::mbar_wait(&acc_full[buf], use & 1, g.status));
          if (!ok) break;
          tc::tc_fence_after();
        }
        uint32_t raw[NCH][kW];
#pragma unroll
        for (int ci = 0; ci < NCH; ++ci)
          tc::tmem_ld_issue<kW>(tmem + ((uint32_t)(q * 32) << 16) + buf * Cfg::TBUF + ci * BN + j0,
                              raw[ci]);
        tc::tmem_ld_wait();
        float acc[NCH][kW];
#pragma unroll
        for (int ci = 0; ci < NCH; ++ci) {
          tc::tmem_ld_fence(raw[ci]);
#pragma unroll
          for (int j = 0; j < kW; ++j) acc[ci][j] = __uint_as_float(raw[ci][j]);
        }
        if (jc == nchunks - 1) {  // this warp's columns of the buffer are drained
          tc::tc_fence_before();
          __syncwarp();
          if (lane == 0) tc::mbar_arrive(&acc_empty[buf]);
        }
        if constexpr (EPI == 0) {
#pragma unroll
          for (int j = 0; j < kW; ++j) {
#pragma unroll
            for (int c = 0; c < C; ++c) out[c][j] = acc[c][j];
            out[0][j] += bias_c[j];
          }
#pragma unroll
          for (int c = 0; c < C; ++c)
#pragma unroll
            for (int j = 0; j < kW; ++j)  // [C][N][n_pad]: a warp stores 32 points
              g.z_out[((size_t)c * g.N + col + j) * g.n_pad + p] = out[c][j];
#pragma unroll
          for (int j = 0; j < kW; ++j) {
            float v[C];
#pragma unroll
            for (int c = 0; c < C; ++c) v[c] = out[c][j];
            jet_act_forward<C>(v);
#pragma unroll
            for (int c = 0; c < C; ++c) out[c][j] = v[c];
          }
        } else {
#pragma unroll
          for (int j = 0; j < kW; ++j) {
            float z[C], v[C];
#pragma unroll
            for (int c = 0; c < C; ++c) z[c] = out[c][j];
            if constexpr (EPI == 2) {
              v[0] = 0.f;
#pragma unroll
              for (int c = 1; c < C; ++c) v[c] = w2 * acc[c - 1][j];
            } else {
#pragma unroll
              for (int c = 0; c < C; ++c) v[c] = acc[c][j];
            }
            jet_act_backward<C>(z, v);
#pragma unroll
            for (int c = 0; c < C; ++c) out[c][j] = v[c];
          }
        }
        // split outputs [2][C][N][n_pad] (points contiguous): each store of a
        // warp writes 32 consecutive points (64 bytes)
#pragma unroll
        for (int c = 0; c < C; ++c) {
#pragma unroll
          for (int j = 0; j < kW; ++j) {
            __nv_bfloat16 h, l;
            tc::split_bf16(out[c][j], h, l);
            const size_t gi = ((size_t)c * g.N + col + j) * g.n_pad + p;
            g.yt_out[gi] = h;
            g.yt_out[plane + gi] = l;
          }
        }
      }
    }
  }
  tc::tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    tc::tc_fence_after();
    tc::tmem_dealloc(tmem, 512);
  }
}

// ----------------------------------------------------------- rowsum kernel
// part[z][m][n] = sum over K-chunks kq in split z of A(m, kq) . B(n, kq),
// where the K index runs over (channel ci, point block): A rows
// (pl * aC + a_ch0 + ci) * M + m, B rows (pl * bC + b_ch0 + ci) * N + n.
struct RowsumArgs {
  int M, N, n_pad, n_ch, a_ch0, b_ch0, aC, bC, splits, ldp;
  int lo_lo;  // also accumulate A_lo B_lo: the Grams need it (without it the
              // missing product acts as a systematic negative ridge)
  float* part;  // FP32 chunk-group partials, combined with compensation by reduce_parts
  int* status;
};

template <int BN> struct RowCfg {
  static constexpr int ST = 3;
  static constexpr int A_BYTES = 2 * kTileBytes;
  static constexpr int B_BYTES = 2 * BN * 128;
  static constexpr int SMEM = 1024 + ST * (A_BYTES + B_BYTES) + 256;
  static constexpr int TMEM = 2 * BN < 32 ? 32 : 2 * BN;  // two accumulator buffers
};

// The tensor cores' FP32 accumulation rounds toward zero, so a long run of
// same-sign MMAs into one accumulator drifts (a few 1e-6 relative on a Gram
// diagonal after a few hundred MMAs, which shows up as a ridge on the mass
// matrix).  Each 64-point chunk is therefore accumulated in its own tensor
// memory buffer (16 MMAs) and drained by the epilogue warps into
// round-to-nearest FP32 register sums, double-buffered against the MMAs.
template <int BN>
__global__ void __launch_bounds__(320, 1)
tc_rowsum(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB,
          RowsumArgs g) {
  using Cfg = RowCfg<BN>;
  constexpr int ST = Cfg::ST;
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = align1024(smem_raw);
  uint8_t* a_smem = smem;
  uint8_t* b_smem = smem + ST * Cfg::A_BYTES;
  uint64_t* bars = reinterpret_cast<uint64_t*>(b_smem + ST * Cfg::B_BYTES);
  uint64_t* full = bars;
  uint64_t* empty = bars + ST;
  uint64_t* acc_ready = bars + 2 * ST;      // [2]
  uint64_t* acc_free = bars + 2 * ST + 2;   // [2]
  uint64_t* mma_done = bars + 2 * ST + 4;   // every MMA of this CTA completed
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars + 2 * ST + 5);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int ntiles = g.N / BN;
  const int m0 = (blockIdx.x / ntiles) * 128, n0 = (blockIdx.x % ntiles) * BN;
  const int pblocks = g.n_pad / 64;
  const int total = g.n_ch * pblocks;
  const int per = (total + g.splits - 1) / g.splits;
  const int k_begin = blockIdx.y * per;
  const int k_end = min(total, k_begin + per);
  const int n_it = k_end > k_begin ? k_end - k_begin : 0;

  if (threadIdx.x == 0) {
    for (int i = 0; i < ST; ++i) {
      tc::mbar_init(&full[i], 1);
      tc::mbar_init(&empty[i], 1);
    }
    for (int i = 0; i < 2; ++i) {
      tc::mbar_init(&acc_ready[i], 1);
      tc::mbar_init(&acc_free[i], 256);
    }
    tc::mbar_init(mma_done, 1);
    tc::fence_mbar_init();
  }
  if (warp == 1) {
    tc::tmem_alloc(tmem_slot, Cfg::TMEM);
    tc::tmem_relinquish();
  }
  tc::tc_fence_before();
  __syncthreads();
  tc::tc_fence_after();
  const uint32_t tmem = *tmem_slot;

  if (warp == 0 && lane == 0) {
    // producer: stops at the first wait that gives up, then drains the
    // copies it issued before the CTA exits
    int issued = 0;
    for (int it = 0; it < n_it; ++it) {
      const int kq = k_begin + it, s = it % ST;
      const int ci = kq / pblocks, pb = kq % pblocks;
      if (!tc::mbar_wait(&empty[s], ((it / ST) & 1) ^ 1, g.status)) break;
      tc::mbar_expect_tx(&full[s], Cfg::A_BYTES + Cfg::B_BYTES);
      for (int pl = 0; pl < 2; ++pl) {
        tc::tma_load_2d(a_smem + s * Cfg::A_BYTES + pl * kTileBytes, &tmA, &full[s], pb * 64,
                        (pl * g.aC + g.a_ch0 + ci) * g.M + m0);
        tc::tma_load_2d(b_smem + s * Cfg::B_BYTES + pl * (BN * 128), &tmB, &full[s], pb * 64,
                        (pl * g.bC + g.b_ch0 + ci) * g.N + n0);
      }
      ++issued;
    }
    tc::drain_ring(full, ST, issued, g.status);
  } else if (warp == 1 && lane == 0) {
    constexpr uint32_t idesc = tc::idesc_bf16(128, BN);
    for (int it = 0; it < n_it; ++it) {
      const int s = it % ST, buf = it & 1;
      if (it >= 2 && !tc::mbar_wait(&acc_free[buf], ((it >> 1) & 1) ^ 1, g.status)) break;
      if (!tc::mbar_wait(&full[s], (it / ST) & 1, g.status)) break;
      tc::tc_fence_after();
      const uint32_t d = tmem + buf * BN;
      const uint32_t a_hi = tc::smem_u32(a_smem + s * Cfg::A_BYTES), a_lo = a_hi + kTileBytes;
      const uint32_t b_hi = tc::smem_u32(b_smem + s * Cfg::B_BYTES), b_lo = b_hi + BN * 128;
#pragma unroll
      for (int kk = 0; kk < 4; ++kk) {
        const uint32_t off = kk * 32;
        const uint64_t dah = tc::desc_sw128(a_hi + off), dal = tc::desc_sw128(a_lo + off);
        const uint64_t dbh = tc::desc_sw128(b_hi + off), dbl = tc::desc_sw128(b_lo + off);
        tc::mma_bf16(d, dah, dbh, idesc, kk != 0);
        tc::mma_bf16(d, dal, dbh, idesc, 1);
        tc::mma_bf16(d, dah, dbl, idesc, 1);
        if (g.lo_lo) tc::mma_bf16(d, dal, dbl, idesc, 1);
      }
      tc::mma_commit(&empty[s]);
      tc::mma_commit(&acc_ready[buf]);
    }
    // the MMAs issued so far must complete before the tensor memory is freed
    tc::mma_commit(mma_done);
    tc::mbar_wait_drain(mma_done, 0, g.status);
  } else if (warp >= 2) {
    // eight drain warps: lane quarter q = warp % 4, column half h
    constexpr int HB = BN / 2;
    const int q = warp & 3, h = (warp - 2) >> 2;
    const int m = m0 + q * 32 + lane;
    float sum[HB];
#pragma unroll
    for (int j = 0; j < HB; ++j) sum[j] = 0.f;
    for (int it = 0; it < n_it; ++it) {
      const int buf = it & 1;
      // warp-uniform: the TMEM loads below are warp-collective
      if (!__all_sync(0xffffffffu, tc::mbar_wait(&acc_ready[buf], (it >> 1) & 1, g.status)))
        break;
      tc::tc_fence_after();
      uint32_t raw[HB / 16][16];
#pragma unroll
      for (int c16 = 0; c16 < HB / 16; ++c16)
        tc::tmem_ld16_issue(tmem + ((uint32_t)(q * 32) << 16) + buf * BN + h * HB + c16 * 16,
                            raw[c16]);
      tc::tmem_ld_wait();
#pragma unroll
      for (int c16 = 0; c16 < HB / 16; ++c16) {
        tc::tmem_ld_fence(raw[c16]);
#pragma unroll
        for (int j = 0; j < 16; ++j) sum[c16 * 16 + j] += __uint_as_float(raw[c16][j]);
      }
      tc::tc_fence_before();
      tc::mbar_arrive(&acc_free[buf]);
    }
    float* out = g.part + ((size_t)blockIdx.y * g.M + m) * g.ldp + n0 + h * HB;
#pragma unroll
    for (int j = 0; j < HB; j += 4)
      *reinterpret_cast<float4*>(out + j) = make_float4(sum[j], sum[j + 1], sum[j + 2], sum[j + 3]);
  }
  tc::tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    tc::tc_fence_after();
    tc::tmem_dealloc(tmem, Cfg::TMEM);
  }
}

// ------------------------------------------------------- helper kernels
// Interleaved float features [n][C][F] -> split planar X_0 [2][C][n_pad][Fp]
// and its transpose XT_0 [2][C][Fp][n_pad], zero padded.
__global__ void prep_features(const float* __restrict__ f, int n, int F, int n_pad, int Fp,
                              __nv_bfloat16* __restrict__ XT) {
  const size_t total = (size_t)C * n_pad * Fp;
  const size_t plane = total;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total;
       i += (size_t)gridDim.x * blockDim.x) {
    // i enumerates (c, k, p) with p fastest so the writes coalesce
    int p = (int)(i % n_pad);
    int k = (int)((i / n_pad) % Fp);
    int c = (int)(i / ((size_t)n_pad * Fp));
    float v = (p < n && k < F) ? f[((size_t)p * C + c) * F + k] : 0.f;
    __nv_bfloat16 h, l;
    tc::split_bf16(v, h, l);
    XT[i] = h;
    XT[plane + i] = l;
  }
}

// W [out][in] float -> Ws [2][out][inp] (zero padded), optionally WT [2][inp][out].
__global__ void split_weight(const float* __restrict__ W, int out, int in, int inp,
                             __nv_bfloat16* __restrict__ Ws, __nv_bfloat16* __restrict__ WT) {
  const size_t total = (size_t)out * inp;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total;
       i += (size_t)gridDim.x * blockDim.x) {
    int o = (int)(i / inp), k = (int)(i % inp);
    float v = k < in ? W[(size_t)o * in + k] : 0.f;
    __nv_bfloat16 h, l;
    tc::split_bf16(v, h, l);
    Ws[i] = h;
    Ws[total + i] = l;
    if (WT) {
      size_t t = (size_t)k * out + o;
      WT[t] = h;
      WT[total + t] = l;
    }
  }
}

// G_M, G_S (double [H][H]) -> [3 planes][2 (M, S)][H][H] bf16 with
// G = b1 + b2 + b3 to 24 significant bits (the residuals are formed in FP64).
__global__ void split_gram_adjoint(const double* __restrict__ GM, const double* __restrict__ GS,
                                   int H, __nv_bfloat16* __restrict__ out) {
  const size_t hh = (size_t)H * H;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < 2 * hh;
       i += (size_t)gridDim.x * blockDim.x) {
    const double v = i < hh ? GM[i] : GS[i - hh];
    const __nv_bfloat16 b1 = __double2bfloat16(v);
    const double r1 = v - (double)__bfloat162float(b1);
    const __nv_bfloat16 b2 = __double2bfloat16(r1);
    const double r2 = r1 - (double)__bfloat162float(b2);
    out[i] = b1;
    out[2 * hh + i] = b2;
    out[4 * hh + i] = __double2bfloat16(r2);
  }
}

// wHT[pl][ci][f][p] = split(w_p * (XT_L[c = ci + 1][f][p])) for the three field
// channels; w_p = 0 for padded points.  Eight points (16 bytes per plane) per
// thread step; n_pad is a multiple of 128.
__global__ void weighted_fields_t(const __nv_bfloat16* __restrict__ XT, const float* __restrict__ qw,
                                  int n, int n_pad, int H, __nv_bfloat16* __restrict__ out) {
  const size_t total = (size_t)3 * H * n_pad, total8 = total / 8;
  const size_t src_plane = (size_t)C * H * n_pad;
  for (size_t v8 = blockIdx.x * (size_t)blockDim.x + threadIdx.x; v8 < total8;
       v8 += (size_t)gridDim.x * blockDim.x) {
    const size_t i = v8 * 8;
    const int p0 = (int)(i % n_pad);
    const size_t src = (size_t)H * n_pad + i;  // channel ci + 1
    const uint4 ah = *reinterpret_cast<const uint4*>(XT + src);
    const uint4 al = *reinterpret_cast<const uint4*>(XT + src_plane + src);
    const __nv_bfloat16* hh = reinterpret_cast<const __nv_bfloat16*>(&ah);
    const __nv_bfloat16* ll = reinterpret_cast<const __nv_bfloat16*>(&al);
    float w[8];
    if (p0 + 8 <= n && (reinterpret_cast<uintptr_t>(qw) & 15) == 0) {
      const float4 w0 = *reinterpret_cast<const float4*>(qw + p0);
      const float4 w1 = *reinterpret_cast<const float4*>(qw + p0 + 4);
      w[0] = w0.x; w[1] = w0.y; w[2] = w0.z; w[3] = w0.w;
      w[4] = w1.x; w[5] = w1.y; w[6] = w1.z; w[7] = w1.w;
    } else {
#pragma unroll
      for (int t = 0; t < 8; ++t) w[t] = p0 + t < n ? qw[p0 + t] : 0.f;
    }
    uint4 oh, ol;
    __nv_bfloat16* h8 = reinterpret_cast<__nv_bfloat16*>(&oh);
    __nv_bfloat16* l8 = reinterpret_cast<__nv_bfloat16*>(&ol);
#pragma unroll
    for (int t = 0; t < 8; ++t) {
      const float v = (__bfloat162float(hh[t]) + __bfloat162float(ll[t])) * w[t];
      tc::split_bf16(v, h8[t], l8[t]);
    }
    *reinterpret_cast<uint4*>(out + i) = oh;
    *reinterpret_cast<uint4*>(out + total + i) = ol;
  }
}

// out[m * ldo + j] = sum_z part[(z * M + m) * ldp + j] for j < ncols: the
// FP32 partials are summed with an error term (TwoSum), so the sum keeps
// about twice FP32 precision without double-precision arithmetic; sym
// averages the sum with its transpose.
__device__ __forceinline__ void two_sum_acc(float& hi, float& lo, float x) {
  const float s = hi + x, bb = s - hi;
  lo += (hi - (s - bb)) + (x - bb);
  hi = s;
}

// Sum of the FP32 chunk-group partials part[z][m][j] over z (in order,
// TwoSum compensated, four z loads in flight), one output per thread, a
// 256-thread block on 8 rows x 32 columns (a warp reads 128-byte lines).
// sym (square): out = (P + P^T) / 2; the mirrored 32 x 8 tile is summed on
// reads of 32-byte row pieces and exchanged through shared memory.
__device__ __forceinline__ void sum_splits(const float* __restrict__ p, size_t zs, int splits,
                                           float& hi, float& lo) {
  hi = 0.f;
  lo = 0.f;
  int z = 0;
  for (; z + 4 <= splits; z += 4) {
    const float a0 = p[z * zs], a1 = p[(z + 1) * zs], a2 = p[(z + 2) * zs],
                a3 = p[(z + 3) * zs];
    two_sum_acc(hi, lo, a0);
    two_sum_acc(hi, lo, a1);
    two_sum_acc(hi, lo, a2);
    two_sum_acc(hi, lo, a3);
  }
  for (; z < splits; ++z) two_sum_acc(hi, lo, p[z * zs]);
}

__global__ void __launch_bounds__(256) reduce_parts(const float* __restrict__ part, int splits,
                                                    int M, int ldp, int ncols, int ldo, int sym,
                                                    int accumulate, float* __restrict__ outf,
                                                    double* __restrict__ outd) {
  __shared__ float th[32][9], tl[32][9];
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  const int j0 = blockIdx.x * 32, m0 = blockIdx.y * 8;
  const size_t zs = (size_t)M * ldp;
  const int m = m0 + ty, j = j0 + tx;
  float hi = 0.f, lo = 0.f;
  if (m < M && j < ncols) sum_splits(part + (size_t)m * ldp + j, zs, splits, hi, lo);
  if (sym) {
    // thread t sums the mirror element (j0 + t / 8, m0 + t % 8)
    const int r = threadIdx.x >> 3, c = threadIdx.x & 7;
    float a = 0.f, b = 0.f;
    if (j0 + r < M && m0 + c < ncols)
      sum_splits(part + (size_t)(j0 + r) * ldp + m0 + c, zs, splits, a, b);
    th[r][c] = a;
    tl[r][c] = b;
    __syncthreads();
    two_sum_acc(hi, lo, th[tx][ty]);  // element (j, m)
    lo += tl[tx][ty];
    hi *= 0.5f;
    lo *= 0.5f;
  }
  if (m >= M || j >= ncols) return;
  if (outf) {
    float* o = outf + (size_t)m * ldo + j;
    *o = accumulate ? *o + (hi + lo) : hi + lo;
  }
  if (outd) {
    double* o = outd + (size_t)m * ldo + j;
    *o = accumulate ? *o + ((double)hi + (double)lo) : (double)hi + (double)lo;
  }
}

// Bias gradient: gb[o] = sum over points of the value plane of Zbar (hi +
// lo), Zbar in [2][C][N][n_pad] (points contiguous).  A 256-thread block
// takes two outputs, four warps each over a quarter of the points (16-byte
// loads, FP32 sums of 8-point groups accumulated in FP64), combined in
// shared memory.
__global__ void __launch_bounds__(256) bias_rows_tc(const __nv_bfloat16* __restrict__ zb,
                                                   int n_pad, int N, int accumulate,
                                                   float* __restrict__ out) {
  __shared__ double part[8];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int o = blockIdx.x * 2 + (warp >> 2), quarter = warp & 3;
  double acc = 0.0;
  if (o < N) {
    const size_t plane = (size_t)C * N * n_pad;
    const uint4* hi = reinterpret_cast<const uint4*>(zb + (size_t)o * n_pad);
    const uint4* lo = reinterpret_cast<const uint4*>(zb + plane + (size_t)o * n_pad);
    const int nv = n_pad / 8, per = (nv + 3) / 4;
    const int v0 = quarter * per, v1 = min(nv, v0 + per);
    for (int v = v0 + lane; v < v1; v += 32) {
      const uint4 a = hi[v], b = lo[v];
      const __nv_bfloat16* ha = reinterpret_cast<const __nv_bfloat16*>(&a);
      const __nv_bfloat16* lb = reinterpret_cast<const __nv_bfloat16*>(&b);
      float s8 = 0.f;
#pragma unroll
      for (int t = 0; t < 8; ++t) s8 += __bfloat162float(ha[t]) + __bfloat162float(lb[t]);
      acc += (double)s8;
    }
  }
#pragma unroll
  for (int sh = 16; sh > 0; sh >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, sh);
  if (lane == 0) part[warp] = acc;
  __syncthreads();
  if (threadIdx.x < 2) {
    const int oo = blockIdx.x * 2 + threadIdx.x;
    if (oo < N) {
      const double* q = part + threadIdx.x * 4;
      const float v = (float)((q[0] + q[1]) + (q[2] + q[3]));
      out[oo] = accumulate ? out[oo] + v : v;
    }
  }
}

// ---------------------------------------------------------- host helpers
struct Dims {
  int L, F, Fp, H;
  int64_t n, n_pad;
  int w[NEB_MAX_HIDDEN + 2];   // real widths
  int wp[NEB_MAX_HIDDEN + 2];  // padded K widths
};

Dims dims_of(const neb_net* net, int64_t n) {
  Dims d{};
  d.L = net->n_hidden;
  d.n = n;
  d.n_pad = round_up(n, 128);
  for (int l = 0; l <= d.L + 1; ++l) {
    d.w[l] = net->widths[l];
    d.wp[l] = l == 0 ? (int)round_up(net->widths[0], 64) : net->widths[l];
  }
  d.F = d.w[0];
  d.Fp = d.wp[0];
  d.H = d.w[d.L];
  return d;
}

size_t a256(size_t x) { return (x + 255) & ~size_t(255); }

// TC workspace: [status][W splits per layer][WT splits][G split][wHT][Zbar A][Zbar B]
//               [FP64 split partials][bias sums]
constexpr int kMaxSplits = 32;
struct TcWs {
  size_t status, w[NEB_MAX_HIDDEN + 1], wt[NEB_MAX_HIDDEN + 1], gsplit, wht, zb0, zb1, part,
      total;
};

TcWs tc_ws(const Dims& d) {
  TcWs t{};
  size_t off = 0;
  t.status = off;
  off += 256;
  int mw = 0;
  for (int l = 1; l <= d.L; ++l) {
    t.w[l] = off;
    off += a256((size_t)2 * d.w[l] * d.wp[l - 1] * 2);
    t.wt[l] = off;
    off += l >= 2 ? a256((size_t)2 * d.w[l] * d.wp[l - 1] * 2) : 0;
    mw = mw > d.w[l] ? mw : d.w[l];
  }
  t.gsplit = off;
  off += a256((size_t)6 * d.H * d.H * 2);
  t.wht = off;
  off += a256((size_t)2 * 3 * d.H * d.n_pad * 2);
  size_t zb = a256((size_t)2 * C * d.n_pad * mw * 2);
  t.zb0 = off;
  off += zb;
  t.zb1 = off;
  off += zb;
  int mx = mw > d.wp[0] ? mw : d.wp[0];
  t.part = off;
  off += a256((size_t)kMaxSplits * mx * mx * 8);
  t.total = off;
  return t;
}

template <int EPI>
int launch_jet(const CUtensorMap& A, const CUtensorMap& B, const JetGemmArgs& args, int n_tiles,
               int p_tiles, cudaStream_t s, const char* name, double flops, double bytes) {
  int dev = 0, sms = 0;
  if (int st = device_sms(&dev, &sms)) return st;
  static bool configured[kMaxDevices] = {};
  if (!configured[dev]) {
    NEB_CUDA_CHECK(cudaFuncSetAttribute(tc_jet_gemm<EPI>,
                                        cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        JetCfg<EPI>::SMEM));
    configured[dev] = true;
  }
  (void)n_tiles;
  NEB_REQUIRE(args.N % JetCfg<EPI>::BN == 0, "jet GEMM: N = %d must be a multiple of %d", args.N,
              JetCfg<EPI>::BN);
  const int tiles = (args.N / JetCfg<EPI>::BN) * p_tiles;
  KernelScope ks(name, s, flops, bytes);
  tc_jet_gemm<EPI><<<std::min(tiles, sms), kJetThreads, JetCfg<EPI>::SMEM, s>>>(A, B, args);
  NEB_LAUNCH_CHECK();
  return NEB_OK;
}

// part = per-split partials of A . B^T over (channels, points); M rows of A,
// N rows of B.
template <int BN>
int launch_rowsum_bn(const CUtensorMap& A, const CUtensorMap& B, RowsumArgs g, cudaStream_t s,
                     const char* name, double flops, double bytes) {
  int dev = 0, sms = 0;
  if (int st = device_sms(&dev, &sms)) return st;
  static bool configured[kMaxDevices] = {};
  if (!configured[dev]) {
    NEB_CUDA_CHECK(cudaFuncSetAttribute(tc_rowsum<BN>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        RowCfg<BN>::SMEM));
    configured[dev] = true;
  }
  KernelScope ks(name, s, flops, bytes);
  dim3 grid((g.M / 128) * (g.N / BN), g.splits);
  tc_rowsum<BN><<<grid, 320, RowCfg<BN>::SMEM, s>>>(A, B, g);
  NEB_LAUNCH_CHECK();
  return NEB_OK;
}

int launch_rowsum(const void* a_base, int aC, int a_ch0, const void* b_base, int bC, int b_ch0,
                  int n_ch, int M, int N, int64_t n_pad, float* part, int* status,
                  cudaStream_t s, const char* name, double flops, int* splits_out,
                  bool lo_lo = false) {
  NEB_REQUIRE(M % 128 == 0, "tensor-core rowsum: M = %d must be a multiple of 128", M);
  int BN = N % 128 == 0 ? 128 : (N % 64 == 0 ? 64 : 0);
  NEB_REQUIRE(BN, "tensor-core rowsum: N = %d must be a multiple of 64", N);
  int tiles = (M / 128) * (N / BN);
  int total = n_ch * (int)(n_pad / 64);
  int dev = 0, sms = 0;
  if (int st = device_sms(&dev, &sms)) return st;
  int splits = (int)std::max(1, std::min(kMaxSplits, (2 * sms + tiles - 1) / tiles));
  splits = std::min(splits, total);
  CUtensorMap ma, mb;
  int st = make_map(&ma, a_base, (int64_t)2 * aC * M, n_pad, 128);
  if (st) return st;
  st = make_map(&mb, b_base, (int64_t)2 * bC * N, n_pad, BN);
  if (st) return st;
  RowsumArgs g{M, N, (int)n_pad, n_ch, a_ch0, b_ch0, aC, bC, splits, N, lo_lo ? 1 : 0, part,
               status};
  double bytes = (double)n_ch * n_pad * (M + N) * 4;
  *splits_out = splits;
  if (BN == 128) return launch_rowsum_bn<128>(ma, mb, g, s, name, flops, bytes);
  return launch_rowsum_bn<64>(ma, mb, g, s, name, flops, bytes);
}

int reduce(const float* part, int splits, int M, int ldp, int ncols, int ldo, bool sym,
           float* outf, double* outd, cudaStream_t s, int accumulate = 0) {
  KernelScope ks("reduce_chunks", s, 0, (double)splits * M * ncols * 4);
  NEB_REQUIRE(!sym || M == ncols, "reduce: a symmetric sum needs a square matrix");
  const dim3 grid((ncols + 31) / 32, (M + 7) / 8);
  reduce_parts<<<grid, 256, 0, s>>>(part, splits, M, ldp, ncols, ldo, sym ? 1 : 0, accumulate,
                                    outf, outd);
  NEB_LAUNCH_CHECK();
  return NEB_OK;
}

int check_dims(const neb_net* net) {
  NEB_REQUIRE(net->dim == 2, "NEB_PREC_BF16X3: 2D scalar potential only");
  for (int l = 1; l <= net->n_hidden; ++l)
    NEB_REQUIRE(net->widths[l] % 128 == 0,
                "NEB_PREC_BF16X3: hidden widths must be multiples of 128 (layer %d: %d)", l,
                net->widths[l]);
  return NEB_OK;
}

}  // namespace

// ======================================================================
size_t tc_tape_bytes(const neb_net* net, int64_t n, size_t* x_off, size_t* z_off) {
  Dims d = dims_of(net, n);
  size_t off = 0;
  for (int l = 0; l <= d.L; ++l) {
    if (l > 0) {
      if (z_off) z_off[l] = off;
      off += a256((size_t)C * d.n_pad * d.w[l] * 4);
    }
    if (x_off) x_off[l] = off;
    off += a256((size_t)2 * C * d.n_pad * d.wp[l] * 2);  // X, points contiguous
  }
  return off;
}

size_t tc_workspace_bytes(const neb_net* net, int64_t n) { return tc_ws(dims_of(net, n)).total; }

int tc_forward(const neb_net* net, const float* const* W, const float* const* b, const float* feats,
               int64_t n, const TcTape& tape, char* ws, cudaStream_t s) {
  int st = check_dims(net);
  if (st) return st;
  Dims d = dims_of(net, n);
  TcWs t = tc_ws(d);
  int* status = (int*)(ws + t.status);
  NEB_CUDA_CHECK(cudaMemsetAsync(status, 0, sizeof(int), s));
  {
    KernelScope ks("tc_prep_features", s, 0, (double)n * C * d.F * 4 + 8.0 * C * d.n_pad * d.Fp);
    size_t total = (size_t)C * d.n_pad * d.Fp;
    int blocks = (int)std::min<size_t>((total + 255) / 256, 8192);
    prep_features<<<blocks, 256, 0, s>>>(feats, (int)n, d.F, (int)d.n_pad, d.Fp,
                                         (__nv_bfloat16*)tape.x[0]);
    NEB_LAUNCH_CHECK();
  }
  for (int l = 1; l <= d.L; ++l) {
    KernelScope ks("tc_split_weight", s, 0, (double)d.w[l] * d.wp[l - 1] * 12);
    size_t total = (size_t)d.w[l] * d.wp[l - 1];
    int blocks = (int)std::min<size_t>((total + 255) / 256, 4096);
    split_weight<<<blocks, 256, 0, s>>>(W[l - 1], d.w[l], d.w[l - 1], d.wp[l - 1],
                                        (__nv_bfloat16*)(ws + t.w[l]),
                                        l >= 2 ? (__nv_bfloat16*)(ws + t.wt[l]) : nullptr);
    NEB_LAUNCH_CHECK();
  }
  for (int l = 1; l <= d.L; ++l) {
    const int K = d.wp[l - 1], N = d.w[l];
    CUtensorMap ma, mb;
    if ((st = make_map(&ma, tape.x[l - 1], (int64_t)2 * C * K, d.n_pad, 64))) return st;
    if ((st = make_map(&mb, ws + t.w[l], (int64_t)2 * N, K, JetCfg<0>::BN))) return st;
    JetGemmArgs g{};
    g.n_points = (int)n;
    g.n_pad = (int)d.n_pad;
    g.K = K;
    g.N = N;
    g.bias = b[l - 1];
    g.z_out = (float*)tape.z[l];
    g.yt_out = (__nv_bfloat16*)tape.x[l];
    g.status = status;
    if ((st = launch_jet<0>(ma, mb, g, N / 128, (int)(d.n_pad / 128), s, "tc_jet_layer_fwd",
                            2.0 * n * C * (double)d.w[l - 1] * N,
                            (double)d.n_pad * C * (K * 4 + N * 8))))
      return st;
  }
  return NEB_OK;
}

int tc_hidden_gram(const neb_net* net, const float* qw, int64_t n, const void* hl, double* AM,
                   double* AS, int accumulate, char* ws, cudaStream_t s) {
  int st = check_dims(net);
  if (st) return st;
  Dims d = dims_of(net, n);
  TcWs t = tc_ws(d);
  char* part = ws + t.part;
  int* status = (int*)(ws + t.status);
  const int H = d.H;
  const char* XT = (const char*)hl;
  __nv_bfloat16* wht = (__nv_bfloat16*)(ws + t.wht);
  {
    KernelScope ks("tc_weighted_fields", s, 0, 3.0 * H * d.n_pad * 8);
    size_t total8 = (size_t)3 * H * d.n_pad / 8;
    int blocks = (int)std::min<size_t>((total8 + 255) / 256, 8192);
    weighted_fields_t<<<blocks, 256, 0, s>>>((const __nv_bfloat16*)XT, qw, (int)n, (int)d.n_pad,
                                             H, wht);
    NEB_LAUNCH_CHECK();
  }
  int splits = 0;
  // A_M: channels (d/dx, d/dy) = wHT channels 0, 1 against XT channels 1, 2
  if ((st = launch_rowsum(wht, 3, 0, XT, C, 1, 2, H, H, d.n_pad, (float*)part, status, s,
                          "tc_gram", 2.0 * 2 * n * (double)H * H, &splits, true)))
    return st;
  if ((st = reduce((float*)part, splits, H, H, H, H, true, nullptr, AM, s, accumulate)))
    return st;
  if ((st = launch_rowsum(wht, 3, 2, XT, C, 3, 1, H, H, d.n_pad, (float*)part, status, s,
                          "tc_gram", 2.0 * n * (double)H * H, &splits, true)))
    return st;
  return reduce((float*)part, splits, H, H, H, H, true, nullptr, AS, s, accumulate);
}

int tc_backward_hidden(const neb_net* net, const double* GMh, const double* GSh, const float* qw,
                       int64_t n, const TcTape& tape, float* const* gW, float* const* gb,
                       int accumulate, char* ws, cudaStream_t s) {
  int st = check_dims(net);
  if (st) return st;
  Dims d = dims_of(net, n);
  TcWs t = tc_ws(d);
  char* part = ws + t.part;
  int* status = (int*)(ws + t.status);
  const int L = d.L, H = d.H;
  __nv_bfloat16* gs = (__nv_bfloat16*)(ws + t.gsplit);
  {
    KernelScope ks("tc_split_gram_adjoint", s, 0, (double)H * H * 2 * 14);
    split_gram_adjoint<<<(int)std::min<size_t>((2ull * H * H + 255) / 256, 4096), 256, 0, s>>>(
        GMh, GSh, H, gs);
    NEB_LAUNCH_CHECK();
  }
  // Zbar of the current layer and the next, [2][C][w][n_pad] (points contiguous)
  char* zb[2] = {ws + t.zb0, ws + t.zb1};
  // Gram adjoint + tanh transpose of layer L
  {
    CUtensorMap ma, mb;
    if ((st = make_map(&ma, tape.x[L], (int64_t)2 * C * H, d.n_pad, 64))) return st;
    if ((st = make_map(&mb, gs, (int64_t)JetCfg<2>::NPL * 2 * H, H, JetCfg<2>::BN))) return st;
    JetGemmArgs g{};
    g.n_points = (int)n;
    g.n_pad = (int)d.n_pad;
    g.K = H;
    g.N = H;
    g.zprev = (const float*)tape.z[L];
    g.qw = qw;
    g.yt_out = (__nv_bfloat16*)zb[0];
    g.status = status;
    if ((st = launch_jet<2>(ma, mb, g, H / 128, (int)(d.n_pad / 128), s, "tc_gram_adjoint_bwd",
                            2.0 * 3 * n * (double)H * H, (double)d.n_pad * C * H * 12)))
      return st;
  }
  // The parameter gradients of layer l (weight-gradient GEMM, its reduction,
  // the bias sums) run on a side stream, concurrently with the data gradient
  // of layer l on the main stream: both only read Zbar_l, so the side work
  // fills the SMs the data-gradient GEMM leaves idle in its last wave.  The
  // main stream waits for the side work of layer l before the data gradient
  // of layer l-1 overwrites that Zbar buffer, and before returning.
  int dev = 0;
  NEB_CUDA_CHECK(cudaGetDevice(&dev));
  NEB_REQUIRE(dev >= 0 && dev < kMaxDevices, "tensor-core backward: device index %d", dev);
  static thread_local cudaStream_t side[kMaxDevices] = {};
  static thread_local cudaEvent_t ev_z[kMaxDevices] = {}, ev_w[kMaxDevices][2] = {},
                                  ev_j[kMaxDevices] = {};
  if (!side[dev]) {
    NEB_CUDA_CHECK(cudaStreamCreateWithFlags(&side[dev], cudaStreamNonBlocking));
    NEB_CUDA_CHECK(cudaEventCreateWithFlags(&ev_z[dev], cudaEventDisableTiming));
    for (int q = 0; q < 2; ++q)
      NEB_CUDA_CHECK(cudaEventCreateWithFlags(&ev_w[dev][q], cudaEventDisableTiming));
    NEB_CUDA_CHECK(cudaEventCreateWithFlags(&ev_j[dev], cudaEventDisableTiming));
  }
  cudaStream_t s2 = side[dev];
  SideStreamJoin join{s, s2, ev_j[dev], true};
  int cur = 0;
  for (int l = L; l >= 1; --l) {
    const int out = d.w[l], in = d.w[l - 1], inp = d.wp[l - 1];
    NEB_CUDA_CHECK(cudaEventRecord(ev_z[dev], s));  // Zbar_l is complete
    NEB_CUDA_CHECK(cudaStreamWaitEvent(s2, ev_z[dev], 0));
    // weight gradient: gW_l[o][i] = sum_c sum_p Zbar_l[c][o][p] X_{l-1}[c][i][p]
    const char* x_prev = (const char*)tape.x[l - 1];
    int splits = 0;
    if ((st = launch_rowsum(zb[cur], C, 0, x_prev, C, 0, C, out, inp, d.n_pad, (float*)part,
                            status, s2, "tc_weight_grad", 2.0 * C * n * (double)out * in,
                            &splits)))
      return st;
    if ((st = reduce((float*)part, splits, out, inp, in, in, false, gW[l - 1], nullptr, s2,
                     accumulate)))
      return st;
    {
      KernelScope ks("bias_grad", s2, 0, (double)d.n_pad * out * 4);
      bias_rows_tc<<<(out + 1) / 2, 256, 0, s2>>>((const __nv_bfloat16*)zb[cur], (int)d.n_pad,
                                                  out, accumulate, gb[l - 1]);
      NEB_LAUNCH_CHECK();
    }
    NEB_CUDA_CHECK(cudaEventRecord(ev_w[dev][l & 1], s2));  // side work of layer l issued
    if (l == 1) {
      NEB_CUDA_CHECK(cudaStreamWaitEvent(s, ev_w[dev][1], 0));
      join.armed = false;
      break;
    }
    // the data gradient of layer l overwrites the Zbar buffer the side work
    // of layer l+1 read
    if (l < L) NEB_CUDA_CHECK(cudaStreamWaitEvent(s, ev_w[dev][(l + 1) & 1], 0));
    // data gradient through W_l and the tanh transpose of layer l-1
    CUtensorMap ma, mb;
    if ((st = make_map(&ma, zb[cur], (int64_t)2 * C * out, d.n_pad, 64))) return st;
    if ((st = make_map(&mb, ws + t.wt[l], (int64_t)2 * in, out, JetCfg<1>::BN))) return st;
    JetGemmArgs g{};
    g.n_points = (int)n;
    g.n_pad = (int)d.n_pad;
    g.K = out;
    g.N = in;
    g.zprev = (const float*)tape.z[l - 1];
    g.yt_out = (__nv_bfloat16*)zb[cur ^ 1];
    g.status = status;
    if ((st = launch_jet<1>(ma, mb, g, in / 128, (int)(d.n_pad / 128), s,
                            "tc_jet_layer_bwd_data", 2.0 * C * n * (double)out * in,
                            (double)d.n_pad * C * (out * 4 + in * 12))))
      return st;
    cur ^= 1;
  }
  return NEB_OK;
}

int tc_output(const neb_net*, const float*, const float*, int, int, int64_t, const void*, void*,
              cudaStream_t) {
  set_error("NEB_PREC_BF16X3 stores no output-layer jets; evaluate them with NEB_PREC_FP32");
  return NEB_ERR_UNSUPPORTED;
}

// One CTA waits, with the same bounded mbarrier wait every tensor-core
// pipeline uses, for a phase that completes only if `arrive` is set (thread
// 1 arrives); no copy or MMA is involved.  Without the arrival the wait runs
// out after `limit` polls and records bit 0 in *status.
__global__ void wait_selftest_kernel(int arrive, uint32_t limit, int* status) {
  __shared__ uint64_t bar;
  if (threadIdx.x == 0) {
    tc::mbar_init(&bar, 1);
    tc::fence_mbar_init();
  }
  __syncthreads();
  if (arrive && threadIdx.x == 1) tc::mbar_arrive(&bar);
  if (threadIdx.x == 0) tc::mbar_wait(&bar, 0, status, limit);
}

int tc_wait_selftest(int arrive, uint32_t limit, int* status, cudaStream_t s, int* out) {
  NEB_CUDA_CHECK(cudaMemsetAsync(status, 0, sizeof(int), s));
  {
    KernelScope ks("wait_selftest", s, 0, 0);
    wait_selftest_kernel<<<1, 32, 0, s>>>(arrive, limit, status);
    NEB_LAUNCH_CHECK();
  }
  NEB_CUDA_CHECK(cudaMemcpyAsync(out, status, sizeof(int), cudaMemcpyDeviceToHost, s));
  NEB_CUDA_CHECK(cudaStreamSynchronize(s));
  return NEB_OK;
}

int tc_read_status(const neb_net* net, int64_t n, char* ws, cudaStream_t s, int* out) {
  Dims d = dims_of(net, n);
  TcWs t = tc_ws(d);
  NEB_CUDA_CHECK(cudaMemcpyAsync(out, ws + t.status, sizeof(int), cudaMemcpyDeviceToHost, s));
  NEB_CUDA_CHECK(cudaStreamSynchronize(s));
  return NEB_OK;
}

}  // namespace neb
