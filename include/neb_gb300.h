/*
 * neb_gb300 — C ABI of the GB300 (sm_103a) neural-eigenfluid hot path.
 *
 * Every entry point takes device pointers, explicit sizes and a CUDA stream,
 * returns an int status (NEB_OK or a negative NEB_ERR_* code, with a message
 * in neb_last_error()), allocates no device memory on the hot path (the caller
 * owns every buffer, including the workspace and the activation tape), and
 * never synchronises the host except where noted.
 *
 * Device layout of a jet array: [n_points][C][width] row-major, C = 4 in 2D
 * (value, d/dx, d/dy, Laplacian) and C = 10 in 3D (value, d/dx, d/dy, d/dz,
 * Hessian xx, xy, xz, yy, yz, zz).  Parameters: W_l is [width_out][width_in]
 * row-major, b_l is [width_out]; "master" type is float for NEB_PREC_FP32 and
 * NEB_PREC_BF16X3 and double for NEB_PREC_FP64.
 *
 * The reference (baiming-zhang/NEB) is Python/CuPy and has no C interface;
 * each entry names the reference function whose role it takes over.  Paths
 * are relative to the reference project:
 *   HB  = experiments/2d/_backend/periodic_core/vortex_merger/src/eigenfluid/
 *         gen/vortex_merger2d/hardcoded_backend.py
 *   NCC = experiments/metaball/_backend/flow/cases/metaball/native_cupy_core.py
 *   VTJ2= experiments/metaball/_backend/flow/cases/metaball/velocity_trace_jet2.py
 *   VC  = experiments/metaball/_backend/flow/cases/metaball/velocity/core.py
 *   ROLL= experiments/periodic/paper_rollout.py
 */
#ifndef NEB_GB300_H
#define NEB_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct CUstream_st* neb_stream_t; /* a cudaStream_t; NULL = legacy stream */

enum {
  NEB_OK = 0,
  NEB_ERR_ARG = -1,          /* bad shape / pointer / option (ValueError)          */
  NEB_ERR_CUDA = -2,         /* CUDA runtime or library failure                     */
  NEB_ERR_WORKSPACE = -3,    /* workspace smaller than neb_*_workspace_bytes        */
  NEB_ERR_NOT_PD = -4,       /* mass matrix not positive definite (rank gate)       */
  NEB_ERR_NONFINITE = -5,    /* non-finite value detected (FloatingPointError)      */
  NEB_ERR_SOLVER = -6,       /* eigensolver did not converge                        */
  NEB_ERR_UNSUPPORTED = -7,  /* configuration not built for this device / options  */
  NEB_ERR_TIMEOUT = -8       /* a bounded device-side wait gave up                  */
};

enum { NEB_PREC_FP32 = 0, NEB_PREC_FP64 = 1, NEB_PREC_BF16X3 = 2, NEB_PREC_TF32 = 3,
       NEB_PREC_BF16X9 = 4 };
/* NEB_PREC_TF32 / NEB_PREC_BF16X9: FP32 storage, masters and jet epilogues as
 * NEB_PREC_FP32, with the layer GEMMs (forward, data and weight gradients)
 * on the tensor cores through cuBLAS -- TF32 inputs with FP32 accumulation
 * (one pass), or the BF16x9 emulation of FP32 products; the Grams keep the
 * FP32 (optionally compensated) sums. */
/* Accumulation of the FP32 Grams (FP64 always sums in FP64; split-BF16 sums
 * in tensor memory, drained every 64 points): PLAIN sums the products in
 * FP32; COMPENSATED forms every product exactly (FMA) and keeps each chunk
 * sum as a TwoSum pair, for bases whose mass matrix is nearly singular,
 * where the ~1e-7 relative error a plain FP32 sum leaves in every entry
 * moves the small eigenvalues of the pencil. */
enum { NEB_GRAM_PLAIN = 0, NEB_GRAM_COMPENSATED = 1 };
enum { NEB_FEAT_PERIODIC = 0, NEB_FEAT_MULTIHOLE = 1, NEB_FEAT_RAW3D = 2 };

#define NEB_MAX_HIDDEN 8

/* Shape of the shared tanh MLP: widths[0] input features, widths[1..n_hidden]
 * hidden widths, widths[n_hidden + 1] outputs (K in 2D, 3K in 3D). */
typedef struct neb_net {
  int32_t dim;        /* 2 or 3 */
  int32_t n_hidden;   /* 1..NEB_MAX_HIDDEN */
  int32_t widths[NEB_MAX_HIDDEN + 2];
  int32_t precision;  /* NEB_PREC_* */
  int32_t gram;       /* NEB_GRAM_* (0 = plain) */
} neb_net;

/* Thread-local message of the last failing call. */
const char* neb_last_error(void);

/* Instrumentation (the role of the reference's synchronised stage timers,
 * VC:25-30 timed): neb_kernel_launches() counts every kernel this library has
 * launched (its own kernels; cuSOLVER / cuBLAS calls count once each).
 * Between neb_timing_begin() and neb_timing_end() every launch is bracketed
 * by CUDA events on its stream; neb_timing_end synchronises those events and
 * reports, per kernel name, the launch count, total milliseconds and the
 * algorithmic flops and bytes of those launches (up to max_kernels entries;
 * names are written as NUL-terminated strings of name_len bytes each). */
unsigned long long neb_kernel_launches(void);
int neb_timing_begin(void);
int neb_timing_end(int max_kernels, char* names, int name_len, int* launches, double* total_ms,
                   double* flops, double* bytes, int* n_kernels);

/* Bytes of the activation tape (inputs and pre-activations of every layer,
 * in the precision's storage format) for n_points; and of the scratch
 * workspace every neb_* call below needs for n_points. */
size_t neb_tape_bytes(const neb_net* net, int64_t n_points);
size_t neb_workspace_bytes(const neb_net* net, int64_t n_points);

/* Input features with their spatial jets, written as a [n][C][widths[0]]
 * master-type array.  kind = NEB_FEAT_PERIODIC: sin/cos(2 pi k s / period),
 * s in (x, y), k = 1..n_freq (params[0] = period; HB:576-588 encoding_jet2,
 * periodic_sincos_xy).  NEB_FEAT_MULTIHOLE: (x, y, atan2 about each centre),
 * params = centres (2 per hole, at most 32 holes).  NEB_FEAT_RAW3D: (x, y, z).
 * params is a HOST array; points: [n][dim] double, device. */
int neb_features(const neb_net* net, int kind, int n_freq, const double* params,
                 int n_params, const double* points, int64_t n_points, void* features,
                 neb_stream_t stream);

/* Hidden layers of the jet MLP: for l = 1..n_hidden, z_l = W_l x_{l-1} (+ b_l
 * on the value channel), x_l = tanh-jet(z_l); inputs and pre-activations are
 * kept in the tape for the reverse pass.  Replaces HB:1716-1880
 * forward_stream_jet1/2 with HB:1005-1070 linear_forward_batch_jet2 +
 * sine_forward_jet2 per layer, NCC:130-140 Model.forward, VTJ2:65-76 forward.
 * W, b: host arrays of n_hidden + 1 device pointers (the output layer's are
 * not read here). */
int neb_forward(const neb_net* net, const void* const* W, const void* const* b,
                const void* features, int64_t n_points, void* tape, void* workspace,
                size_t workspace_bytes, neb_stream_t stream);

/* Output-layer jets psi = W_out x_L + b_out for output rows [start, stop):
 * psi is [n][C][stop - start], master type.  Role of the output linear of
 * NCC:138-139 / VTJ2:71-73. */
int neb_output(const neb_net* net, const void* W_out, const void* b_out, int start,
               int stop, int64_t n_points, const void* tape, void* psi,
               neb_stream_t stream);

/* Envelope jet times output jets (Leibniz rule on the jet channels):
 * y = e * x (reverse = 0) or the adjoint of x given the adjoint x of the
 * product (reverse != 0; y may alias x for neither).  envelope: [n][C] one
 * scalar jet per point; x, y: [n][C][width], the network's master type (use
 * the FP32 / FP64 evaluation network).  2D uses the Laplacian channel
 * (lap(e f) = e lap f + f lap e + 2 grad e . grad f), 3D the Hessian.
 * Replaces NCC:139 product1 and NCC:144 envelope_product_backward_jet1,
 * VTJ2 product / product_reverse. */
int neb_envelope_product(const neb_net* net, const void* envelope, int64_t n_points, int width,
                         const void* x, void* y, int reverse, neb_stream_t stream);

/* 2D scalar potential: weighted Grams of the last hidden layer's field
 * channels, A_M = sum_p w_p (h_x h_x^T + h_y h_y^T), A_S = sum_p w_p h_lap
 * h_lap^T (FP64, [H][H]); per-CTA partial sums, FP64 cross-CTA reduction.
 * With psi = W_out h + b: M = W_out A_M W_out^T, S = W_out A_S W_out^T, i.e.
 * the Grams of ROLL:178-179 and VC:40-46.  qw: [n] quadrature weights,
 * master type.  accumulate != 0 adds to A_M, A_S (point-chunked Grams). */
int neb_hidden_gram(const neb_net* net, const void* qw, int64_t n_points,
                    const void* tape, double* A_M, double* A_S, int accumulate,
                    void* workspace, size_t workspace_bytes, neb_stream_t stream);

/* neb_hidden_gram for FP32 / FP64 networks without a workspace argument: no
 * counterpart in the reference (its CuPy code always has a memory pool).
 * For hosts that cannot pass a workspace; allocates nothing.  The per-chunk
 * partials live in a fixed 8 MiB device array: chunks x H x H doubles must
 * fit (H <= 128 at any n_points), else NEB_ERR_ARG.  The first call on each
 * device sets up the array's address and should come before any stream
 * capture; calls overlapping in time on one device race on the array.  The
 * address is cached per device for the life of the process: after
 * cudaDeviceReset on a device the cached address is stale, so a process
 * that resets a device must not call this entry point on it again. */
int neb_hidden_gram_static(const neb_net* net, const void* qw, int64_t n_points,
                           const void* tape, double* A_M, double* A_S, neb_stream_t stream);

/* Direct route: FP64 K x K Grams of the fields of every mode, from the
 * output jets psi = W_out h of this call's points (kept in the workspace,
 * FP32 / FP64 networks): 2D K = widths[L+1] scalar potentials,
 * u = (psi_y, -psi_x), omega = -lap psi; 3D K = widths[L+1] / 3 vector
 * potentials A_k = (psi_3k, psi_3k+1, psi_3k+2), u = curl A,
 * omega = curl curl A (VTJ2:93-98, VC:32-38).  M = sum_p w u_i.u_j,
 * S = sum_p w omega_i.omega_j (ROLL:178-179, VC:40-46).  accumulate != 0
 * adds into M and S, so a large point set is processed in chunks, each chunk
 * with its own neb_forward (the recompute of VC:88-99). */
int neb_fields_gram(const neb_net* net, const void* W_out, const void* qw,
                    int64_t n_points, const void* tape, double* M, double* S, int accumulate,
                    void* workspace, size_t workspace_bytes, neb_stream_t stream);

/* FP64 spectral stage on an m x m pencil (S, M), M positive definite:
 * Cholesky of M, generalized symmetric eigensolve S v = lam M v with
 * V^T M V = I (ascending lam), loss = sum_k c_k lam_k and its adjoints
 * G_S = dL/dS = V diag(c) V^T, G_M = dL/dM = -V diag(c lam) V^T.
 * Replaces ROLL:180-187 (rank gate + scipy eigh(S, M)), VTJ2:107-117
 * trace_objective (c = 1) and VC:48-69 coefficient_peel's FP64 Cholesky.
 * Outputs lam[m], V[m][m], G_M, G_S [m][m], loss[1] (all device, FP64);
 * info[1] (device int) receives the solver status without a host
 * synchronisation: 0 = success, > m = M not positive definite (rank gate),
 * other > 0 = no convergence, -1 = non-finite loss. */
size_t neb_spectral_workspace_bytes(int m);
int neb_spectral(int m, const double* M, const double* S, const double* c, double* lam,
                 double* V, double* G_M, double* G_S, double* loss, int* info,
                 void* workspace, size_t workspace_bytes, neb_stream_t stream);

/* Finite pencil of a possibly singular mass matrix, FP64 (cuSOLVER syevd):
 * M = Q diag(e) Q^T; the r = #{e_i > rank_rtol * e_max} leading directions
 * span range(M) (the eigenvalue-ratio rank test of ROLL:180-186, which
 * rejects where this restricts); lam[0..r) ascending eigenvalues of
 * (S, M) on that range, rows 0..r-1 of V their M-orthonormal eigenvectors,
 * loss = sum_{k<r} c_k lam_k, G_S = V^T diag(c) V, G_M = -V^T diag(c lam) V.
 * Equal to neb_spectral when r = m.  Synchronises the stream once (the rank
 * sizes the reduced problem) and writes r to *rank (host pointer). */
size_t neb_spectral_range_workspace_bytes(int m);
int neb_spectral_range(int m, const double* M, const double* S, const double* c,
                       double rank_rtol, double* lam, double* V, double* G_M, double* G_S,
                       double* loss, int* rank, int* info, void* workspace,
                       size_t workspace_bytes, neb_stream_t stream);

/* Same contract as neb_spectral for m a multiple of 64 up to 512, computed
 * with the precision where the conditioning lives: the Cholesky of M and the
 * reduction C = L^-1 S L^-T in compensated FP32 (value = hi + lo, FP64-class
 * accuracy); the reduced, well conditioned C rounded to FP32 and reduced to
 * tridiagonal form in FP32 by one 16-CTA thread-block cluster; eigenvalues of
 * the tridiagonal by FP32 Sturm multisection, eigenvectors by FP32 twisted
 * factorisations, eigenvalues refined to their Rayleigh quotients; FP32
 * back-transformation and adjoints.  Eigenvalue relative error
 * ~ eps_32 cond(C) (1e-6 on the periodic training pencil).  info as for
 * neb_spectral, plus -2 = the cluster's exchange stalled (bounded wait).
 * Replaces the same reference functions as neb_spectral. */
size_t neb_spectral_mixed_workspace_bytes(int m);
int neb_spectral_mixed(int m, const double* M, const double* S, const double* c, double* lam,
                       double* V, double* G_M, double* G_S, double* loss, int* info,
                       void* workspace, size_t workspace_bytes, neb_stream_t stream);

/* K x H output weights between the hidden pencil and the K x K pencil
 * (FP64): M = W A_M W^T, S = W A_S W^T; and back: G_Mh = W^T G_M W,
 * G_Sh = W^T G_S W, gW = 2 (G_M W A_M + G_S W A_S). */
size_t neb_pencil_workspace_bytes(int K, int H);
int neb_pencil_project(int K, int H, const double* W_out, const double* A_M,
                       const double* A_S, double* M, double* S, void* workspace,
                       size_t workspace_bytes, neb_stream_t stream);
int neb_pencil_pullback(int K, int H, const double* W_out, const double* A_M,
                        const double* A_S, const double* G_M, const double* G_S,
                        double* G_Mh, double* G_Sh, double* gW_out, void* workspace,
                        size_t workspace_bytes, neb_stream_t stream);

/* Reverse pass from the hidden-Gram adjoints (2D scalar potential):
 * h_bar_x,y = 2 w h_x,y G_Mh, h_bar_lap = 2 w h_lap G_Sh, then through every
 * hidden layer (tanh-jet transpose, data and weight gradients).  gW, gb:
 * host arrays of n_hidden device pointers, overwritten (accumulate == 0) or
 * added to (point-chunked reverse passes).  Replaces
 * HB:2034-2138 backward_gradients_block_jet1/2 with HB:1115-1173 and
 * VTJ2:77-82 backward, VC:88-103. */
int neb_backward_hidden(const neb_net* net, const void* const* W, const double* G_Mh,
                        const double* G_Sh, const void* qw, int64_t n_points,
                        const void* tape, void* const* gW, void* const* gb, int accumulate,
                        void* workspace, size_t workspace_bytes, neb_stream_t stream);

/* Reverse pass from adjoint output jets psibar ([n][C][stop - start]) of
 * output rows [start, stop): gradients of every layer (output layer: rows
 * [start, stop) of gW[n_hidden], gb[n_hidden]).  NCC:142-154 Model.backward.
 * accumulate != 0 adds into gW / gb (point chunks of one objective). */
int neb_backward_output(const neb_net* net, const void* const* W, int start, int stop,
                        const void* psibar, int64_t n_points, const void* tape,
                        void* const* gW, void* const* gb, int accumulate, void* workspace,
                        size_t workspace_bytes, neb_stream_t stream);

/* Reverse pass from the K x K Gram adjoints G_M, G_S of neb_fields_gram:
 * recomputes this call's output jets and fields from the tape, field
 * adjoints 2 w u G_M, 2 w omega G_S (VTJ2:114-116, VC:94-95), their
 * transpose onto the output jets (VTJ2:102-106), then every layer.  gW, gb:
 * n_hidden + 1 device pointers; accumulate != 0 adds (point chunks). */
int neb_backward_fields(const neb_net* net, const void* const* W, const double* G_M,
                        const double* G_S, const void* qw, int64_t n_points,
                        const void* tape, void* const* gW, void* const* gb, int accumulate,
                        void* workspace, size_t workspace_bytes, neb_stream_t stream);

/* Synchronises the stream and reports whether a bounded device-side wait of
 * the tensor-core kernels gave up since the last neb_forward on this
 * workspace (NEB_ERR_TIMEOUT), i.e. whether the step's results are invalid.
 * NEB_OK for the SIMT precisions. */
int neb_check_status(const neb_net* net, int64_t n_points, void* workspace,
                     size_t workspace_bytes, neb_stream_t stream);

/* One Adam transaction over n_tensors parameter tensors (float when dtype
 * is 0, double when 1): global gradient norm, clip scale min(1, clip/norm),
 * commit only when every gradient is finite and the norm positive (device
 * flag; nothing changes otherwise), bias-corrected moments with t = number
 * of committed steps + 1.  The committed-step count is *step_counter (a
 * device int, read on the device and advanced there only when the update
 * commits, so a rejected step leaves it unchanged without a host
 * synchronisation) or, when step_counter is NULL, the host argument `step`.
 * gate (device int, may be NULL): the objective's status word; the update
 * commits only when it is 0 (the physical-validity gate of the reference's
 * device Adam transaction, HB:2184-2277 physical_valid, HB:3677-3721), so a
 * failed eigensolve or peel changes nothing without a host round trip.
 * Replaces NCC:156-171 Model.adam (epoch advanced only after a committed
 * update, NCC:157-158, 170) and HB:2184-2277 adam_step_jet1_device.
 * norm_out, committed_out: device pointers (double, int).  One shared
 * network has one parameter vector, so the clip norm is global: norm_out is
 * the single entry of what NCC returns per mode. */
size_t neb_adam_workspace_bytes(void);
int neb_adam(int dtype, int n_tensors, void* const* params, void* const* exp_avg,
             void* const* exp_avg_sq, const void* const* grads, const int64_t* sizes,
             int step, int* step_counter, const int* gate, double lr, double clip,
             double beta1, double beta2, double eps, double* norm_out, int* committed_out,
             void* workspace, size_t workspace_bytes, neb_stream_t stream);

/* Self-test of the bounded device-side wait that every tensor-core pipeline
 * uses (no counterpart in the reference, whose CuPy kernels never wait on
 * the device): one CTA waits on an mbarrier phase that completes only when
 * `arrive` is non-zero; without the arrival the wait gives up after
 * spin_limit polls (1024 .. 2^24), records the give-up in *status (device
 * int) and the call returns NEB_ERR_TIMEOUT, leaving the context usable.
 * No copy or MMA is in flight during the wait.  Synchronises the stream. */
int neb_wait_selftest(int arrive, uint32_t spin_limit, int* status, neb_stream_t stream);

/* ------------------------------------------------------------------------
 * Mode-stacked SIREN networks: the reference's own per-mode architecture.
 * K independent networks (one per mode) with weights stacked [K][out][in]
 * and biases [K][out]; hidden layers y = sin(omega (W x + b)) (omega_first on
 * the first layer, omega_hidden after), a linear output layer, the output jet
 * multiplied by an envelope jet.  Jets: order 1 = value and gradient
 * (C = 1 + dim), order 2 adds the compact Hessian (2D xx, xy, yy; 3D xx, xy,
 * xz, yy, yz, zz).  Layout per mode [n][C][width]; a block of B modes
 * [B][n][C][width]; features [n][C][widths[0]] and the envelope [n][C]
 * (one column; NULL = the identity envelope) are shared by all modes.
 * NCC:111-154 (Model, order 1, 3D) and VTJ2:26-82 (order 2, 3D). */
typedef struct neb_modes {
  int32_t dim;        /* 2 or 3 */
  int32_t order;      /* 1 or 2 */
  int32_t n_layers;   /* linear layers including the output layer, 1..NEB_MAX_HIDDEN+1 */
  int32_t widths[NEB_MAX_HIDDEN + 2]; /* widths[0] inputs .. widths[n_layers] outputs per mode */
  int32_t n_modes;    /* K: modes stacked in every parameter array */
  int32_t precision;  /* NEB_PREC_FP32 or NEB_PREC_FP64 */
  double omega_first;
  double omega_hidden;
} neb_modes;

/* Bytes of the activation tape of a block of n_block modes (scaled
 * pre-activations and outputs of every hidden layer) and of the reverse
 * pass's workspace. */
size_t neb_modes_tape_bytes(const neb_modes* net, int n_block, int64_t n_points);
size_t neb_modes_workspace_bytes(const neb_modes* net, int n_block, int64_t n_points);

/* Output jets of modes [start, stop) into out ([stop-start][n][C][widths[L]],
 * envelope applied), keeping the tape.  W, b: host arrays of n_layers device
 * pointers to the FULL stacked parameters (the call offsets to `start`).
 * Replaces NCC:130-140 Model.forward and VTJ2:65-76 forward. */
int neb_modes_forward(const neb_modes* net, int start, int stop, const void* const* W,
                      const void* const* b, const void* features, const void* envelope,
                      int64_t n_points, void* tape, size_t tape_bytes, void* out,
                      neb_stream_t stream);

/* Parameter gradients of <adjoint, output> for modes [start, stop) from the
 * tape of the matching neb_modes_forward: gW, gb are n_layers device
 * pointers to BLOCK arrays [stop-start][out][in], [stop-start][out],
 * overwritten (accumulate = 0) or added to.  NCC:142-154 Model.backward,
 * VTJ2:77-82 backward. */
int neb_modes_backward(const neb_modes* net, int start, int stop, const void* const* W,
                       const void* features, const void* envelope, int64_t n_points,
                       const void* tape, const void* adjoint, void* const* gW, void* const* gb,
                       int accumulate, void* workspace, size_t workspace_bytes,
                       neb_stream_t stream);

/* Velocity u = curl A and its gradient d_j u_a of 3D second-order vector
 * potentials (3 outputs per mode) for modes [start, stop): writes columns
 * start..stop-1 of U [3n][n_modes] (rows p*3 + a) and D [9n][n_modes] (rows
 * p*9 + a*3 + j).  VTJ2:93-101 velocity / velocity_grad; and the adjoint
 * (VC:32-38 lift): GU, GD in the same layouts -> output-jet adjoints
 * [stop-start][n][10][3]. */
int neb_velocity_fields(int precision, const void* out, int start, int stop, int64_t n_points,
                        int n_modes, void* U, void* D, neb_stream_t stream);
int neb_velocity_lift(int precision, const void* GU, const void* GD, int start, int stop,
                      int64_t n_points, int n_modes, void* adjoint, neb_stream_t stream);

/* 2D scalar potential of one output per mode with first-order jets (the
 * periodic backend's streamfunction, HB:3455-3460): value of modes
 * [start, stop) into columns of V [n][n_modes], gradient into G [2n][n_modes]
 * (rows p*2 + a); and the adjoint: dV, dG -> output-jet adjoints
 * [stop-start][n][3][1].  neb_column_center subtracts each column's mean
 * over the rows (the mean-zero gauge, HB:3461-3465, and its transpose,
 * HB:3579-3583), FP64 sums. */
int neb_potential_fields(int precision, const void* out, int start, int stop, int64_t n_points,
                         int n_modes, void* V, void* G, neb_stream_t stream);
int neb_potential_lift(int precision, const void* dV, const void* dG, int start, int stop,
                       int64_t n_points, int n_modes, void* adjoint, neb_stream_t stream);
int neb_column_center(int precision, int64_t rows, int K, void* A, neb_stream_t stream);

/* Evaluation-only forward of modes [start, stop): the same output jets as
 * neb_modes_forward, with no tape (the hidden layers' outputs alternate
 * between two buffers of the scratch and no pre-activation is kept), so a
 * block needs neb_modes_eval_scratch_bytes instead of the tape.  For
 * basis evaluation at many points (experiments/metaball/evaluate.py:100-105
 * with velocity/core.py:71-77 fields). */
size_t neb_modes_eval_scratch_bytes(const neb_modes* m, int n_block, int64_t n_points);
int neb_modes_forward_eval(const neb_modes* m, int start, int stop, const void* const* W,
                           const void* const* b, const void* features, const void* envelope,
                           int64_t n_points, void* scratch, size_t scratch_bytes, void* out,
                           neb_stream_t stream);

/* ---- Periodic evaluation of a trained basis (no counterpart entry points in
 * the reference; they replace its CuPy code at the lines cited). ----
 *
 * Fourier feature jets of order 1, 2 or 3 (3, 6 or 10 channels: value,
 * d/dx, d/dy, xx, xy, yy, xxx, xxy, xyy, yyy) of points already shifted to
 * the box origin, [n][C][4 n_freq]: sin and cos of 2 pi h s / L for s = x,
 * then y, h = 1..n_freq (HB:418-438 encoding_jet1, HB:791-809 for Jet3;
 * the reference's pi h (s_n + 1)). */
int neb_periodic_features(int precision, int order, int n_freq, double length_x,
                          double length_y, const double* points, int64_t n_points,
                          void* features, neb_stream_t stream);

/* Stream-function fields of modes [start, stop) from their output jets
 * [stop-start][n][C][1] (order 2 or 3): UV [n][2][n_modes] (u = psi_y,
 * v = -psi_x), Om [n][n_modes] (omega = -lap psi) and, with order 3 and diag
 * not NULL, diag [n][3][n_modes] (psi, -lap u, -lap v) -- the six channels of
 * evaluate_large_comparison.py:29-35. */
int neb_stream_fields(int precision, int order, const void* out, int start, int stop,
                      int64_t n_points, int n_modes, void* UV, void* Om, void* diag,
                      neb_stream_t stream);

/* In place: norm_k = sqrt(M_kk), M_ij /= norm_i norm_j, S_ij /= norm_i
 * norm_j -- the unit-velocity normalisation of every mode before the Ritz
 * stage (ROLL:173-176), applied to the Grams instead of the fields. */
int neb_normalize_pencil(int K, double* M, double* S, double* norm, neb_stream_t stream);

/* R [2][K][K]: R = D^-1 T with T[:, i] = V[i] (rows of V: M-orthonormal
 * eigenvectors, as neb_spectral writes them) and D = diag(norm), the map
 * from Ritz coefficients to coefficients of the raw fields (ROLL:187-192),
 * followed by its transpose.  The rollout entry points take this pair. */
int neb_ritz_transform(int K, const double* V, const double* norm, double* R,
                       neb_stream_t stream);

/* ETDRK4 weights coef [6][K] = (e, e2, q, f1, f2, f3) for the linear part
 * -nu lam and step h, phi functions by the 32-point contour mean (ROLL:56-64). */
int neb_etdrk4_coefficients(int K, const double* lam, double nu, double h, double* coef,
                            neb_stream_t stream);

/* Matrix-free Galerkin right-hand side in the Ritz basis (ROLL:37-41):
 * out = R^T [U^T (w omega v) - V^T (w omega u)] with (u, v, omega) =
 * (UV[:,0], UV[:,1], Om) R x, FP64 result; FP32 fields are summed with
 * compensated FP32 arithmetic.  neb_etdrk4_step advances c (FP64 [K]) by one
 * ETDRK4 step with the weights of neb_etdrk4_coefficients (ROLL:65-72);
 * neb_rollout_project gives the Ritz coefficients of a velocity field,
 * c = R^T w (U^T u0 + V^T v0) (ROLL:197); neb_rollout_fields writes
 * fields [3][n] = (u, v, omega) of the coefficients c.  No host
 * synchronisation; the step graph-captures. */
size_t neb_rollout_workspace_bytes(int64_t n_points, int K);
int neb_rollout_rhs(int precision, int64_t n_points, int K, const void* UV, const void* Om,
                    const double* R, double weight, const double* x, double* out,
                    void* workspace, size_t workspace_bytes, neb_stream_t stream);
int neb_etdrk4_step(int precision, int64_t n_points, int K, const void* UV, const void* Om,
                    const double* R, double weight, const double* coef, double* c,
                    void* workspace, size_t workspace_bytes, neb_stream_t stream);
int neb_rollout_project(int precision, int64_t n_points, int K, const void* UV, const double* R,
                        const double* u0, const double* v0, double weight, double* c,
                        void* workspace, size_t workspace_bytes, neb_stream_t stream);
int neb_rollout_fields(int precision, int64_t n_points, int K, const void* UV, const void* Om,
                       const double* R, const double* c, double* fields, void* workspace,
                       size_t workspace_bytes, neb_stream_t stream);

/* Per-mode Adam (NCC:156-171 Model.adam; HB:2184-2277 adam_step_jet1_device):
 * the clip norm of mode k runs over mode k's slice of every tensor (tensors
 * stacked [n_modes][...], sizes[i] elements in total); beta1 0.9, beta2
 * 0.999, eps 1e-8 as the reference.  The transaction commits only when the
 * gate (device int, may be NULL: the objective's status word) is 0 and
 * every active mode's norm is finite and positive; then the active modes
 * update (active: device int [n_modes], may be NULL = all) and nothing else
 * changes.  step_counter (device int): the committed steps, one shared count
 * (steps_per_mode = 0, NCC's epoch) or one per mode ([n_modes],
 * steps_per_mode = 1, HB's per-mode counts); the updated modes' counts
 * advance.  norms_out [n_modes] (device double, may be NULL), committed_out
 * (device int, may be NULL). */
size_t neb_modes_adam_workspace_bytes(int n_modes);
int neb_modes_adam(int dtype, int n_modes, int n_tensors, void* const* params,
                   void* const* exp_avg, void* const* exp_avg_sq, const void* const* grads,
                   const int64_t* sizes, int* step_counter, int steps_per_mode, const int* active,
                   const int* gate, double lr, double clip, double* norms_out,
                   int* committed_out, void* workspace, size_t workspace_bytes,
                   neb_stream_t stream);

/* G = scale A^T A (FP64, K x K) of the columns of A [rows][K] (FP32 or
 * FP64, row-major), per-chunk partials reduced in FP64; compensated != 0
 * sums FP32 products exactly paired (see NEB_GRAM_COMPENSATED).  The Grams
 * of VC:40-46 (M = U^T U / n, S = D^T D / n). */
size_t neb_column_gram_workspace_bytes(int64_t rows, int K);
int neb_column_gram(int precision, int64_t rows, int K, const void* A, double scale,
                    int compensated, double* G, void* workspace, size_t workspace_bytes,
                    neb_stream_t stream);

/* out = scale A C for A [rows][K] (FP32 or FP64) and C [K][K] FP64, both
 * row-major; out in A's type.  FP64: one DGEMM.  FP32: scale C as a sum of
 * two floats and two FP32 GEMMs with FP32 accumulation.  The field adjoints
 * U Cu / n, D Cd / n of VC:94-95 and w V Cu, w G Cd of HB:3513-3534. */
size_t neb_column_apply_workspace_bytes(int64_t rows, int K);
int neb_column_apply(int precision, int64_t rows, int K, const void* A, const double* C,
                     double scale, void* out, void* workspace, size_t workspace_bytes,
                     neb_stream_t stream);

/* Causal Rayleigh peel in Gram form, FP64 (VC:48-69 coefficient_peel):
 * order = stable ascending sort of S_kk / M_kk when sort != 0 (the
 * reference's geometry_rayleigh sorting), the identity when sort == 0 (its
 * fixed_order, HB:3471-3475); the ordered M orthonormalised
 * by a scaled Cholesky factor applied twice (T with T^T M_sorted T = I);
 * losses[r] = (T^T S_sorted T)_rr in causal order; T_out [K][K] row-major
 * with rows in mode order; Cu, Cd [K][K] with dL/dU = U Cu / n and
 * dL/dD = D Cd / n for L = sum(losses); relative_mass[r] and ortho_error
 * (device, may be NULL).  info (device int): 0 ok, 1 a Cholesky factor
 * failed (rank), 2 the gate failed: with mass_floor <= 0 the gate of VC:60-62
 * (a non-finite or non-positive loss, relative mass below 1e-4,
 * orthogonality error above 1e-5), with mass_floor > 0 the gate of the 2D
 * peel, HB:3555-3567 (a non-finite value, a raw or peeled mass at or below
 * the floor).  No host synchronisation. */
size_t neb_peel_workspace_bytes(int K);
int neb_coefficient_peel(int K, const double* M, const double* S, double mass_floor,
                         int sort, double* losses, int* order,
                         double* T_out, double* Cu, double* Cd, double* relative_mass,
                         double* ortho_error, int* info, void* workspace,
                         size_t workspace_bytes, neb_stream_t stream);

#ifdef __cplusplus
}
#endif

#endif /* NEB_GB300_H */
