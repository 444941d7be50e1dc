#!/usr/bin/env python
"""Benchmark: objective + gradient training steps/s of the periodic eigenfluid
basis at K = 1024 on GB300.

Workload (one "step"): 16,384 quadrature points drawn uniformly in [0, 2 pi)^2
from a seeded generator, 64 Fourier features with value / gradient /
Laplacian jets, 4 x 512 tanh layers, K = 1024 outputs, hidden-layer mass and
stiffness Grams, FP64 generalized eigensolve, ordering objective
sum_k lam_k / k, hand-written reverse pass and one Adam update (lr 1e-3).

Arms:
  --impl neb        (default) this library; the headline precision
                    (--precision, default bf16x3: split-BF16 tcgen05 GEMMs with
                    FP32 accumulation, FP64 reductions and eigensolve), with the
                    plain FP32 SIMT form timed beside it.
  --impl reference  the reference algorithm on the host CPU (the FP64 NumPy
                    restatement in oracle/; the reference itself is CuPy-only),
                    rank 0 only.

Multi-GPU: the step does not shard without a collective, so N GPUs run N
independent replicas (weak scaling); value = steps of all ranks / max time.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
METRIC = ("objective+grad steps/s at K=1024: TF32/BF16 vs FP32 plain, "
          "eig rel err ≤1e-4")
WORKLOAD = ("periodic_train: 2D periodic potential, 64 Fourier features (value, grad, "
            "Laplacian jets), 4x512 tanh, K=1024 outputs, 16384 uniform random points "
            "per step, ordering objective sum lam_k/k, FP64 eigensolve, Adam lr 1e-3")


# precision of each part of the headline step's spectral stage (the mixed
# stage of the split-BF16 and plain FP32 forms)
SPECTRAL_STAGES = {
    "hidden_grams": "split-BF16 products, FP32 tensor-memory sums drained every 64 points, "
                    "compensated FP32 cross-CTA reduction, FP64 result",
    "cholesky_of_M": "compensated FP32 (float pairs, ~2^-44 relative)",
    "reduction_L^-1 S L^-T": "compensated FP32 right-looking triangular solves",
    "tridiagonalisation": "FP32 Householder (one 16-CTA cluster)",
    "tridiagonal_eigenpairs": "FP32 Sturm multisection + twisted factorisations, eigenvalues "
                              "refined to compensated Rayleigh quotients",
    "back_transform_and_adjoints": "FP32 (WY back-transform, V = L^-T X by compensated solve, "
                                   "FP32 Gram-adjoint products)",
    "gram_adjoint_operand": "G_M, G_S split three ways (24 significant bits) for the "
                            "tensor-core Gram-adjoint GEMM",
}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["neb", "reference"], default="neb")
    ap.add_argument("--precision", default="bf16x3", choices=["bf16x3", "fp32", "fp64"])
    ap.add_argument("--no-fp32-plain", action="store_true")
    ap.add_argument("--no-accuracy", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--modes", default="32,1024",
                    help="mode counts of the reference_velocity / reference_potential workloads "
                         "(the largest also sets the periodic_rollout basis)")
    ap.add_argument("--grid", type=int, default=256,
                    help="grid side of the periodic_rollout workload")
    ap.add_argument("--mode-precision", default="fp32", choices=["fp32", "bf16x9", "tf32"],
                    help="per-mode network form of reference_velocity / metaball_eval: FP32 "
                         "SIMT, or the per-mode GEMMs on the tensor cores (BF16x9 emulation "
                         "of FP32 products, TF32)")
    ap.add_argument("--points", type=int, default=0,
                    help="first points of the metaball_eval workload (0: all 1,599,754)")
    ap.add_argument("--workload", default="periodic_train",
                    choices=["periodic_train", "periodic_small", "periodic_eval", "multihole",
                             "metaball3d", "reference_velocity", "reference_potential",
                             "periodic_rollout", "metaball_eval"],
                    help="periodic_train is the headline line; the others print one line "
                         "each for the remaining configurations (timing and FP64-oracle "
                         "errors), not the headline metric")
    return ap.parse_args()


def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return dict(hbm=d["hbm_gbs"], bf16=d["bf16_tflops"],
                    bf16_sustained=d.get("bf16_tflops_sustained", d["bf16_tflops"]),
                    source="measured")
    return dict(hbm=6800.0, bf16=1900.0, bf16_sustained=1700.0, source="fallback")


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 50 ms (the headline
    pass takes a few tenths of a second)."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "50"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.thread.join(timeout=2)

    def summary(self):
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                smax = float(parts[1])
            except ValueError:
                continue
            for nm, val in zip(names, parts[4:8]):
                if val.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": smax, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


# ------------------------------------------------------------- replicas
# N GPUs run N independent replicas of the step (the path has no exchange
# without an all-reduce of the Grams): each rank draws its own point batches,
# times its own steps, and rank 0 reports the whole job from the slowest rank.
def replica_seed(base_seed: int, rank: int) -> int:
    return base_seed + 1000 * rank


def max_over_ranks(x: float, world: int, device=None) -> float:
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_steps_per_s(world: int, steps: int, ms_max: float) -> float:
    return world * steps / (ms_max / 1e3)


def cpu_threads():
    return os.cpu_count() or 1


def oracle_step_time(n_points: int, seed: int = 0, step: int = 0):
    """Seconds of one FP64 oracle training step (factored route + Adam) on
    n_points of the periodic workload."""
    sys.path.insert(0, str(ROOT))
    from oracle import neb_oracle as O
    from neb_gb300 import configs as CF
    cfg = CF.CONFIGS["periodic_train"]
    params = O.glorot_init(list(cfg.widths), seed)
    mom = O.zero_moments(params)
    pts, w = CF.periodic_uniform(n_points, seed, step)
    t0 = time.perf_counter()
    X0 = O.features_periodic(pts, cfg.n_freq)
    r = O.objective_and_grad_factored(params, X0, w[0], cfg.objective)
    O.adam_step(params, mom, r.grads, 0, cfg.lr, cfg.clip)
    return time.perf_counter() - t0


def run_reference(args, world, rank):
    """The reference algorithm on the host cores: full training steps (all
    16,384 points, K = 1024, FP64 eigensolve, Adam) of the FP64 NumPy
    restatement, one warm-up step, then the timed steps."""
    if rank != 0:
        return
    full = 16384
    for _ in range(min(args.warmup, 1)):
        oracle_step_time(full)
    times = [oracle_step_time(full, seed=0, step=i) for i in range(args.steps)]
    per_step = float(np.mean(times))
    value = 1.0 / per_step
    cores = cpu_threads()
    line = {
        "metric": METRIC, "value": value, "unit": "steps/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": per_step * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic: seeded uniform random points, Glorot-normal init (seed 0)",
        "config": {"workload": WORKLOAD, "K": 1024, "points_per_step": full},
        "impl": "reference",
        "cpu_baseline": {"value": value, "unit": "steps/s", "cores": cores, "kind": "port",
                         "sample": f"{args.steps} full training steps ({full} points each, "
                                   f"FP64 NumPy restatement, {cores} BLAS threads), "
                                   "no extrapolation"},
        "e2e": {"value": value, "unit": "steps/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# ------------------------------------------------- the other configurations
def _rel_max(a, b) -> float:
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return float(np.max(np.abs(a - b)) / max(float(np.max(np.abs(b))), 1e-300))


def _grad_rel(grads, ref_grads) -> float:
    num = den = 0.0
    for gs, rs in zip(grads, zip(*ref_grads)):
        for g, r in zip(gs, rs):
            d = g.detach().cpu().double().numpy() - r
            num += float((d * d).sum())
            den += float((r * r).sum())
    return math.sqrt(num / den)


def _params64(model):
    return [(a.detach().cpu().double().numpy(), b.detach().cpu().double().numpy())
            for a, b in zip(model.W, model.b)]


def _eig_rel(lam, ref_lam) -> float:
    lam = np.asarray(lam, dtype=np.float64)
    ref_lam = np.asarray(ref_lam, dtype=np.float64)
    if lam.shape != ref_lam.shape:
        return float("nan")
    return float(np.max(np.abs(lam - ref_lam) / np.abs(ref_lam)))




def _pencil_errors(r, ref) -> dict:
    return {"rank": int(r.rank), "oracle_rank": int(ref.rank),
            "eig_rel_err_max": _eig_rel(r.eigenvalues.cpu().numpy(), ref.lam),
            "gram_M_rel_err": _rel_max(r.M.cpu().numpy(), ref.M),
            "gram_S_rel_err": _rel_max(r.S.cpu().numpy(), ref.S),
            "grad_rel_err": _grad_rel(r.grads, ref.grads),
            "loss_rel_err": abs(float(r.loss) - ref.loss) / abs(ref.loss)}


def _timed(step, W, K):
    """ms per step over K steps after W warm-up steps (CUDA events)."""
    import torch
    for i in range(W):
        step(i)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for i in range(W, W + K):
        step(i)
    e1.record()
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / K


def _kernel_table(N, step, K):
    """Per-kernel ms per step of K further steps (library timers)."""
    import torch
    torch.cuda.synchronize()
    N.timing_begin()
    for i in range(K):
        step(i)
    torch.cuda.synchronize()
    kern = N.timing_end()
    return {k: round(v[1] / K, 4) for k, v in sorted(kern.items(), key=lambda kv: -kv[1][1])[:12]}


def gram_rate(gram_ms_per_step: float, rows, K: int) -> dict:
    """Gram throughput in the symmetric-count convention: sum over the Grams
    of R * K * (K + 1) flops, R = rows of the field matrix (points x field
    components), K = its columns."""
    flops = float(sum(r * K * (K + 1) for r in rows))
    return {"tflops": flops / (gram_ms_per_step / 1e3) / 1e12 if gram_ms_per_step > 0 else None,
            "ms_per_step": gram_ms_per_step, "flops_per_step": flops,
            "convention": "sum over Grams of R*K*(K+1), R = field rows"}


def _gram_ms(kern_ms: dict) -> float:
    return sum(v for k, v in kern_ms.items() if k in ("tc_gram", "simt_gram"))


# The reference's own 3D velocity training configuration
# (experiments/metaball/configs/metaball-velocity-k1024-seed0.json): K
# per-mode SIRENs of 5 x 128 sine layers (omega 40 / 36) on 15 input
# features, vector potentials (3 outputs), second-order jets, 6,144 points
# per step, the Gram-form causal peel, Adam (lr 2.8e-5, clip 8).  Its
# published per-update stage means at K = 1024 (data/paper/
# initial_capacity_training.json:83-92, hardware not stated) sum to 11.94 s.
REF_VELOCITY = dict(hidden=128, hidden_layers=5, siren_first_omega0=40.0,
                    siren_hidden_omega0=36.0, points=6144, lr=2.8e-5, clip=8.0,
                    published_s_per_update_k1024=2.698278 + 8.952445 + 0.265934 + 0.018048)


# The reference's periodic vortex-merger Potential training configuration
# (checkpoints/2d/periodic-potential-k1024-seed0/model.json): K per-mode
# SIRENs 24 -> 4 x 32 sine (omega 8/30) -> 1, 6 Fourier frequencies, 4096
# uniform points per update, the streamfunction Rayleigh peel, Adam (clip 5,
# cosine schedule from 2e-4).  Published: 2,000 updates in 6,228-6,599 s at
# K = 1024 (data/paper/periodic_merger.json:26,1297,2568; hardware not stated).
REF_POTENTIAL = dict(modes=1024, hidden=32, hidden_layers=4, frequencies=6, input_features=24,
                     xmin=0.0, xmax=2 * math.pi, ymin=0.0, ymax=2 * math.pi,
                     geometry_mode="periodic_box", envelope_mode="periodic_identity",
                     input_encoding="periodic_sincos_xy", canonical_siren=True,
                     siren_first_omega0=8.0, siren_hidden_omega0=30.0,
                     basis_objective="potential_rayleigh", causal_sorting="geometry_rayleigh",
                     reorthogonalization_passes=2, mass_floor=1e-14, learning_rate=2e-4,
                     grad_clip=5.0, spatial_derivative_order=1, mode_forward_batch=32,
                     mode_backward_batch=32, mlp_compute_dtype="float32",
                     sampling_mode="uniform_random", points_per_step=4096, seed=0)
PUBLISHED_POTENTIAL_S_PER_UPDATE = (6228.0 / 2000, 6599.0 / 2000)


def time_potential(K: int, steps: int, warmup: int, dev, precision: str = "fp32"):
    """ms per training update of the reference's Potential configuration at
    K modes through the periodic backend's API (hardcoded.peel_step): each
    update samples its points on the host (fluid_points, seed + 1009 epoch,
    as the trainer does), uploads them, and reads the diagnostics back.
    Returns (ms per update, last result)."""
    import torch
    from types import SimpleNamespace
    from neb_gb300 import hardcoded as H
    cfg = SimpleNamespace(**dict(REF_POTENTIAL, modes=K))
    model = H.HardcodedModel(cfg, H.initial_arrays(cfg), precision=precision, device=dev)
    n = cfg.points_per_step

    def step(epoch):
        pts = H.fluid_points(cfg, n, 0.0, 0.0, cfg.seed + epoch * 1009)
        return H.peel_step(cfg, model, pts, 0.0, 0.0, True)

    for e in range(warmup):
        step(e)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for e in range(warmup, warmup + steps):
        r = step(e)
    e1.record()
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / steps, r, step


# The reference's frozen-basis evaluation of the periodic Potential basis at
# K = 1024 (experiments/periodic/paper_rollout.py, evaluate_large_comparison
# fields): Jet3 sampling on the 256^2 grid and the Gram + Ritz stage, published
# as 142-150 s and 1.61-1.73 s (data/paper/periodic_merger.json:1280-1281 and
# the five other records; hardware not stated).  The rollout integrates the
# vortex merger to T = 18 pi at dt = 0.005 (paper_rollout.py main).
PUBLISHED_SAMPLING_S = (142.0, 150.0)
PUBLISHED_RITZ_S = (1.61, 1.73)


def vortex_pair(points: np.ndarray, separation: float = 1.35, core: float = 0.3):
    """Velocity of two co-rotating Gaussian vortices a separation apart about
    the box centre (a synthetic stand-in for the merger's initial DNS field):
    psi = sum_j exp(-|x - x_j|^2 / (2 core^2)), (u, v) = (psi_y, -psi_x)."""
    c = np.array([math.pi, math.pi])
    u = np.zeros(len(points))
    v = np.zeros(len(points))
    for sgn in (-1.0, 1.0):
        d = points - (c + sgn * np.array([separation / 2, 0.0]))
        g = np.exp(-(d ** 2).sum(1) / (2 * core * core))
        u += -d[:, 1] / core ** 2 * g
        v += d[:, 0] / core ** 2 * g
    return u, v


def velocity_inputs(n: int, seed: int = 0):
    """Synthetic inputs with the configuration's shapes: points uniform in
    the unit cube; features (2x - 1 for the coordinates, 12 constant
    geometry codes in [-1, 1]) with their jets; a smooth bubble envelope
    prod_a 4 x_a (1 - x_a) with analytic gradient and Hessian.  Channel-
    first [10, n, F] arrays."""
    rng = np.random.default_rng(seed)
    x = rng.random((n, 3))
    return velocity_features(x, rng.uniform(-1, 1, 12))


def velocity_features(x: np.ndarray, codes: np.ndarray):
    """Feature and envelope jets of points x [n, 3] in the unit cube with
    the 12 geometry codes (see velocity_inputs)."""
    n = len(x)
    X0 = np.zeros((10, n, 15))
    X0[0, :, :3] = 2 * x - 1
    X0[0, :, 3:] = codes[None]
    for a in range(3):
        X0[1 + a, :, a] = 2.0
    f = 4 * x * (1 - x)
    df = 4 - 8 * x
    E = np.zeros((10, n, 1))
    E[0, :, 0] = f.prod(1)
    for a in range(3):
        E[1 + a, :, 0] = df[:, a] * np.prod(np.delete(f, a, 1), 1)
    pairs = [(0, 0), (0, 1), (0, 2), (1, 1), (1, 2), (2, 2)]
    for k, (i, j) in enumerate(pairs):
        if i == j:
            E[4 + k, :, 0] = -8 * np.prod(np.delete(f, i, 1), 1)
        else:
            E[4 + k, :, 0] = df[:, i] * df[:, j] * f[:, 3 - i - j]
    return X0, E


def time_velocity(K: int, steps: int, warmup: int, dev, block: int = 256,
                  precision: str = "fp32"):
    """ms per training step (velocity objective + gradient + Adam) of the
    reference's velocity configuration at K modes, CUDA events."""
    import torch
    from types import SimpleNamespace
    from neb_gb300 import ModeModel
    from neb_gb300.training import velocity_train_step
    c = SimpleNamespace(**{k: REF_VELOCITY[k] for k in ("hidden", "hidden_layers",
                                                       "siren_first_omega0",
                                                       "siren_hidden_omega0")})
    model = ModeModel(c, K=K, seed=0, inputs=15, outputs=3, dim=3, order=2, device=dev,
                      precision=precision)
    X0, E = velocity_inputs(REF_VELOCITY["points"])
    feats = torch.tensor(np.moveaxis(X0, 0, 1), dtype=torch.float32, device=dev).contiguous()
    env = torch.tensor(np.moveaxis(E, 0, 1), dtype=torch.float32, device=dev).contiguous()
    data = SimpleNamespace(features=feats, envelope=env)

    def step():
        return velocity_train_step(model, data, REF_VELOCITY["lr"], REF_VELOCITY["clip"],
                                   block=block)

    for _ in range(warmup):
        step()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(steps):
        r = step()
    e1.record()
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / steps, int(r["info"].item())


def run_workload(args, world, rank, local):
    """One line per configuration other than the headline: device-timed
    steps, the plain FP32 form where the configuration asks for it, and the
    errors of eigenvalues, Gram entries and gradients against the FP64
    oracle on the same seeded inputs."""
    import torch
    sys.path.insert(0, str(ROOT))
    from neb_gb300 import CONFIGS, Model, spectral_step, train_step
    from neb_gb300 import _native as N
    from neb_gb300 import configs as CF
    from oracle import neb_oracle as O

    if rank != 0:
        return
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    name = args.workload
    W, K = max(args.warmup, 1), args.steps
    line = {"workload": name, "n_gpus": 1, "steps": K, "warmup": W}
    if name in CONFIGS:
        cfg = CONFIGS[name]
        line.update({"data": "synthetic: seeded samples of the configuration, Glorot-normal "
                             "init", "widths": list(cfg.widths), "objective": cfg.objective})

    def dev_inputs(pts, w):
        return torch.tensor(pts, device=dev), torch.tensor(w, device=dev)

    if name == "metaball_eval":
        # the reference's 3D basis evaluation (experiments/metaball/evaluate.py,
        # Velocity): u = curl of every mode's vector potential, with the
        # second-order forward of velocity/core.py fields, at all points of
        # the metaball region; published 488 s (K = 512) and 748 s (K = 1024)
        # including the streamed FP64 output (data/paper_results/
        # primary_basis_runtime.csv:8-9, hardware not stated)
        from types import SimpleNamespace
        from neb_gb300 import ModeModel
        from neb_gb300.modes import velocity_fields
        Km = max(int(k) for k in args.modes.split(","))
        c = SimpleNamespace(**{k: REF_VELOCITY[k] for k in ("hidden", "hidden_layers",
                                                           "siren_first_omega0",
                                                           "siren_hidden_omega0")})
        model = ModeModel(c, K=Km, seed=0, inputs=15, outputs=3, dim=3, order=2, device=dev,
                          precision=args.mode_precision)
        pts, _ = CF.sample(CONFIGS["metaball3d"])
        if args.points:
            pts = pts[:int(args.points)]
        n = len(pts)
        codes = np.random.default_rng(1).uniform(-1, 1, 12)
        chunk, block = 65536, 32
        host_u = torch.empty((3 * min(chunk, n), Km), dtype=torch.float32, pin_memory=True)
        warm = velocity_features(pts[:1024], codes)
        velocity_fields(model, SimpleNamespace(
            features=torch.tensor(np.moveaxis(warm[0], 0, 1), dtype=torch.float32, device=dev),
            envelope=torch.tensor(np.moveaxis(warm[1], 0, 1), dtype=torch.float32, device=dev)),
            block=block)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for a in range(0, n, chunk):
            X0, E = velocity_features(pts[a:a + chunk], codes)
            data = SimpleNamespace(
                features=torch.tensor(np.moveaxis(X0, 0, 1), dtype=torch.float32, device=dev),
                envelope=torch.tensor(np.moveaxis(E, 0, 1), dtype=torch.float32, device=dev))
            U, _ = velocity_fields(model, data, block=block)
            host_u[:U.shape[0]].copy_(U, non_blocking=True)  # the streamed output
        e1.record()
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
        flops = 2.0 * n * 10 * Km * sum(a * b for a, b in zip(model.widths[:-1], model.widths[1:]))
        pub = {512: 488.2863621, 1024: 747.6812867}.get(Km)
        line.update({
            "metric": "3D basis evaluation: velocity (curl of every mode's vector potential) "
                      "of the reference's per-mode SIREN (5x128 sine, omega 40/36, second-order "
                      "jets) at every point of the metaball region",
            "value": wall, "unit": "s", "higher_is_better": False, "modes": Km, "points": n,
            "device_s": e0.elapsed_time(e1) / 1e3, "forward_tflops": flops / wall / 1e12,
            "mode_precision": args.mode_precision,
            "dtype": "f32", "output": "U [3 n, K] FP32 streamed to pinned host memory per "
                                      "65,536-point chunk",
            "published_reference_s": pub,
            "speedup_vs_published": pub / wall if pub and n == 1599754 else None,
            "data": "synthetic: the metaball configuration's 1,599,754 seeded points, 12 "
                    "constant geometry codes, a bubble envelope; reference initialisation"})
    elif name == "periodic_rollout":
        # frozen-basis evaluation of the reference's periodic Potential
        # network at K = 1024: Jet3 sampling on the grid, Ritz, ETDRK4
        from types import SimpleNamespace
        from neb_gb300 import hardcoded as H
        from neb_gb300.rollout import Rollout, grid_points, ritz, sample_basis
        grid = int(args.grid)
        cfg = SimpleNamespace(**dict(REF_POTENTIAL,
                                     modes=max(int(k) for k in args.modes.split(","))))
        model = H.HardcodedModel(cfg, H.initial_arrays(cfg), device=dev)
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(6)]
        # warm-up: kernel attributes, the allocator, the cuSOLVER / cuBLAS handles
        try:
            ritz(sample_basis(model, cfg, 64))
        except ArithmeticError:
            pass
        torch.cuda.synchronize()
        ev[0].record()
        gb = sample_basis(model, cfg, grid, diagnostics=True)
        ev[1].record()
        model.core._bufs.clear()  # the sampling tape is not needed any more
        torch.cuda.empty_cache()
        rb = ritz(gb)
        ev[2].record()
        roll = Rollout(gb, rb, 1e-3)
        pts = grid_points(grid, cfg)
        u0, v0 = vortex_pair(pts)
        c0 = roll.project(u0, v0)
        roll.c.copy_(c0)
        roll._set_step(0.005)
        roll.advance(2)  # graph capture and warm-up
        torch.cuda.synchronize()
        nsteps = max(20, args.steps * 10)
        ev[3].record()
        roll.advance(nsteps)
        ev[4].record()
        torch.cuda.synchronize()
        skew = roll.energy_skew()
        kern_ritz = _kernel_table(N, lambda i: ritz(gb), 1)
        kern_step = _kernel_table(N, lambda i: roll.rhs(roll.c), 3)
        t_sample = ev[0].elapsed_time(ev[1]) / 1e3
        t_ritz = ev[1].elapsed_time(ev[2]) / 1e3
        ms_step = ev[3].elapsed_time(ev[4]) / nsteps
        steps_total = int(math.ceil(18 * math.pi / 0.005))
        line.update({
            "metric": "frozen-basis evaluation of the reference's periodic Potential basis "
                      "(K=1024 per-mode SIRENs 24 -> 4x32 sine): Jet3 sampling and Gram + Ritz "
                      "on the 256^2 grid, ETDRK4 Galerkin steps",
            "value": 1e3 / ms_step, "unit": "ETDRK4 steps/s", "dtype": "f32 fields, f64 "
            "coefficients", "sampling_s": t_sample, "published_sampling_s": PUBLISHED_SAMPLING_S,
            "ritz_s": t_ritz, "published_ritz_s": PUBLISHED_RITZ_S,
            "speedup_sampling_vs_published": [PUBLISHED_SAMPLING_S[0] / t_sample,
                                              PUBLISHED_SAMPLING_S[1] / t_sample],
            "speedup_ritz_vs_published": [PUBLISHED_RITZ_S[0] / t_ritz,
                                          PUBLISHED_RITZ_S[1] / t_ritz],
            "ms_per_etdrk4_step": ms_step, "steps_timed": nsteps,
            "trajectory_T18pi_dt0005_s": ms_step * steps_total / 1e3,
            "energy_skew": skew, "ritz_lambda_min_max": [float(rb.lam[0]), float(rb.lam[-1])],
            "ritz_kernel_ms": kern_ritz, "rhs_kernel_ms": kern_step,
            "points": grid * grid, "modes": model.core.K,
            "data": "synthetic: the reference trainer's epoch-0 initialisation (no trained "
                    "checkpoint is available), a Gaussian vortex pair as the initial velocity"})
    elif name == "reference_potential":
        # the reference's own 2D training configuration through its backend
        # API: GPU updates at each K, and the FP64 oracle's update at K = 32
        from types import SimpleNamespace
        from neb_gb300 import hardcoded as H
        out = {}
        psteps = max(2, min(args.steps, 10))
        modes = [int(k) for k in args.modes.split(",")]
        for Km in modes:
            ms, r, step = time_potential(Km, psteps, 2, dev, precision=args.mode_precision)
            out[f"K{Km}"] = {"ms_per_update": ms, "updates_per_s": 1e3 / ms, "steps": psteps,
                             "loss": r["loss"], "orth_error": r["orth_error"]}
            if Km == max(modes):
                out[f"K{Km}"]["kernel_ms_per_update"] = _kernel_table(
                    N, lambda i: step(1000 + i), 2)
        top = f"K{max(modes)}"
        cpu = None
        if not args.no_cpu_baseline:
            cfg = SimpleNamespace(**dict(REF_POTENTIAL, modes=32))
            arr = H.initial_arrays(cfg)
            labels = [f"l{i}" for i in range(cfg.hidden_layers)] + ["output"]
            Wn = [np.stack([arr[f"m{k:03d}.{lab}.weight"] for k in range(32)]).astype(np.float64)
                  for lab in labels]
            bn = [np.stack([arr[f"m{k:03d}.{lab}.bias"] for k in range(32)]).astype(np.float64)
                  for lab in labels]
            pts = H.fluid_points(cfg, cfg.points_per_step, 0.0, 0.0, cfg.seed).astype(np.float64)
            t0 = time.perf_counter()
            O.potential_peel_step(Wn, bn, O.features_periodic(pts, cfg.frequencies)[:3],
                                  (2 * math.pi) ** 2 / len(pts),
                                  O.mode_omegas(cfg.hidden_layers + 1, 8.0, 30.0),
                                  lr=cfg.learning_rate, clip=cfg.grad_clip)
            t_cpu = time.perf_counter() - t0
            cpu = {"value": 1.0 / t_cpu, "unit": "updates/s", "cores": cpu_threads(),
                   "kind": "port", "sample": "1 training update at K=32 of the FP64 NumPy "
                   "restatement (potential_peel_step)"}
        lo, hi = PUBLISHED_POTENTIAL_S_PER_UPDATE
        line.update({
            "metric": "Potential (streamfunction Rayleigh peel) training updates/s through the "
                      "periodic backend API, the reference's per-mode SIREN (24 -> 4x32 sine, "
                      "omega 8/30), 4096 points per update",
            "value": out[top]["updates_per_s"], "unit": "updates/s",
            "ms_per_update": out[top]["ms_per_update"], "dtype": "f32", "modes": out,
            "mode_precision": args.mode_precision,
            "e2e_note": "each update samples its points on the host, uploads them and reads "
                        "the diagnostic table back, as the reference's trainer does",
            "published_reference_s_per_update_k1024": [lo, hi],
            "speedup_vs_published_k1024": [lo / (out["K1024"]["ms_per_update"] / 1e3),
                                           hi / (out["K1024"]["ms_per_update"] / 1e3)]
            if "K1024" in out else None,
            "cpu_baseline": cpu,
            "data": "synthetic: the reference trainer's epoch-0 initialisation and its "
                    "uniform point sampler"})
    elif name == "reference_velocity":
        # the reference's own architecture and objective: GPU steps at K = 32
        # and K = 1024, and the FP64 oracle's step at K = 32 on the host
        out = {}
        vsteps = max(1, min(args.steps, 5))
        modes = [int(k) for k in args.modes.split(",")]
        for K in modes:
            ms, info = time_velocity(K, vsteps, 1, dev, precision=args.mode_precision)
            out[f"K{K}"] = {"ms_per_step": ms, "steps_per_s": 1e3 / ms, "steps": vsteps,
                            "peel_info": info}
        top = f"K{max(modes)}"
        from types import SimpleNamespace
        from neb_gb300.modes import siren_init
        c = SimpleNamespace(**{k: REF_VELOCITY[k] for k in ("hidden", "hidden_layers",
                                                           "siren_first_omega0",
                                                           "siren_hidden_omega0")})
        cpu = None
        if not args.no_cpu_baseline:
            Wn, bn = siren_init(c, 32, 0, 15, 3)
            X0, E = velocity_inputs(REF_VELOCITY["points"])
            t0 = time.perf_counter()
            O.velocity_step([w.astype(np.float64) for w in Wn],
                            [x.astype(np.float64) for x in bn], X0, E,
                            O.mode_omegas(6, 40.0, 36.0))
            t_cpu = time.perf_counter() - t0
            cpu = {"value": 1.0 / t_cpu, "unit": "steps/s", "cores": cpu_threads(),
                   "kind": "port", "sample": "1 objective+gradient step at K=32 of the FP64 "
                   "NumPy restatement (velocity_step)"}
        line.update({
            "metric": "velocity objective+grad+Adam steps/s, the reference's per-mode SIREN "
                      "(5x128 sine, omega 40/36), 6144 points, causal peel",
            "value": out[top]["steps_per_s"], "unit": "steps/s",
            "ms_per_step": out[top]["ms_per_step"], "dtype": "f32", "modes": out,
            "mode_precision": args.mode_precision,
            "published_reference_s_per_update_k1024": REF_VELOCITY["published_s_per_update_k1024"],
            "speedup_vs_published_k1024": (REF_VELOCITY["published_s_per_update_k1024"]
                                           / (out["K1024"]["ms_per_step"] / 1e3))
            if "K1024" in out else None,
            "cpu_baseline": cpu,
            "data": "synthetic: uniform points in the unit cube, coordinate features with 12 "
                    "constant geometry codes, bubble envelope; reference initialisation"})
    elif name == "periodic_small":
        pts, w = CF.sample(cfg)
        dp, dw = dev_inputs(pts, w)
        model = Model(cfg, precision="fp64", seed=0, device=dev)
        ms = _timed(lambda i: train_step(model, dp, dw, check=False), W, K)
        kern = _kernel_table(N, lambda i: train_step(model, dp, dw, check=False), 2)
        m0 = Model(cfg, precision="fp64", seed=0, device=dev)
        r = spectral_step(m0, dp, dw, training=True, return_grams=True)
        X0 = O.features_periodic(pts, cfg.n_freq, cfg.period)
        t0 = time.perf_counter()
        ref = O.objective_and_grad(_params64(m0), X0, w, 2, cfg.objective)
        O.adam_step(_params64(m0), O.zero_moments(_params64(m0)), ref.grads, 0, cfg.lr, cfg.clip)
        t_cpu = time.perf_counter() - t0
        line.update({
            "metric": "objective+grad steps/s, FP64, K=64, 64^2 grid (trace objective)",
            "value": 1e3 / ms, "unit": "steps/s", "ms_per_step": ms, "dtype": "f64",
            "kernels_ms_per_step": kern,
            "accuracy": {"eig_rel_err_max": _eig_rel(r.eigenvalues.cpu().numpy(), ref.lam),
                         "gram_M_rel_err": _rel_max(r.M.cpu().numpy(), ref.M),
                         "gram_S_rel_err": _rel_max(r.S.cpu().numpy(), ref.S),
                         "grad_rel_err": _grad_rel(r.grads, ref.grads),
                         "loss_rel_err": abs(float(r.loss) - ref.loss) / abs(ref.loss)},
            "cpu_baseline": {"value": 1.0 / t_cpu, "unit": "steps/s", "cores": cpu_threads(),
                             "kind": "port", "sample": "1 full step of the FP64 NumPy "
                             "restatement (direct K x K route) + Adam"}})
    elif name == "periodic_eval":
        pts, w = CF.sample(cfg)
        dp, dw = dev_inputs(pts, w)
        n = len(w)
        X0 = O.features_periodic(pts, cfg.n_freq, cfg.period)
        arms, acc = {}, {}
        for prec in ("bf16x3", "fp32"):
            model = Model(cfg, precision=prec, seed=0, device=dev)
            step = (lambda i, m=model: spectral_step(m, dp, dw, training=False,
                                                     return_grams=True, check=False))
            ms = _timed(step, W, K)
            arms[prec] = {"ms_per_step": ms, "steps_per_s": 1e3 / ms,
                          "point_mode_evals_per_s": n * cfg.K / (ms / 1e3),
                          "kernels_ms_per_step": _kernel_table(N, step, 2)}
        for seed in (0, 1, 2):
            ref = None
            for prec in ("bf16x3", "fp32"):
                model = Model(cfg, precision=prec, seed=seed, device=dev)
                r = spectral_step(model, dp, dw, training=False, return_grams=True)
                if ref is None:
                    ref = O.objective_and_grad_factored(_params64(model), X0, w, cfg.objective,
                                                        want_grad=False)
                acc[f"{prec}_seed{seed}"] = {
                    "eig_rel_err_max": _eig_rel(r.eigenvalues.cpu().numpy(), ref.lam),
                    "gram_M_rel_err": _rel_max(r.M.cpu().numpy(), ref.M),
                    "gram_S_rel_err": _rel_max(r.S.cpu().numpy(), ref.S),
                    "n_eigenvalues": int(r.rank)}
        ms = arms["bf16x3"]["ms_per_step"]
        H = cfg.widths[-2]  # hidden Grams (factored route)
        for prec in arms:
            arms[prec]["gram"] = gram_rate(_gram_ms(arms[prec]["kernels_ms_per_step"]),
                                           (2 * n, n), H)
        line.update({
            "gram": arms["bf16x3"]["gram"],
            "metric": "forward + Gram + eigensolve steps/s, K=1024, 256^2 grid",
            "value": 1e3 / ms, "unit": "steps/s", "ms_per_step": ms, "dtype": "bf16x3",
            "point_mode_evals_per_s": n * cfg.K / (ms / 1e3),
            "fp32_plain": arms["fp32"], "split_bf16": arms["bf16x3"],
            "speedup_vs_fp32_plain": arms["fp32"]["ms_per_step"] / ms, "accuracy": acc})
    elif name == "multihole":
        pts, w = CF.sample(cfg)
        dp, dw = dev_inputs(pts, w)
        X0 = O.features_multihole(pts, np.asarray(cfg.centres))
        arms, acc, ref, t_cpu = {}, {}, {}, None
        # errors at each form's own rank tolerance (model.RANK_RTOL), the
        # oracle solving the same pencil at the same tolerance
        for prec in ("bf16x3", "fp32", "fp64"):
            model = Model(cfg, precision=prec, seed=0, device=dev)
            if prec != "fp64":
                step = (lambda i, m=model: train_step(m, dp, dw, check=False))
                ms = _timed(step, W, K)
                arms[prec] = {"ms_per_step": ms, "steps_per_s": 1e3 / ms, "gram": model.gram,
                              "kernels_ms_per_step": _kernel_table(N, step, 2)}
            m0 = Model(cfg, precision=prec, seed=0, device=dev)
            rt = m0.rank_rtol
            if rt not in ref:
                t0 = time.perf_counter()
                ref[rt] = O.objective_and_grad_factored(_params64(m0), X0, w, cfg.objective,
                                                        rank_rtol=rt)
                t_cpu = time.perf_counter() - t0
            r = spectral_step(m0, dp, dw, training=True, return_grams=True)
            acc[f"{prec}_rank_rtol_{rt:g}"] = _pencil_errors(r, ref[rt])
        ms = arms["bf16x3"]["ms_per_step"]
        H, n = cfg.widths[-2], len(w)  # hidden Grams (factored route)
        for prec in arms:
            arms[prec]["gram"] = gram_rate(_gram_ms(arms[prec]["kernels_ms_per_step"]),
                                           (2 * n, n), H)
        line.update({
            "gram": arms["bf16x3"]["gram"],
            "metric": "objective+grad steps/s, K=1024, multiply connected domain, 200k points",
            "value": 1e3 / ms, "unit": "steps/s", "ms_per_step": ms, "dtype": "bf16x3",
            "fp32_plain": arms["fp32"], "split_bf16": arms["bf16x3"],
            "speedup_vs_fp32_plain": arms["fp32"]["ms_per_step"] / ms, "accuracy": acc,
            "cpu_baseline": {"value": 1.0 / t_cpu, "unit": "steps/s", "cores": cpu_threads(),
                             "kind": "port", "sample": "1 full step (200,000 points) of the "
                             "FP64 NumPy restatement, factored route, without Adam"}})
    elif name == "metaball3d":
        pts, w = CF.sample(cfg)
        dp, dw = dev_inputs(pts, w)
        n = len(w)
        forms = {}
        for prec in ("tf32", "bf16x9", "fp32"):
            model = Model(cfg, precision=prec, seed=0, device=dev)

            def step(i, model=model):
                r = spectral_step(model, dp, dw, training=True, check=False)
                model.adam_async(*r.grads, lr=cfg.lr, clip=cfg.clip)
                return r

            t = _timed(step, W, K)
            forms[prec] = {"ms_per_step": t, "steps_per_s": 1e3 / t}
        ms = forms["fp32"]["ms_per_step"]
        kern = _kernel_table(N, step, 1)
        r_full = spectral_step(Model(cfg, precision="fp32", seed=0, device=dev), dp, dw,
                               training=False)
        # errors on a seeded subsample that the FP64 oracle finishes in about a minute
        sub = np.random.default_rng(7).choice(n, size=min(n, 8192), replace=False)
        ps, ws_ = pts[sub], w[sub] * (n / len(sub))
        X0 = O.features_raw3d(ps)
        acc = {}
        for prec in ("tf32", "bf16x9", "fp32", "fp64"):
            m0 = Model(cfg, precision=prec, seed=0, device=dev)
            rt = m0.rank_rtol
            ref = O.objective_and_grad(_params64(m0), X0, ws_, 3, cfg.objective, rank_rtol=rt)
            r = spectral_step(m0, torch.tensor(ps, device=dev), torch.tensor(ws_, device=dev),
                              training=True)
            acc[f"{prec}_rank_rtol_{rt:g}"] = _pencil_errors(r, ref)
        line.update({
            "metric": "objective+grad steps/s, 3D curl basis K=512, 1,599,754 points",
            "value": 1e3 / ms, "unit": "steps/s", "ms_per_step": ms, "dtype": "f32",
            "forms": forms, "tf32_vs_fp32": ms / forms["tf32"]["ms_per_step"],
            "bf16x9_vs_fp32": ms / forms["bf16x9"]["ms_per_step"],
            "points": n, "chunk_points": 1 << 17, "rank_at_init": int(r_full.rank),
            "kernels_ms_per_step": kern, "accuracy_subsample_8192": acc,
            "gram": gram_rate(_gram_ms(kern), (3 * n, 3 * n), cfg.K),
            "note": "fp32: SIMT kernels; tf32 / bf16x9: the same with the layer GEMMs on the "
                    "tensor cores (cuBLAS, TF32 inputs or the BF16x9 emulation of FP32 "
                    "products); point-chunked recompute and compensated Grams; at "
                    "Glorot init the curl fields are nearly dependent, so M is numerically "
                    "singular and the pencil is solved on range(M) in FP64 at the form's rank "
                    "tolerance"})
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    world, rank, local = dist_env()
    if args.impl == "reference":
        run_reference(args, world, rank)
        return
    if args.workload != "periodic_train":
        run_workload(args, world, rank, local)
        return
    import torch
    import torch.distributed as dist
    sys.path.insert(0, str(ROOT))
    from neb_gb300 import CONFIGS, Model, spectral_step, train_step
    from neb_gb300 import _native as N
    from neb_gb300 import configs as CF

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if world > 1:
        dist.init_process_group("nccl", device_id=dev)

    def barrier():
        if world > 1:
            dist.barrier()

    def max_ms(x: float) -> float:
        return max_over_ranks(x, world, dev)

    cfg = CONFIGS["periodic_train"]
    K, W = args.steps, args.warmup
    n = cfg.n_points
    batches = [CF.sample(cfg, step=s, seed=replica_seed(cfg.seed, rank)) for s in range(K + W)]
    dev_batches = [(torch.tensor(p, device=dev), torch.tensor(w, device=dev, dtype=torch.float32))
                   for p, w in batches]

    def device_timed(precision, timing=False, spectral=None, config=None, batches=None):
        model = Model(config or cfg, precision=precision, seed=0, device=dev, spectral=spectral)
        batches = batches or dev_batches
        for s in range(W):
            train_step(model, *batches[s % len(batches)], check=False)
        torch.cuda.synchronize()
        barrier()
        torch.cuda.synchronize()
        launches0 = N.kernel_launches()
        if timing:
            N.timing_begin()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for s in range(W, W + K):
            res = train_step(model, *batches[s % len(batches)], check=False)
        e1.record()
        torch.cuda.synchronize()
        kernels = N.timing_end() if timing else None
        launches = N.kernel_launches() - launches0
        barrier()
        ms = e0.elapsed_time(e1)
        return model, res, ms, kernels, launches

    pk = peaks()
    # the headline runs without the library's per-kernel timers (their CUDA
    # events sit between kernels); a second pass over the same steps fills
    # the kernel table and the roofline
    with ClockSampler(local) as clocks:
        model, res, ms, _, launches = device_timed(args.precision, timing=False)
    _, _, _, kernels, _ = device_timed(args.precision, timing=True)
    ms_max = max_ms(ms)
    value = whole_job_steps_per_s(world, K, ms_max)
    clk = clocks.summary()
    info_ok = int(res.info.item()) == 0

    # plain FP32 SIMT form beside it (the ratio's denominator)
    fp32 = None
    if not args.no_fp32_plain and args.precision != "fp32":
        _, _, ms32, _, _ = device_timed("fp32")
        ms32 = max_ms(ms32)
        fp32 = {"value": world * K / (ms32 / 1e3), "ms_per_step": ms32 / K}

    # both forms again with the strict FP64 spectral stage (cuSOLVER Dsygvd
    # and FP64 adjoint products) in place of the mixed one, so the cost of an
    # FP64-datatype eigensolve is visible beside the headline ratio
    strict = None
    if not args.no_fp32_plain and args.precision != "fp32":
        _, _, ms_s, _, _ = device_timed(args.precision, spectral="fp64")
        _, _, ms_s32, _, _ = device_timed("fp32", spectral="fp64")
        ms_s, ms_s32 = max_ms(ms_s), max_ms(ms_s32)
        strict = {"spectral": "fp64 (cuSOLVER Dsygvd, cuBLAS FP64 adjoints)",
                  args.precision: {"value": world * K / (ms_s / 1e3), "ms_per_step": ms_s / K},
                  "fp32": {"value": world * K / (ms_s32 / 1e3), "ms_per_step": ms_s32 / K},
                  "speedup_vs_fp32_plain": ms_s32 / ms_s}

    # the reference's own per-mode architecture and causal peel at its K =
    # 1024 velocity configuration (beside its published per-update time)
    ref_arch = None
    if not args.no_fp32_plain and world == 1:
        ms_v, info_v = time_velocity(1024, 2, 1, dev)
        ref_arch = {"workload": "reference velocity configuration: K=1024 per-mode SIRENs "
                                "(5x128 sine, omega 40/36), 6144 points, second-order jets, "
                                "Gram-form causal peel, Adam; FP32 SIMT mode kernels",
                    "value": 1e3 / ms_v, "unit": "steps/s", "ms_per_step": ms_v,
                    "peel_info": info_v,
                    "published_reference_s_per_update": REF_VELOCITY[
                        "published_s_per_update_k1024"],
                    "published_hardware": "not stated (16 GB-class GPU guard)"}

    # objective + gradient + Adam on the 256^2 periodic grid (65,536 points,
    # the grid of the evaluation configuration), both forms
    grid256 = None
    if not args.no_fp32_plain and args.precision != "fp32":
        gcfg = CONFIGS["periodic_eval"]
        gp, gw = CF.sample(gcfg)
        gb = [(torch.tensor(gp, device=dev), torch.tensor(gw, device=dev, dtype=torch.float32))]
        _, _, ms_g, _, _ = device_timed(args.precision, config=gcfg, batches=gb)
        _, _, ms_g32, _, _ = device_timed("fp32", config=gcfg, batches=gb)
        ms_g, ms_g32 = max_ms(ms_g), max_ms(ms_g32)
        grid256 = {"workload": "periodic 256^2 grid (65,536 points), 4x512 tanh, K=1024, "
                               "ordering objective, reverse pass and Adam per step",
                   "value": world * K / (ms_g / 1e3), "unit": "steps/s", "ms_per_step": ms_g / K,
                   "fp32_plain": {"value": world * K / (ms_g32 / 1e3), "ms_per_step": ms_g32 / K},
                   "speedup_vs_fp32_plain": ms_g32 / ms_g}

    # end to end through the public API: host (pinned) points and weights in
    # (asynchronous H2D inside the timed region), loss and solver status of
    # every step read back to pinned host memory, each read one step later so
    # the host does not drain the stream between steps (a non-zero status
    # raises, as train_step(check=True) would)
    e2e = None
    if not args.no_e2e:
        host = [(torch.tensor(p).pin_memory(), torch.tensor(w, dtype=torch.float32).pin_memory())
                for p, w in batches]
        model_e = Model(cfg, precision=args.precision, seed=0, device=dev)
        for s in range(W):
            r = train_step(model_e, *host[s], check=True)
            float(r.loss)
        torch.cuda.synchronize()
        barrier()
        slots = [torch.empty(2, dtype=torch.float64).pin_memory() for _ in range(2)]
        done = [torch.cuda.Event() for _ in range(2)]
        losses = []

        def collect(i):
            done[i].synchronize()
            loss_v, info_v = slots[i].tolist()
            if info_v != 0:
                raise FloatingPointError(f"spectral stage failed (info={int(info_v)})")
            losses.append(loss_v)

        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        prev = None
        for s in range(W, W + K):
            r = train_step(model_e, *host[s], check=False)
            i = s & 1
            slots[i].copy_(torch.stack((r.loss.double(), r.info.double())), non_blocking=True)
            done[i].record()
            if prev is not None:
                collect(prev)
            prev = i
        collect(prev)
        e1.record()
        torch.cuda.synchronize()
        ms_e = max_ms(e0.elapsed_time(e1))
        h2d = host[0][0].numel() * 8 + host[0][1].numel() * 4
        d2h = 16  # loss and solver status (FP64 pair)
        e2e = {"value": world * K / (ms_e / 1e3), "unit": "steps/s", "h2d_bytes_per_step": h2d,
               "d2h_bytes_per_step": d2h, "ms_per_step": ms_e / K}

    if rank != 0:
        if world > 1:
            dist.destroy_process_group()
        return

    # roofline of the dominant jet-MLP kernel (by total time; tc_* / simt_*
    # timers).  The spectral stage works on a 512 x 512 pencil: it is bound by
    # dependent-operation latency and barriers, not by the tensor pipe or HBM,
    # and is reported separately below.  The reverse-data GEMM and the
    # weight-gradient GEMM of a layer run concurrently on two streams, so
    # their event durations include the other kernel's share of the GPU:
    # the pick is among the kernels that run alone.
    concurrent = {"tc_jet_layer_bwd_data", "tc_weight_grad", "bias_grad", "reduce_chunks"}
    own = {k: v for k, v in kernels.items()
           if k.startswith(("tc_", "simt_")) and k not in concurrent}
    dom = max(own, key=lambda k: own[k][1])
    launches_dom, total_ms_dom, flops_dom, bytes_dom = own[dom]
    per_launch_s = total_ms_dom / launches_dom / 1e3
    flops_l, bytes_l = flops_dom / launches_dom, bytes_dom / launches_dom
    # the binding roof for this kernel: whichever of its algorithmic flops at
    # the bf16 peak and its algorithmic bytes at the copy bandwidth takes longer
    t_tensor = flops_l / (pk["bf16"] * 1e12)
    t_hbm = bytes_l / (pk["hbm"] * 1e9)
    tensor_frac = t_tensor / per_launch_s
    hbm_frac = t_hbm / per_launch_s
    tensor = t_tensor >= t_hbm
    if tensor:
        achieved, peak_v, unit = flops_l / per_launch_s / 1e12, pk["bf16"], "TFLOP/s"
    else:
        achieved, peak_v, unit = bytes_l / per_launch_s / 1e9, pk["hbm"], "GB/s"
    traffic = None
    tf = ROOT / "profiles" / "traffic.json"
    if tf.exists():
        traffic = json.loads(tf.read_text()).get(dom)
    roofline = {"bound": "tensor" if tensor else "hbm", "kernel": dom, "achieved": achieved,
                "peak": peak_v, "unit": unit, "frac": achieved / peak_v, "traffic": traffic,
                "peak_source": pk["source"],
                "per_launch_ms": per_launch_s * 1e3,
                "algorithmic_flops_per_launch": flops_l,
                "algorithmic_bytes_per_launch": bytes_l,
                "tensor_frac": tensor_frac, "hbm_frac": hbm_frac}
    stages = {k: {"launches_per_step": v[0] / K, "ms_per_step": v[1] / K} for k, v in
              sorted(kernels.items(), key=lambda kv: -kv[1][1])}
    # the same roofline arithmetic for every tensor-core kernel of the step,
    # largest first (concurrent ones marked: their event durations include
    # the kernel they share the GPU with)
    tc_roofline = {}
    for k, v in sorted(kernels.items(), key=lambda kv: -kv[1][1]):
        if not k.startswith("tc_") or v[0] == 0 or v[1] <= 0:
            continue
        per = v[1] / v[0] / 1e3
        tc_roofline[k] = {"per_launch_ms": per * 1e3,
                          "tensor_frac": v[2] / v[0] / per / 1e12 / pk["bf16"],
                          "hbm_frac": v[3] / v[0] / per / 1e9 / pk["hbm"],
                          "concurrent": k in concurrent}
    spectral_ms = sum(v[1] for k, v in kernels.items()
                      if k.startswith(("spec_", "cusolver", "cublas", "scale_", "weighted_sum"))) / K
    gram = gram_rate(sum(v[1] for k, v in kernels.items() if k in ("tc_gram", "simt_gram")) / K,
                     (2 * n, n), cfg.widths[-2])

    # accuracy of this step against the FP64 oracle (same parameters, points)
    accuracy = None
    if not args.no_accuracy:
        from oracle import neb_oracle as O
        pts, w = batches[0]
        m_acc = Model(cfg, precision=args.precision, seed=0, device=dev)
        r = spectral_step(m_acc, torch.tensor(pts, device=dev),
                          torch.tensor(w, dtype=torch.float32, device=dev), training=True)
        params = [(a.cpu().double().numpy(), b.cpu().double().numpy())
                  for a, b in zip(m_acc.W, m_acc.b)]
        ref = O.objective_and_grad_factored(params, O.features_periodic(pts, cfg.n_freq), w,
                                            cfg.objective)
        lam = r.eigenvalues.cpu().numpy()
        num = den = 0.0
        for gs, rs in zip(r.grads, zip(*ref.grads)):
            for g, rr in zip(gs, rs):
                num += float(((g.cpu().double().numpy() - rr) ** 2).sum())
                den += float((rr ** 2).sum())
        accuracy = {"eig_rel_err_max": float(np.max(np.abs(lam - ref.lam) / np.abs(ref.lam))),
                    "grad_rel_err": math.sqrt(num / den),
                    "loss_rel_err": abs(float(r.loss) - ref.loss) / abs(ref.loss),
                    "n_eigenvalues": int(lam.size)}

    cpu = None
    if not args.no_cpu_baseline:
        t = oracle_step_time(n)
        cpu = {"value": 1.0 / t, "unit": "steps/s", "cores": cpu_threads(), "kind": "port",
               "sample": f"1 full step (16384 points, K=1024) of the FP64 NumPy restatement "
                         f"in oracle/, {cpu_threads()} BLAS threads"}

    line = {
        "metric": METRIC, "value": value, "unit": "steps/s", "n_gpus": world, "steps": K,
        "warmup": W, "ms_per_step": ms_max / K, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": args.precision,
        "data": "synthetic: seeded uniform random points per step, Glorot-normal init (seed 0)",
        "config": {"workload": WORKLOAD, "K": 1024, "hidden": [512] * 4, "points_per_step": n,
                   "parallelism": "replicas" if world > 1 else "single",
                   "l2": "no flush: each step rewrites ~1.1 GB of activation tape (> 129 MB L2)",
                   "spectral": SPECTRAL_STAGES},
        "roofline": roofline,
        "tc_kernels_roofline": tc_roofline,
        "strict_fp64_spectral": strict,
        "grid256": grid256,
        "reference_architecture": ref_arch,
        "cpu_baseline": cpu,
        "e2e": e2e,
        "gpu_launches": int(launches),
        "clocks": clk,
        "fp32_plain": fp32,
        "speedup_vs_fp32_plain": (value / fp32["value"]) if fp32 else None,
        "accuracy": accuracy,
        "solver_ok": info_ok,
        "spectral_stage_ms_per_step": spectral_ms,
        "gram": gram,
        "kernels_ms_per_step": stages,
    }
    print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
