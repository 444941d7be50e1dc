"""Every workload configuration at its own size against the FP64 oracle
(GB300 only, through the C ABI).

Targets of the workloads: eigenvalue relative error <= 1e-4 (max over the
finite eigenvalues) and gradient relative error <= 1e-3 (norm-wise over all
parameters).

* periodic_eval  (256^2 grid, 4 x 512, K = 1024), seeds 0, 1, 2: forward,
  hidden Grams and eigensolve in split-BF16, and in FP32 for seed 0.
* periodic_train (16,384 random points per step): split-BF16 at seeds 0, 1,
  2, and again after the 25 Adam steps of the configuration; central finite
  differences (h = 1e-4, FP64 form) on 32 seeded parameter entries of the
  full network against the hand-written gradient.
* multihole (200,000 points, 4 x 256, K = 1024) and metaball3d (8,192 of
  the 1,599,754 points, 4 x 512, K = 512 x 3): the finite pencil on range(M)
  at the precision's rank tolerance (model.RANK_RTOL), which the oracle
  solves at the same tolerance; the ranks agree.
"""
import math

import numpy as np
import pytest
import torch

from oracle import neb_oracle as O
from neb_gb300 import CONFIGS, Model, spectral_step, train_step
from neb_gb300 import configs as CF
from neb_gb300.model import RANK_RTOL

pytestmark = pytest.mark.gpu

EIG_TOL = 1e-4
GRAD_TOL = 1e-3
# one pass of TF32 inputs (10-bit mantissa) in the layer GEMMs does not meet
# the targets: measured eig 3.5e-4 / 7.8e-4, grad 1.0e-3 / 4.1e-3 on
# multihole / the metaball subsample; it is checked at this looser bar
TF32_TOL = (2e-3, 1e-2)


def _tols(precision):
    return TF32_TOL if precision == "tf32" else (EIG_TOL, GRAD_TOL)


def _needs_gpu():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def _params64(model):
    return [(W.detach().cpu().double().numpy(), b.detach().cpu().double().numpy())
            for W, b in zip(model.W, model.b)]


def _grad_rel(gpu_grads, ref_grads):
    gW, gb = gpu_grads
    num = den = 0.0
    for j, (rW, rb) in enumerate(ref_grads):
        for g, r in ((gW[j], rW), (gb[j], rb)):
            d = g.detach().cpu().double().numpy() - r
            num += float(np.sum(d * d))
            den += float(np.sum(r * r))
    return math.sqrt(num / den)


def _eig_rel(res, ref):
    lam = res.eigenvalues.cpu().numpy()
    assert lam.shape == ref.lam.shape, (lam.shape, ref.lam.shape)
    return float(np.max(np.abs(lam - ref.lam) / np.abs(ref.lam)))


# ------------------------------------------------------------ periodic_eval
@pytest.mark.parametrize("precision,seed", [("bf16x3", 0), ("bf16x3", 1), ("bf16x3", 2),
                                            ("fp32", 0)])
def test_periodic_eval_256_grid(precision, seed):
    _needs_gpu()
    cfg = CONFIGS["periodic_eval"]
    pts, w = CF.sample(cfg)
    model = Model(cfg, precision=precision, seed=seed)
    res = spectral_step(model, pts, w, training=False, return_grams=True)
    ref = O.objective_and_grad_factored(_params64(model), O.features_periodic(pts, cfg.n_freq), w,
                                        cfg.objective, want_grad=False)
    assert res.rank == ref.rank == 512
    eig = _eig_rel(res, ref)
    gram = float(np.max(np.abs(res.M.cpu().numpy() - ref.M)) / np.max(np.abs(ref.M)))
    assert eig <= EIG_TOL, eig
    assert gram <= 1e-4, gram
    assert abs(float(res.loss) - ref.loss) <= 1e-4 * abs(ref.loss)


# ----------------------------------------------------------- periodic_train
def _train_case(model, cfg, step=0, seed=0):
    pts, w = CF.sample(cfg, step=step, seed=seed)
    res = spectral_step(model, pts, w, training=True)
    ref = O.objective_and_grad_factored(_params64(model), O.features_periodic(pts, cfg.n_freq), w,
                                        cfg.objective)
    return _eig_rel(res, ref), _grad_rel(res.grads, ref.grads)


@pytest.mark.parametrize("seed", [1, 2])
def test_periodic_train_seeds(seed):
    """Seeds 1 and 2 of the training configuration (seed 0 is in
    test_gpu_tc.py), split-BF16 against the oracle."""
    _needs_gpu()
    cfg = CONFIGS["periodic_train"]
    model = Model(cfg, precision="bf16x3", seed=seed)
    eig, grad = _train_case(model, cfg, seed=seed)
    assert eig <= EIG_TOL and grad <= GRAD_TOL, (eig, grad)


def test_periodic_train_after_25_adam_steps():
    """The configuration's 25 Adam steps (lr 1e-3, a fresh 128^2 batch per
    step) in split-BF16, then the step-25 objective and gradient at the
    trained parameters against the oracle."""
    _needs_gpu()
    cfg = CONFIGS["periodic_train"]
    model = Model(cfg, precision="bf16x3", seed=0)
    losses = []
    for step in range(cfg.steps):
        pts, w = CF.sample(cfg, step=step)
        losses.append(float(train_step(model, pts, w).loss))
    assert model.epoch == cfg.steps == 25
    assert all(math.isfinite(v) for v in losses)
    eig, grad = _train_case(model, cfg, step=cfg.steps)
    assert eig <= EIG_TOL and grad <= GRAD_TOL, (eig, grad)


def test_periodic_train_central_differences():
    """Central differences of the objective (h = 1e-4, FP64 form, the full
    64 -> 4 x 512 -> 1024 network on one 128^2 batch) at 32 seeded parameter
    entries against the hand-written reverse pass (the reference's own
    directional check is tests/test_network_backends.py:73-92)."""
    _needs_gpu()
    cfg = CONFIGS["periodic_train"]
    pts, w = CF.sample(cfg)
    model = Model(cfg, precision="fp64", seed=0)
    feats = model.features(pts)
    wt = torch.as_tensor(w, dtype=torch.float64, device="cuda")
    res = spectral_step(model, features=feats, weights=wt, training=True)
    gW, gb = res.grads
    params = [*model.W, *model.b]
    grads = [*gW, *gb]
    rng = np.random.default_rng(2024)
    # hidden layers only: with K >= H the finite eigenvalues do not depend on
    # the output layer (its gradient is zero, checked below)
    hidden = list(range(len(model.W) - 1)) + [len(model.W) + j for j in range(len(model.b) - 1)]
    h = 1e-4
    fd, an = [], []
    for _ in range(32):
        t = int(rng.choice(hidden))
        idx = tuple(int(rng.integers(0, s)) for s in params[t].shape)
        x0 = float(params[t][idx])
        vals = []
        for sgn in (1.0, -1.0):
            params[t][idx] = x0 + sgn * h
            vals.append(float(spectral_step(model, features=feats, weights=wt,
                                            training=False).loss))
        params[t][idx] = x0
        fd.append((vals[0] - vals[1]) / (2 * h))
        an.append(float(grads[t][idx]))
    fd, an = np.asarray(fd), np.asarray(an)
    err = float(np.linalg.norm(fd - an) / np.linalg.norm(an))
    assert err <= 1e-5, (err, fd[:4], an[:4])
    assert float(gW[-1].abs().max()) == 0.0 and float(gb[-1].abs().max()) == 0.0


# ---------------------------------------------------- multihole, metaball3d
def _pencil_case(model, X0, pts, w, dim, factored):
    res = spectral_step(model, torch.tensor(pts, device="cuda"),
                        torch.tensor(w, device="cuda"), training=True)
    p = _params64(model)
    if factored:
        ref = O.objective_and_grad_factored(p, X0, w, model.c.objective,
                                            rank_rtol=model.rank_rtol)
    else:
        ref = O.objective_and_grad(p, X0, w, dim, model.c.objective, rank_rtol=model.rank_rtol)
    assert res.rank == ref.rank, (res.rank, ref.rank)
    return _eig_rel(res, ref), _grad_rel(res.grads, ref.grads), res.rank


@pytest.mark.parametrize("precision", ["bf16x3", "fp32", "fp64", "tf32", "bf16x9"])
def test_multihole_200k(precision):
    _needs_gpu()
    cfg = CONFIGS["multihole"]
    pts, w = CF.sample(cfg)
    model = Model(cfg, precision=precision, seed=0)
    assert model.rank_rtol == RANK_RTOL[precision]
    X0 = O.features_multihole(pts, np.asarray(cfg.centres))
    eig, grad, rank = _pencil_case(model, X0, pts, w, 2, True)
    assert rank >= (10 if precision == "tf32" else 19)
    eig_tol, grad_tol = _tols(precision)
    assert eig <= eig_tol and grad <= grad_tol, (eig, grad, rank)


@pytest.mark.parametrize("precision", ["fp32", "fp64", "tf32", "bf16x9"])
def test_metaball3d_subsample(precision):
    """8,192 seeded points of the 1,599,754 (weights rescaled to the full
    volume): the direct route with curl and curl-curl fields."""
    _needs_gpu()
    cfg = CONFIGS["metaball3d"]
    pts, w = CF.sample(cfg)
    sub = np.random.default_rng(7).choice(len(w), size=8192, replace=False)
    ps, ws = pts[sub], w[sub] * (len(w) / 8192)
    model = Model(cfg, precision=precision, seed=0)
    eig, grad, rank = _pencil_case(model, O.features_raw3d(ps), ps, ws, 3, False)
    assert rank >= (5 if precision == "tf32" else 11)
    eig_tol, grad_tol = _tols(precision)
    assert eig <= eig_tol and grad <= grad_tol, (eig, grad, rank)


@pytest.mark.parametrize("precision", ["bf16x3", "fp32"])
def test_factored_route_point_chunks_recompute(precision):
    """The factored route over point chunks (Grams accumulated chunk by
    chunk, the reverse pass recomputing every chunk's activations but the
    last) equals the one-chunk step, and stays within the oracle targets."""
    _needs_gpu()
    cfg = CONFIGS["periodic_train"]
    pts, w = CF.sample(cfg)
    model = Model(cfg, precision=precision, seed=1)
    whole = spectral_step(model, pts, w, training=True)
    parts = spectral_step(model, pts, w, training=True, chunk_points=4096 + 128)
    assert whole.chunks == 1 and parts.chunks == 4
    lam1, lam2 = whole.eigenvalues.cpu().numpy(), parts.eigenvalues.cpu().numpy()
    assert float(np.max(np.abs(lam1 - lam2) / np.abs(lam1))) <= 1e-5
    ref = O.objective_and_grad_factored(_params64(model), O.features_periodic(pts, cfg.n_freq), w,
                                        cfg.objective)
    g_whole = _grad_rel(whole.grads, ref.grads)
    g_parts = _grad_rel(parts.grads, ref.grads)
    assert _eig_rel(parts, ref) <= EIG_TOL and g_parts <= GRAD_TOL, g_parts
    assert abs(g_parts - g_whole) <= 0.2 * g_whole + 1e-6, (g_whole, g_parts)
