"""Split-BF16 tcgen05 path (NEB_PREC_BF16X3) against the SIMT FP32 path and
the FP64 oracle (GB300 only).  Tolerances: eigenvalues 1e-4 relative,
gradients 1e-3 relative (norm over all parameters) against the oracle; the
hidden Grams within 5e-5 of the FP32 path's."""
import math

import numpy as np
import pytest
import torch

from oracle import neb_oracle as O
from neb_gb300 import CONFIGS, Model, spectral_step, train_step
from neb_gb300 import configs as CF

pytestmark = pytest.mark.gpu


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


@pytest.mark.parametrize("scale", [dict(hidden=128, outputs=160, n_points=300),
                                   dict(hidden=256, outputs=96, n_points=1000)])
def test_tc_step_matches_fp32_path(scale):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    cfg = CONFIGS["periodic_train"].scaled(**scale)
    pts, w = CF.sample(cfg)
    res = {}
    for prec in ("fp32", "bf16x3"):
        model = Model(cfg, precision=prec, seed=3)
        res[prec] = spectral_step(model, pts, w, training=True)
    a, b = res["fp32"], res["bf16x3"]
    for x, y in ((a.A_M, b.A_M), (a.A_S, b.A_S)):
        err = float((x - y).abs().max() / x.abs().max())
        assert err < 5e-5, err
    lam_a, lam_b = a.eigenvalues.cpu().numpy(), b.eigenvalues.cpu().numpy()
    assert np.max(np.abs(lam_a - lam_b) / np.abs(lam_a)) < 1e-4
    ref = [(gw.cpu().double().numpy(), gb.cpu().double().numpy()) for gw, gb in zip(*a.grads)]
    assert _grad_rel(b.grads, ref) < 1e-3


def test_tc_periodic_train_k1024_accuracy():
    """Full periodic training size: split-BF16 eigenvalues and gradients
    against the FP64 oracle within the targets."""
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    cfg = CONFIGS["periodic_train"]
    pts, w = CF.sample(cfg)
    model = Model(cfg, precision="bf16x3", seed=0)
    res = spectral_step(model, pts, w, training=True)
    ref = O.objective_and_grad_factored(_params64(model), O.features_periodic(pts, 16), w,
                                        cfg.objective)
    lam = res.eigenvalues.cpu().numpy()
    eig = float(np.max(np.abs(lam - ref.lam) / np.abs(ref.lam)))
    grad = _grad_rel(res.grads, ref.grads)
    assert eig <= 1e-4 and grad <= 1e-3, (eig, grad)


def test_tc_training_steps_commit_and_reduce_loss():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    cfg = CONFIGS["periodic_train"].scaled(hidden=128, outputs=128, n_points=4096)
    model = Model(cfg, precision="bf16x3", seed=1)
    losses = []
    for step in range(5):
        pts, w = CF.sample(cfg, step=step)
        losses.append(float(train_step(model, pts, w, lr=3e-3).loss))
    assert model.epoch == 5 and losses[-1] < losses[0]
