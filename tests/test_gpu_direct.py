"""Direct route (K x K field Grams from the output jets, point chunks with
recompute) against the FP64 oracle's direct route, through the C ABI.

2D: u = (psi_y, -psi_x), omega = -lap psi; 3D: u = curl A, omega = curl curl A
of vector potentials A_k = (psi_3k, psi_3k+1, psi_3k+2).  Tolerances: FP64
form 1e-9 (eigenvalues, Grams) and 1e-8 (gradients, norm-wise) on
moderately conditioned pencils; the ill-conditioned and FP32 cases state
theirs.  The pencil is solved on range(M) with the oracle's rank rule.
"""
import math

import numpy as np
import pytest
import torch

from oracle import neb_oracle as O
from neb_gb300 import CONFIGS, Model, spectral_step
from neb_gb300 import configs as CF

pytestmark = pytest.mark.gpu


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


def _oracle_features(cfg, pts):
    if cfg.features == "periodic":
        return O.features_periodic(pts, cfg.n_freq, cfg.period)
    if cfg.features == "multihole":
        return O.features_multihole(pts, np.asarray(cfg.centres))
    return O.features_raw3d(pts)


def _case(name, scale, precision, chunk, seed=0):
    cfg = CONFIGS[name].scaled(**scale)
    pts, w = CF.sample(cfg)
    model = Model(cfg, precision=precision, seed=seed)
    res = spectral_step(model, pts, w, training=True, route="direct", chunk_points=chunk)
    ref = O.objective_and_grad(_params64(model), _oracle_features(cfg, pts), w, cfg.dim,
                               cfg.objective)
    return cfg, model, res, ref, (pts, w)


@pytest.mark.parametrize("name,scale", [
    ("periodic_small", dict(hidden=48, outputs=32, grid_n=24)),
    ("metaball3d", dict(hidden=24, outputs=36, n_points=700)),
    ("multihole", dict(hidden=32, outputs=24, n_points=900)),
])
def test_direct_route_fp64_matches_oracle(name, scale):
    _needs_gpu()
    cfg, model, res, ref, _ = _case(name, scale, "fp64", chunk=256)
    assert res.rank == ref.rank == cfg.K
    np.testing.assert_allclose(res.eigenvalues.cpu().numpy(), ref.lam, rtol=1e-9)
    for got, r in ((res.M, ref.M), (res.S, ref.S)):
        np.testing.assert_allclose(got.cpu().numpy(), r, rtol=1e-9, atol=1e-9 * np.abs(r).max())
    assert abs(float(res.loss) - ref.loss) <= 1e-9 * abs(ref.loss)
    assert _grad_rel(res.grads, ref.grads) < 1e-8


def test_direct_route_chunking_is_invisible():
    """One chunk or many: the same Grams and gradients (FP64 sums of chunk
    partials, so equal to rounding)."""
    _needs_gpu()
    cfg = CONFIGS["metaball3d"].scaled(hidden=16, outputs=24, n_points=1000)
    pts, w = CF.sample(cfg)
    model = Model(cfg, precision="fp64", seed=2)
    one = spectral_step(model, pts, w, route="direct", chunk_points=10**6)
    many = spectral_step(model, pts, w, route="direct", chunk_points=173)
    np.testing.assert_allclose(many.M.cpu().numpy(), one.M.cpu().numpy(), rtol=1e-12,
                               atol=1e-12 * float(one.M.abs().max()))
    assert _grad_rel(many.grads, [(a.cpu().double().numpy(), b.cpu().double().numpy())
                                  for a, b in zip(*one.grads)]) < 1e-11


def test_direct_route_3d_fp32_accuracy():
    """FP32 kernels against FP64.  At Glorot init on [0,1]^3 the network is
    nearly linear, so the curl fields are nearly dependent: cond(M) is about
    7e2 already at K = 4 and FP32 field rounding (1e-7) reaches the
    eigenvalues amplified by it; tolerances 2e-3 (eigenvalues) and 2e-2
    (gradients) reflect that conditioning, not the kernels."""
    _needs_gpu()
    cfg, model, res, ref, _ = _case("metaball3d", dict(hidden=32, outputs=12, n_points=4096),
                                    "fp32", chunk=1500)
    lam = res.eigenvalues.cpu().numpy()
    assert lam.shape == ref.lam.shape
    eig_err = float(np.max(np.abs(lam - ref.lam) / np.abs(ref.lam)))
    assert eig_err <= 2e-3, eig_err
    grad_err = _grad_rel(res.grads, ref.grads)
    assert grad_err <= 2e-2, grad_err


def test_direct_route_ill_conditioned_fp64():
    """cond(M) = 3e7 (K = 32 curl fields of a 48-wide network): still full
    rank; FP64 eigenvalues within 1e-7 of the oracle's."""
    _needs_gpu()
    cfg, model, res, ref, _ = _case("metaball3d", dict(hidden=48, outputs=96, n_points=2000),
                                    "fp64", chunk=700)
    assert res.rank == ref.rank == 32
    np.testing.assert_allclose(res.eigenvalues.cpu().numpy(), ref.lam, rtol=1e-7)
    assert _grad_rel(res.grads, ref.grads) < 1e-5


def test_direct_route_rank_deficient_fp64():
    """K = 64 curl fields of a 64-wide network: M has 58 eigenvalues above
    1e-10 of its largest (the nearest two at 1.03e-10 and 8.2e-11), so the
    finite pencil has 58 pairs, as in the oracle.  The spectrum of M decays
    without a gap, so the directions kept last are determined to ~1e-5:
    eigenvalue tolerance 1e-4."""
    _needs_gpu()
    cfg, model, res, ref, _ = _case("metaball3d", dict(hidden=64, outputs=192, n_points=4096),
                                    "fp64", chunk=2048)
    assert res.rank == ref.rank == 58
    np.testing.assert_allclose(res.eigenvalues.cpu().numpy(), ref.lam, rtol=1e-4)
    assert res.eigenvectors.shape == (58, 64)


def test_direct_route_training_decreases_loss_3d():
    _needs_gpu()
    cfg = CONFIGS["metaball3d"].scaled(hidden=32, outputs=12, n_points=2000)
    pts, w = CF.sample(cfg)
    model = Model(cfg, seed=3)
    assert model.precision == "fp32"
    losses = []
    for _ in range(6):
        res = spectral_step(model, pts, w, training=True, chunk_points=700)
        losses.append(float(res.loss))
        model.adam(*res.grads, lr=3e-3)
    assert losses[-1] < losses[0]


def test_direct_route_rejects_split_bf16_model():
    _needs_gpu()
    cfg = CONFIGS["periodic_small"].scaled(hidden=128, outputs=32, grid_n=16)
    model = Model(cfg, precision="bf16x3")
    pts, w = CF.sample(cfg)
    with pytest.raises(NotImplementedError):
        spectral_step(model, pts, w, route="direct")


def test_factored_route_rank_deficient_multihole_fp64():
    """Multihole basis (raw coordinates and hole angles), 128-wide hidden
    layer, K = 256 > H: the hidden mass Gram has 97 eigenvalues above 1e-10
    of its largest (neighbours 1.36e-10 and 9.4e-11), so the range solve keeps
    97 finite pairs, as the oracle does; tolerance as for the 3D case."""
    _needs_gpu()
    cfg = CONFIGS["multihole"].scaled(hidden=128, outputs=256, n_points=4000)
    pts, w = CF.sample(cfg)
    model = Model(cfg, precision="fp64", seed=0)
    assert model.spectral == "range"
    res = spectral_step(model, pts, w, training=True)
    ref = O.objective_and_grad_factored(_params64(model), _oracle_features(cfg, pts), w,
                                        cfg.objective)
    assert res.rank == ref.rank == 97
    np.testing.assert_allclose(res.eigenvalues.cpu().numpy(), ref.lam, rtol=1e-4)
