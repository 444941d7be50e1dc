"""CUDA path against the FP64 oracle, through the C ABI (GB300 only).

Tolerances: FP64 form to ~1e-9 (FP64 arithmetic, different summation
order); FP32 form and the split-BF16 tensor-core form against the targets
of the workload: eigenvalue relative error <= 1e-4 and gradient relative
error (norm-wise over all parameters) <= 1e-3.
"""
import math

import numpy as np
import pytest
import torch

from oracle import neb_oracle as O
from neb_gb300 import CONFIGS, Model, SpectralObjective, spectral_step, train_step
from neb_gb300 import configs as CF

pytestmark = pytest.mark.gpu

EIG_TOL = 1e-4
GRAD_TOL = 1e-3


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


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
@pytest.mark.parametrize("name", ["periodic_small", "multihole", "metaball3d"])
def test_features_match_oracle(precision, name):
    _needs_gpu()
    cfg = CONFIGS[name]
    pts, _ = CF.sample(cfg.scaled(n_points=777, grid_n=16))
    model = Model(cfg.scaled(hidden=8, outputs=6 if cfg.dim == 2 else 6), precision=precision)
    X = model.features(pts).cpu().double().numpy()
    ref = np.moveaxis(_oracle_features(cfg, pts), 0, 1)
    tol = 1e-12 if precision == "fp64" else 2e-6
    np.testing.assert_allclose(X, ref, rtol=tol, atol=tol * np.abs(ref).max())


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-11), ("fp32", 2e-5)])
@pytest.mark.parametrize("dim", [2, 3])
def test_forward_output_jets_match_oracle(precision, tol, dim):
    _needs_gpu()
    cfg = CONFIGS["periodic_small"] if dim == 2 else CONFIGS["metaball3d"]
    cfg = cfg.scaled(hidden=40, outputs=30, n_points=301, grid_n=17)
    pts, _ = CF.sample(cfg)
    model = Model(cfg, precision=precision, seed=4)
    X0 = model.features(pts)
    field, _ = model.forward(type("D", (), {"features": X0})(), 3, 27)
    _, _, Psi = O.mlp_forward(_params64(model), _oracle_features(cfg, pts), dim)
    ref = Psi[..., 3:27]
    got = [field.value, *[field.grad[..., a] for a in range(dim)]]
    got += [field.lap] if dim == 2 else [field.hess[..., k] for k in range(6)]
    for c, g in enumerate(got):
        r = ref[c]
        np.testing.assert_allclose(g.cpu().double().numpy(), r, rtol=tol,
                                   atol=tol * np.abs(r).max())


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-10), ("fp32", 3e-4)])
@pytest.mark.parametrize("dim", [2, 3])
def test_backward_output_matches_oracle(precision, tol, dim):
    """Model.backward (the reference's Model.backward role) against the
    oracle's hand-written reverse pass with the same output adjoints."""
    _needs_gpu()
    cfg = CONFIGS["periodic_small"] if dim == 2 else CONFIGS["metaball3d"]
    cfg = cfg.scaled(hidden=24, outputs=18, n_points=257, grid_n=16)
    pts, _ = CF.sample(cfg)
    model = Model(cfg, precision=precision, seed=7)
    X0 = model.features(pts)
    data = type("D", (), {"features": X0})()
    field, tape = model.forward(data, 2, 14, cache=True)
    C = 4 if dim == 2 else 10
    adj = torch.randn((X0.shape[0], C, 12), dtype=model.dtype, device=model.device,
                      generator=torch.Generator(device=model.device).manual_seed(3))
    gW, gb = model.backward(data, 2, 14, tape, adj)
    p = _params64(model)
    xs, zs, Psi = O.mlp_forward(p, _oracle_features(cfg, pts), dim)
    Pb = np.zeros_like(Psi)
    Pb[..., 2:14] = np.moveaxis(adj.cpu().double().numpy(), 1, 0)
    ref = O.mlp_backward(p, xs, zs, Pb, dim)
    assert _grad_rel((gW, gb), ref) < tol


def _spectral_case(name, precision, scale, seed=0):
    cfg = CONFIGS[name].scaled(**scale)
    pts, w = CF.sample(cfg)
    model = Model(cfg, precision=precision, seed=seed)
    res = spectral_step(model, pts, w, training=True, return_grams=True)
    X0 = _oracle_features(cfg, pts)
    ref = O.objective_and_grad_factored(_params64(model), X0, w, cfg.objective)
    return cfg, model, res, ref


@pytest.mark.parametrize("scale", [dict(hidden=48, outputs=32, grid_n=24),
                                   dict(hidden=32, outputs=48, grid_n=24)])
def test_spectral_step_fp64_matches_oracle(scale):
    _needs_gpu()
    cfg, model, res, ref = _spectral_case("periodic_small", "fp64", scale)
    lam = res.eigenvalues.cpu().numpy()
    np.testing.assert_allclose(lam, ref.lam, rtol=1e-9)
    assert abs(float(res.loss) - ref.loss) <= 1e-9 * abs(ref.loss)
    np.testing.assert_allclose(res.M.cpu().numpy(), ref.M, rtol=1e-9, atol=1e-9 * np.abs(ref.M).max())
    assert _grad_rel(res.grads, ref.grads) < 1e-8


def test_periodic_small_full_config_fp64():
    """The FP64 small configuration exactly: 64^2 grid, 3 x 128 tanh, K = 64,
    trace objective; checked against the oracle's direct K-space route."""
    _needs_gpu()
    cfg = CONFIGS["periodic_small"]
    pts, w = CF.sample(cfg)
    model = Model(cfg, precision="fp64", seed=0)
    res = spectral_step(model, pts, w, training=True, return_grams=True)
    ref = O.objective_and_grad(_params64(model), O.features_periodic(pts, 16), w, 2, "trace")
    np.testing.assert_allclose(res.eigenvalues.cpu().numpy(), ref.lam, rtol=1e-9)
    np.testing.assert_allclose(res.S.cpu().numpy(), ref.S, rtol=1e-9, atol=1e-9 * np.abs(ref.S).max())
    assert _grad_rel(res.grads, ref.grads) < 1e-8


@pytest.mark.parametrize("precision", ["fp32"])
def test_periodic_train_k1024_accuracy(precision):
    """Full periodic training size (K = 1024, 4 x 512, 128^2 points): eigenvalue
    and gradient errors against the FP64 oracle within the targets."""
    _needs_gpu()
    cfg, model, res, ref = _spectral_case("periodic_train", precision, {})
    lam = res.eigenvalues.cpu().numpy()
    assert lam.shape == ref.lam.shape == (512,)
    eig_err = float(np.max(np.abs(lam - ref.lam) / np.abs(ref.lam)))
    grad_err = _grad_rel(res.grads, ref.grads)
    assert eig_err <= EIG_TOL, eig_err
    assert grad_err <= GRAD_TOL, grad_err


def test_adam_matches_oracle_and_rejects_bad_gradients():
    _needs_gpu()
    cfg = CONFIGS["periodic_small"].scaled(hidden=16, outputs=8)
    model = Model(cfg, precision="fp32", seed=2)
    p0 = _params64(model)
    rng = np.random.default_rng(0)
    grads = [(rng.normal(size=W.shape), rng.normal(size=b.shape)) for W, b in p0]
    gW = [torch.tensor(g, dtype=torch.float32, device="cuda") for g, _ in grads]
    gb = [torch.tensor(g, dtype=torch.float32, device="cuda") for _, g in grads]
    model.adam(gW, gb, 1e-3, clip=0.7)
    model.adam([2 * g for g in gW], [-g for g in gb], 1e-3, clip=0.7)
    ref, mom = O.adam_step(p0, O.zero_moments(p0), grads, 0, 1e-3, 0.7)[:2]
    ref, mom = O.adam_step(ref, mom, [(2 * a, -b) for a, b in grads], 1, 1e-3, 0.7)[:2]
    for (W, b), (rW, rb) in zip(_params64(model), ref):
        np.testing.assert_allclose(W, rW, rtol=2e-6, atol=2e-7)
        np.testing.assert_allclose(b, rb, rtol=2e-6, atol=2e-7)
    assert model.epoch == 2
    before = _params64(model)
    bad = [g.clone() for g in gW]
    bad[0][0, 0] = float("nan")
    with pytest.raises(FloatingPointError):
        model.adam(bad, gb, 1e-3)
    for (W, b), (rW, rb) in zip(_params64(model), before):
        assert np.array_equal(W, rW) and np.array_equal(b, rb)


def test_spectral_step_rejects_singular_mass():
    """A zero last hidden layer makes M singular: the FP64 rank gate raises."""
    _needs_gpu()
    cfg = CONFIGS["periodic_small"].scaled(hidden=16, outputs=8, grid_n=8)
    model = Model(cfg, precision="fp64")
    model.W[-2].zero_()
    pts, w = CF.sample(cfg)
    with pytest.raises(FloatingPointError):
        spectral_step(model, pts, w)


def test_training_loop_decreases_loss_fp32():
    _needs_gpu()
    cfg = CONFIGS["periodic_train"].scaled(hidden=64, outputs=48, n_points=2048)
    model = Model(cfg, precision="fp32", seed=1)
    losses = []
    for step in range(6):
        pts, w = CF.sample(cfg, step=step)
        res = train_step(model, pts, w, lr=3e-3)
        losses.append(float(res.loss))
    assert model.epoch == 6
    assert losses[-1] < losses[0]


def test_spectral_objective_autograd_matches_oracle(tmp_path):
    """SpectralObjective as a torch.autograd.Function: loss and parameter
    gradients through torch.autograd.grad equal the oracle's (FP64 form)."""
    _needs_gpu()
    cfg = CONFIGS["periodic_small"].scaled(hidden=32, outputs=24, grid_n=20)
    pts, w = CF.sample(cfg)
    model = Model(cfg, precision="fp64", seed=5)
    params = [p.detach().requires_grad_() for p in model.parameters()]
    feats = model.features(pts)
    loss = SpectralObjective.apply(model, feats, torch.as_tensor(w, device="cuda"), *params)
    grads = torch.autograd.grad(2.0 * loss, params)
    ref = O.objective_and_grad_factored(_params64(model), _oracle_features(cfg, pts), w,
                                        cfg.objective)
    assert abs(float(loss.detach()) - ref.loss) <= 1e-9 * abs(ref.loss)
    L = len(model.W)
    got = ([g / 2.0 for g in grads[:L]], [g / 2.0 for g in grads[L:]])
    assert _grad_rel(got, ref.grads) < 1e-8
    # save / load round trip keeps parameters, moments and epoch (NCC keys)
    gW, gb = got
    model.adam(gW, gb, 1e-3)
    path = tmp_path / "state.npz"
    model.save(path)
    other = Model(cfg, precision="fp64", seed=9)
    other.load(path)
    assert other.epoch == model.epoch == 1
    for name in ("W", "b", "mW", "vW", "mb", "vb"):
        for a, b in zip(getattr(model, name), getattr(other, name)):
            assert torch.equal(a, b)
