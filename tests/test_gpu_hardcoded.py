"""The periodic backend's HardcodedModel API on the GPU (GB300 only).

* Fields of forward_stream_jet1 and one training step of the streamfunction
  Rayleigh peel against the reference's own outputs (the hb_* golden
  vectors: loss, per-rank energies, causal order, gradient norms and every
  parameter and Adam step count after its device Adam transaction).
* The shape of the reference's native precision check
  (tests/test_network_backends.py:101-155): spatial gradients against
  central differences in the points, and one per-mode Adam step in closed
  form, for FP32 and FP64 masters.
* Jet2 Hessians against differences of the gradients; the block reverse
  pass against the oracle; fixed-order sorting; the active-mode mask and the
  physical-validity gate of the all-mode transaction; the checkpoint arrays.
"""
import math
from types import SimpleNamespace

import numpy as np
import pytest
import torch

from oracle import neb_oracle as O

pytestmark = pytest.mark.gpu

G = np.load(__file__.rsplit("/", 1)[0] + "/golden/reference_vectors.npz")


def _needs_gpu():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def _cfg(**kw):
    base = dict(modes=4, hidden=8, hidden_layers=2, frequencies=3, xmin=0.0, xmax=2 * math.pi,
                ymin=0.0, ymax=2 * math.pi, geometry_mode="periodic_box",
                envelope_mode="periodic_identity", input_encoding="periodic_sincos_xy",
                canonical_siren=True, siren_first_omega0=8.0, siren_hidden_omega0=30.0,
                basis_objective="streamfunction_dirichlet_rayleigh",
                causal_sorting="geometry_rayleigh", reorthogonalization_passes=2,
                mass_floor=1e-14, learning_rate=1e-3, grad_clip=5.0, spatial_derivative_order=1,
                mode_forward_batch=2, mode_backward_batch=2, mlp_compute_dtype="float32")
    base.update(kw)
    return SimpleNamespace(**base)


def _golden_arrays(prefix):
    n = len(prefix) + 1
    return {k[n:]: G[k] for k in G.files if k.startswith(prefix + ".")}


def _model(cfg, arrays, precision):
    from neb_gb300.hardcoded import HardcodedModel
    return HardcodedModel(cfg, arrays, precision=precision)


def _fields(model, cfg, pts):
    out = list(model.forward_stream_jet1(cfg, pts))
    v = np.stack([f.value[:, 0].double().cpu().numpy() for _, f, _ in out])
    g = np.stack([f.grad[:, 0].double().cpu().numpy() for _, f, _ in out])
    return v, g


@pytest.mark.parametrize("precision,rtol", [("fp32", 2e-5), ("fp64", 1e-9)])
def test_forward_stream_jet1_matches_reference(precision, rtol):
    _needs_gpu()
    cfg = _cfg()
    model = _model(cfg, _golden_arrays("hb_in"), precision)
    v, g = _fields(model, cfg, G["hb_points"])
    sv, sg = np.abs(G["hb_value"]).max(), np.abs(G["hb_grad"]).max()
    np.testing.assert_allclose(v, G["hb_value"], rtol=rtol, atol=rtol * sv)
    np.testing.assert_allclose(g, G["hb_grad"], rtol=rtol, atol=rtol * sg)


@pytest.mark.parametrize("precision,rtol,atol", [("fp32", 2e-4, 2e-5), ("fp64", 1e-6, 1e-9)])
def test_peel_step_matches_reference(precision, rtol, atol):
    """One training step of the streamfunction peel: the reference's
    diagnostics and the parameters after its all-mode Adam transaction."""
    _needs_gpu()
    from neb_gb300.hardcoded import peel_step
    cfg = _cfg()
    model = _model(cfg, _golden_arrays("hb_in"), precision)
    res = peel_step(cfg, model, G["hb_points"], 0.0, 0.0, True)
    assert res["causal_order"] == G["hb_order"].tolist()
    np.testing.assert_allclose(res["mode_energies"], G["hb_energies"], rtol=rtol)
    np.testing.assert_allclose(res["loss"], G["hb_loss"], rtol=rtol)
    np.testing.assert_allclose([res["gradient_norm_min"], res["gradient_norm_max"]],
                               [G["hb_norm_min"], G["hb_norm_max"]], rtol=10 * rtol)
    assert res["orth_error"] < (1e-5 if precision == "fp32" else 1e-12)
    after = model.arrays()
    ref = _golden_arrays("hb_out")
    assert set(after) == set(ref)
    for key, value in ref.items():
        if key.endswith(".step"):
            assert int(after[key]) == int(value) == 1, key
        elif key.endswith("output.bias") and precision == "fp32":
            # the output bias adds a constant, which the mean removal projects
            # out: its gradient is zero up to rounding, and Adam's first step
            # g / (|g| + eps) turns that rounding into any move up to lr
            assert np.all(np.abs(after[key] - value) <= 1.01 * cfg.learning_rate), key
        else:
            np.testing.assert_allclose(after[key], value, rtol=rtol, atol=atol, err_msg=key)
    # an evaluation step changes nothing and reads the same energies
    ev = peel_step(cfg, model, G["hb_points"], 0.0, 0.0, False)
    assert math.isnan(ev["gradient_norm_min"])
    assert all(int(v) == 1 for k, v in model.arrays().items() if k.endswith(".step"))


def _free_cfg(precision):
    return _cfg(modes=2, hidden=8, frequencies=0, geometry_mode="free_box",
                envelope_mode="free_identity", input_encoding="raw_xy", canonical_siren=False,
                learning_rate=1e-4, grad_clip=1e6)


def _random_arrays(K, shapes, rng, scale, dtype):
    arrays = {}
    for mode in range(K):
        for layer, (inside, outside) in enumerate(shapes):
            label = f"l{layer}" if layer < len(shapes) - 1 else "output"
            for offset, (kind, shape) in enumerate((("weight", (outside, inside)),
                                                    ("bias", (outside,)))):
                arrays[f"m{mode:03d}.{label}.{kind}"] = rng.normal(0, scale, size=shape).astype(dtype)
                stem = f"m{mode:03d}.adam.p{2 * layer + offset:02d}"
                arrays[stem + ".exp_avg"] = np.zeros(shape, dtype)
                arrays[stem + ".exp_avg_sq"] = np.zeros(shape, dtype)
                arrays[stem + ".step"] = np.asarray(0, "i8")
    return arrays


@pytest.mark.parametrize("precision", ["fp32", "fp64"])
def test_spatial_derivatives_and_per_mode_adam(precision):
    """The reference's native precision check on the free box: gradients
    against central differences of the values, then one per-mode Adam step
    with constant gradients 0.25 in closed form."""
    _needs_gpu()
    dtype = "float32" if precision == "fp32" else "float64"
    cfg = _free_cfg(precision)
    arrays = _random_arrays(2, ((2, 8), (8, 8), (8, 1)), np.random.default_rng(17), 0.02, dtype)
    model = _model(cfg, arrays, precision)
    x = np.array([[2.0, 0.2], [3.0, 0.3], [4.0, 0.4]])
    _, gradient = _fields(model, cfg, x)
    step = 1e-3 if precision == "fp32" else 1e-5
    for axis in range(2):
        plus, minus = x.copy(), x.copy()
        plus[:, axis] += step
        minus[:, axis] -= step
        diff = (_fields(model, cfg, plus)[0] - _fields(model, cfg, minus)[0]) / (2 * step)
        np.testing.assert_allclose(diff, gradient[..., axis],
                                   rtol=2e-2 if precision == "fp32" else 2e-6,
                                   atol=2e-6 if precision == "fp32" else 2e-9)
    mode = model.modes[0]
    assert mode.weights[0].dtype == (torch.float32 if precision == "fp32" else torch.float64)
    params = [p for pair in zip(mode.weights, mode.biases) for p in pair]
    before = [p.double().cpu().numpy().copy() for p in params]
    other = [w[1].double().cpu().numpy().copy() for w in model.core.W]
    mode.adam_step([torch.ones_like(p) * 0.25 for p in params], cfg)
    for p, initial in zip(params, before):
        np.testing.assert_allclose(p.double().cpu().numpy(), initial - 1e-4 * 0.25 / (0.25 + 1e-8),
                                   rtol=2e-6 if precision == "fp32" else 1e-12,
                                   atol=2e-8 if precision == "fp32" else 1e-14)
    assert all(s == 1 for s in mode.steps)
    assert all(s == 0 for s in model.modes[1].steps)
    for w, o in zip(model.core.W, other):
        assert np.array_equal(w[1].double().cpu().numpy(), o)
    # a zero gradient is rejected with nothing changed
    snap = [p.clone() for p in params]
    with pytest.raises(FloatingPointError):
        mode.adam_step([torch.zeros_like(p) for p in params], cfg)
    assert all(torch.equal(a, b) for a, b in zip(params, snap))
    assert all(s == 1 for s in mode.steps)


def test_jet2_hessian_and_block_backward():
    """forward_stream_jet2's Hessians against central differences of the
    gradients, and backward_gradients_block_jet1 against the oracle's
    per-mode reverse pass (FP64)."""
    _needs_gpu()
    cfg = _cfg(modes=3, mode_forward_batch=3)
    arrays = _random_arrays(3, ((12, 8), (8, 8), (8, 1)), np.random.default_rng(3), 0.3, "float64")
    model = _model(cfg, arrays, "fp64")
    pts = np.random.default_rng(4).uniform(0, 2 * math.pi, size=(20, 2))
    out = list(model.forward_stream_jet2(cfg, pts))
    hess = np.stack([f.hess[:, 0].cpu().numpy() for _, f, _ in out])  # [K, n, 3]
    scale = np.abs(hess).max()
    h = 1e-5
    for axis in range(2):
        plus, minus = pts.copy(), pts.copy()
        plus[:, axis] += h
        minus[:, axis] -= h
        d = (_fields(model, cfg, plus)[1] - _fields(model, cfg, minus)[1]) / (2 * h)  # [K, n, 2]
        # central differences of a field with Hessians near 1e5: the
        # truncation error is a few 1e-5 relative
        if axis == 0:
            np.testing.assert_allclose(hess[..., 0], d[..., 0], rtol=2e-4, atol=1e-5 * scale)
            np.testing.assert_allclose(hess[..., 1], d[..., 1], rtol=2e-4, atol=1e-5 * scale)
        else:
            np.testing.assert_allclose(hess[..., 2], d[..., 1], rtol=2e-4, atol=1e-5 * scale)
    # and exactly against the oracle's second-order jets
    P = O.features_periodic(pts, 3)
    X2 = np.zeros((6, 20, 12))
    X2[:3] = P[:3]
    X2[3, :, :6] = P[3, :, :6]   # x-features: hxx is the Laplacian
    X2[5, :, 6:] = P[3, :, 6:]   # y-features: hyy is the Laplacian
    E2 = np.zeros((6, 20, 1)); E2[0] = 1.0
    for k in range(3):
        Wk = [np.asarray(arrays[f"m{k:03d}.{lab}.weight"]) for lab in ("l0", "l1", "output")]
        bk = [np.asarray(arrays[f"m{k:03d}.{lab}.bias"]) for lab in ("l0", "l1", "output")]
        _, _, ref = O.mode_forward(Wk, bk, X2, E2, 2, 2, O.mode_omegas(3, 8.0, 30.0))
        np.testing.assert_allclose(hess[k], np.stack([ref[c][:, 0] for c in (3, 4, 5)], -1),
                                   rtol=1e-9, atol=1e-9 * scale)
    # block reverse pass of modes 1..2 (the caches come from a 3-mode block)
    stream = list(model.forward_stream_jet1(cfg, pts, cache=True))
    rng = np.random.default_rng(5)
    from neb_gb300.jets import Jet
    adj = [Jet(torch.tensor(rng.normal(size=(20, 1)), device="cuda"),
               torch.tensor(rng.normal(size=(20, 1, 2)), device="cuda")) for _ in range(2)]
    gW, gb = model.backward_gradients_block_jet1(cfg, [m for m, _, _ in stream[1:]],
                                                 [c for _, _, c in stream[1:]], adj)
    X0 = O.features_periodic(pts, 3)[:3]
    E = np.zeros((3, 20, 1)); E[0] = 1.0
    om = O.mode_omegas(3, 8.0, 30.0)
    for local, k in enumerate((1, 2)):
        Wk = [np.asarray(arrays[f"m{k:03d}.{lab}.weight"]) for lab in ("l0", "l1", "output")]
        bk = [np.asarray(arrays[f"m{k:03d}.{lab}.bias"]) for lab in ("l0", "l1", "output")]
        xs, pres, _ = O.mode_forward(Wk, bk, X0, E, 2, 1, om)
        A = np.zeros((3, 20, 1))
        A[0] = adj[local].value.cpu().numpy()
        A[1:3, :, 0] = adj[local].grad[:, 0].cpu().numpy().T
        rW, rb = O.mode_backward(Wk, xs, pres, E, A, 2, 1, om)
        for j in range(3):
            np.testing.assert_allclose(gW[j][local].cpu().numpy(), rW[j], rtol=1e-9, atol=1e-11)
            np.testing.assert_allclose(gb[j][local].cpu().numpy(), rb[j], rtol=1e-9, atol=1e-11)


def test_fixed_order_peel_matches_oracle():
    _needs_gpu()
    from neb_gb300.hardcoded import peel_step
    cfg = _cfg(causal_sorting="fixed_order")
    arrays = _golden_arrays("hb_in")
    model = _model(cfg, arrays, "fp64")
    pts = G["hb_points"]
    res = peel_step(cfg, model, pts, 0.0, 0.0, False)
    W = [np.stack([arrays[f"m{k:03d}.{lab}.weight"] for k in range(4)]) for lab in ("l0", "l1", "output")]
    b = [np.stack([arrays[f"m{k:03d}.{lab}.bias"] for k in range(4)]) for lab in ("l0", "l1", "output")]
    ref = O.potential_peel_step(W, b, O.features_periodic(pts, 3)[:3], (2 * math.pi) ** 2 / 48,
                                O.mode_omegas(3, 8.0, 30.0), sort=False)
    assert res["causal_order"] == [0, 1, 2, 3]
    np.testing.assert_allclose(res["mode_energies"], ref["losses"], rtol=1e-9)


def test_active_mask_and_physical_gate():
    """adam_step_jet1_device: an invalid physical flag commits nothing; the
    active mask updates only the active modes and advances their steps."""
    _needs_gpu()
    cfg = _cfg()
    model = _model(cfg, _golden_arrays("hb_in"), "fp32")
    core = model.core
    gW = [torch.ones_like(w) for w in core.W]
    gb = [torch.ones_like(x) for x in core.b]
    W0 = [w.clone() for w in core.W]
    _, committed = model.adam_step_jet1_device(cfg, gW, gb, None,
                                               torch.tensor(False, device="cuda"))
    assert int(committed.item()) == 0
    assert all(torch.equal(a, b) for a, b in zip(core.W, W0))
    active = torch.tensor([True, False, True, False], device="cuda")
    norms, committed = model.adam_step_jet1_device(cfg, gW, gb, active,
                                                   torch.tensor(True, device="cuda"))
    assert int(committed.item()) == 1
    assert model.steps.cpu().tolist() == [1, 0, 1, 0]
    for a, b in zip(core.W, W0):
        assert not torch.equal(a[0], b[0]) and torch.equal(a[1], b[1])
        assert not torch.equal(a[2], b[2]) and torch.equal(a[3], b[3])
    # a non-finite gradient of an inactive mode does not block the commit
    gW[0][1].fill_(float("nan"))
    _, committed = model.adam_step_jet1_device(cfg, gW, gb, active,
                                               torch.tensor(True, device="cuda"))
    assert int(committed.item()) == 1 and model.steps.cpu().tolist() == [2, 0, 2, 0]
    # the checkpoint arrays reload into the same model
    from neb_gb300.hardcoded import HardcodedModel
    again = HardcodedModel(cfg, model.arrays())
    assert again.steps.cpu().tolist() == [2, 0, 2, 0]
    v1, g1 = _fields(model, cfg, G["hb_points"])
    v2, g2 = _fields(again, cfg, G["hb_points"])
    assert np.array_equal(v1, v2) and np.array_equal(g1, g2)


@pytest.mark.parametrize("precision,rtol", [("fp32", 5e-4), ("fp64", 1e-8)])
def test_reference_configuration_update_matches_oracle(precision, rtol):
    """One update of the reference's Potential configuration (24 -> 4 x 32
    sine, omega 8/30, the trainer's epoch-0 arrays and point sampler) at
    K = 8 and 512 points against the oracle's restatement."""
    _needs_gpu()
    from neb_gb300 import hardcoded as H
    cfg = _cfg(modes=8, hidden=32, hidden_layers=4, frequencies=6, input_features=24,
               learning_rate=2e-4, sampling_mode="uniform_random", seed=0)
    arrays = H.initial_arrays(cfg)
    model = H.HardcodedModel(cfg, arrays, precision=precision)
    pts = H.fluid_points(cfg, 512, 0.0, 0.0, 0)
    res = H.peel_step(cfg, model, pts, 0.0, 0.0, True)
    labels = ["l0", "l1", "l2", "l3", "output"]
    W = [np.stack([arrays[f"m{k:03d}.{lab}.weight"] for k in range(8)]).astype(np.float64)
         for lab in labels]
    b = [np.stack([arrays[f"m{k:03d}.{lab}.bias"] for k in range(8)]).astype(np.float64)
         for lab in labels]
    ref = O.potential_peel_step(W, b, O.features_periodic(pts.astype(np.float64), 6)[:3],
                                np.float32((2 * math.pi) ** 2) / np.float32(512),
                                O.mode_omegas(5, 8.0, 30.0), lr=2e-4, clip=5.0)
    assert res["causal_order"] == list(ref["order"])
    np.testing.assert_allclose(res["mode_energies"], ref["losses"], rtol=rtol)
    after = model.arrays()
    got = np.concatenate([after[f"m{k:03d}.{lab}.weight"].astype(np.float64).ravel()
                          for j, lab in enumerate(labels) for k in range(8)])
    want = np.concatenate([ref["state"][0][j][k].ravel()
                           for j, lab in enumerate(labels) for k in range(8)])
    if precision == "fp64":
        np.testing.assert_allclose(got, want, rtol=1e-8, atol=1e-11)
    else:
        # Adam's first step is lr g / (|g| + eps): an entry whose gradient is
        # at the FP32 rounding level of the largest may move anywhere in
        # +-lr, so bound every entry by lr and nearly all tightly
        err = np.abs(got - want)
        assert err.max() <= 2 * cfg.learning_rate
        assert np.mean(err > 2e-6 + rtol * np.abs(want)) <= 1e-3


def test_potential_training_loop(tmp_path):
    """Three epochs of the periodic trainer through training.train: the
    cosine rate, the epoch's seeded points, the peel step, an atomic
    checkpoint that reloads into the same model; epoch 1 equals one peel
    step at the schedule's first rate."""
    _needs_gpu()
    from neb_gb300 import hardcoded as H
    from neb_gb300.training import cosine_learning_rate, potential_train_step, train
    cfg = _cfg(modes=4, learning_rate=0.0, sampling_mode="uniform_random", seed=2,
               points_per_step=96, epochs=3, base_learning_rate=2e-3, min_learning_rate=1e-4)
    arrays = H.initial_arrays(SimpleNamespace(**dict(vars(cfg), input_features=12)))
    model = H.HardcodedModel(cfg, arrays)
    ckpt = tmp_path / "state.npz"
    hist = train(model, lambda m, e, lr: potential_train_step(cfg, m, e, lr), cfg.epochs,
                 cfg.base_learning_rate, cfg.min_learning_rate, checkpoint=ckpt)
    assert [h["epoch"] for h in hist] == [1, 2, 3]
    assert hist[0]["learning_rate"] == cosine_learning_rate(2e-3, 1e-4, 1, 3) == 2e-3
    assert hist[-1]["learning_rate"] == 1e-4
    assert model.steps.cpu().tolist() == [3, 3, 3, 3]
    with np.load(ckpt) as z:
        again = H.HardcodedModel(cfg, {k: z[k] for k in z.files})
    after = model.arrays()
    for k, v in again.arrays().items():
        assert np.array_equal(v, after[k]), k
    # epoch 1 alone, from the same start, equals the loop's first epoch
    one = H.HardcodedModel(cfg, arrays)
    r1 = potential_train_step(cfg, one, 1, 2e-3)
    assert abs(r1["loss"] - hist[0]["loss"]) <= 1e-12 * abs(r1["loss"])


@pytest.mark.parametrize("precision,rtol,atol", [("fp32", 2e-4, 2e-5), ("fp64", 1e-6, 1e-9)])
@pytest.mark.parametrize("case", ["fixed_order", "free_box"])
def test_peel_step_variants_match_reference(case, precision, rtol, atol):
    """The reference's peel step with fixed-order sorting, and on the free
    box (raw_xy inputs, free_identity envelope): energies, order and every
    weight after its device Adam."""
    _needs_gpu()
    from neb_gb300.hardcoded import peel_step
    if case == "fixed_order":
        cfg = _cfg(causal_sorting="fixed_order")
        arrays, pts, tag = _golden_arrays("hb_in"), G["hb_points"], "hbf"
    else:
        cfg = _cfg(modes=3, hidden=8, frequencies=0, xmin=-1.0, xmax=2.0, ymin=0.0, ymax=1.5,
                   geometry_mode="free_box", envelope_mode="free_identity",
                   input_encoding="raw_xy", siren_first_omega0=3.0, siren_hidden_omega0=2.0,
                   mode_forward_batch=3, mode_backward_batch=3)
        arrays, pts, tag = _golden_arrays("hbfree_in"), G["hbfree_points"], "hbfree"
    model = _model(cfg, arrays, precision)
    res = peel_step(cfg, model, pts, 0.0, 0.0, True)
    assert res["causal_order"] == G[tag + "_order"].tolist()
    np.testing.assert_allclose(res["mode_energies"], G[tag + "_energies"], rtol=rtol)
    after = model.arrays()
    ref = _golden_arrays(tag + "_out")
    for key, value in ref.items():
        if key.endswith(".weight"):
            np.testing.assert_allclose(after[key], value, rtol=rtol, atol=atol, err_msg=key)
