"""Mode-stacked SIREN networks on the GPU (through the C ABI) against the
reference's backend contract and the FP64 oracle (GB300 only).

* test_network_backend_contract is the reference's own backend test
  (tests/test_network_backends.py:37-98) with torch in place of CuPy: the
  forward against an independent NumPy forward with the exact first spatial
  derivative (rtol 2e-5), the reverse against a directional central
  difference (rtol 3e-3), and the first Adam step in closed form.
* Forward / reverse of every jet variant (2D / 3D, first / second order)
  with an envelope against the oracle: FP64 to 1e-10, FP32 to 1e-4.
* Per-mode Adam against the oracle, and a rejected step changes nothing.
* The Gram-form causal peel against the oracle (FP64, 1e-9) and its gate.
* The 3D velocity step (fields, Grams, peel, gradient) against the oracle.
"""
from types import SimpleNamespace

import numpy as np
import pytest
import torch

from oracle import neb_oracle as O
from neb_gb300 import ModeModel, coefficient_peel, velocity_step
from neb_gb300.jets import Jet

pytestmark = pytest.mark.gpu


def _needs_gpu():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


# ---------------------------------------------- the reference's backend test
def test_network_backend_contract():
    _needs_gpu()
    cfg = SimpleNamespace(hidden=8, hidden_layers=2, siren_first_omega0=2.3,
                          siren_hidden_omega0=1.7)
    model = ModeModel(cfg, K=2, seed=31)
    rng = np.random.default_rng(82)
    f = rng.normal(size=(5, 15)).astype("f4")
    j = rng.normal(size=(5, 15, 3)).astype("f4")
    e = rng.uniform(.3, .8, size=(5, 1)).astype("f4")
    ej = rng.normal(size=(5, 1, 3)).astype("f4")
    dev = lambda a: torch.tensor(a, device="cuda")
    data = SimpleNamespace(features=Jet(dev(f), dev(j)), envelope=Jet(dev(e), dev(ej)))
    value, tape = model.forward(data, 0, 2, True)
    # independent NumPy forward and exact first spatial derivative
    expected, derivatives = [], []
    for mode in range(2):
        x, dx = f.copy(), j.copy()
        for layer in range(cfg.hidden_layers):
            w, b = model.W[layer][mode].cpu().numpy(), model.b[layer][mode].cpu().numpy()
            omega = cfg.siren_first_omega0 if layer == 0 else cfg.siren_hidden_omega0
            pre = omega * (x @ w.T + b)
            dx = np.cos(pre)[..., None] * omega * np.einsum('oi,nid->nod', w, dx)
            x = np.sin(pre)
        w, b = model.W[-1][mode].cpu().numpy(), model.b[-1][mode].cpu().numpy()
        raw = x @ w.T + b
        expected.append(e * raw)
        derivatives.append(e[..., None] * np.einsum('oi,nid->nod', w, dx) + raw[..., None] * ej)
    np.testing.assert_allclose(value.value.cpu().numpy(), expected, rtol=2e-5, atol=2e-6)
    np.testing.assert_allclose(value.grad.cpu().numpy(), derivatives, rtol=2e-5, atol=2e-6)
    av = dev(rng.normal(size=tuple(value.value.shape)).astype("f4"))
    ag = dev(rng.normal(size=tuple(value.grad.shape)).astype("f4"))
    gw, gb = model.backward(data, 0, 2, tape, Jet(av, ag))
    # directional finite differences cover the joint value / derivative reverse
    dw = [dev(rng.normal(size=tuple(w.shape)).astype("f4")) for w in model.W]
    db = [dev(rng.normal(size=tuple(b.shape)).astype("f4")) for b in model.b]
    exact = float(sum(torch.sum(a * b) for a, b in zip(gw + gb, dw + db)))
    parameters = model.W + model.b
    directions = dw + db
    original = [p.clone() for p in parameters]

    def loss(sign):
        for p, before, delta in zip(parameters, original, directions):
            p.copy_(before + sign * 1e-3 * delta)
        y, _ = model.forward(data, 0, 2)
        return float(torch.sum(y.value * av) + torch.sum(y.grad * ag))

    difference = (loss(1) - loss(-1)) / .002
    for p, before in zip(parameters, original):
        p.copy_(before)
    np.testing.assert_allclose(difference, exact, rtol=3e-3, atol=3e-3)
    model.adam(gw, gb, 1e-4, clip=1e6)
    assert model.epoch == 1
    for p, before, grad in zip(parameters, original, gw + gb):
        g = grad.cpu().numpy()
        expected_step = before.cpu().numpy() - 1e-4 * g / (np.abs(g) + 1e-8)
        np.testing.assert_allclose(p.cpu().numpy(), expected_step, rtol=2e-6, atol=2e-7)


# ----------------------------------------------------- every jet variant
def _random_case(dim, order, K=3, n=37, seed=0):
    rng = np.random.default_rng(seed)
    C = 1 + dim + (dim * (dim + 1) // 2 if order == 2 else 0)
    X0 = rng.normal(size=(C, n, 6)) * 0.8
    E = np.concatenate([rng.uniform(.4, 1, (1, n, 1)), rng.normal(size=(C - 1, n, 1)) * 0.3])
    A = rng.normal(size=(K, C, n, 4))
    return X0, E, A


def _packed(arr, model):  # oracle [C, n, F] -> device [n, C, F]
    return torch.tensor(np.moveaxis(arr, 0, 1), dtype=model.dtype, device="cuda").contiguous()


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-10), ("fp32", 1e-4), ("bf16x9", 1e-4),
                                           ("tf32", 3e-3)])
@pytest.mark.parametrize("dim,order", [(2, 1), (2, 2), (3, 1), (3, 2)])
def test_mode_jets_forward_reverse_match_oracle(dim, order, precision, tol):
    _needs_gpu()
    K = 3
    cfg = SimpleNamespace(hidden=40, hidden_layers=2, siren_first_omega0=3.0,
                          siren_hidden_omega0=2.0)
    model = ModeModel(cfg, K=K, seed=4, inputs=6, outputs=4, dim=dim, order=order,
                      precision=precision)
    X0, E, A = _random_case(dim, order, K)
    feats, env = _packed(X0, model), _packed(E, model)
    out, tape = model.forward_packed(feats, env, 1, 3, cache=True)
    adj = torch.tensor(np.moveaxis(A[1:3], 1, 2), dtype=model.dtype, device="cuda").contiguous()
    gW, gb = model.backward_packed(tape, adj)
    om = O.mode_omegas(3, 3.0, 2.0)
    Wn = [w.double().cpu().numpy() for w in model.W]
    bn = [x.double().cpu().numpy() for x in model.b]
    for blk, k in enumerate((1, 2)):
        xs, pres, ref = O.mode_forward([w[k] for w in Wn], [x[k] for x in bn], X0, E, dim, order,
                                       om)
        got = np.moveaxis(out[blk].double().cpu().numpy(), 1, 0)
        np.testing.assert_allclose(got, ref, rtol=tol, atol=tol * np.abs(ref).max())
        rgW, rgb = O.mode_backward([w[k] for w in Wn], xs, pres, E, A[k], dim, order, om)
        for j in range(3):
            g = gW[j][blk].double().cpu().numpy()
            np.testing.assert_allclose(g, rgW[j], rtol=tol, atol=tol * np.abs(rgW[j]).max())
            g = gb[j][blk].double().cpu().numpy()
            np.testing.assert_allclose(g, rgb[j], rtol=tol, atol=tol * np.abs(rgb[j]).max())


def test_mode_adam_per_mode_norms_and_rejection():
    _needs_gpu()
    cfg = SimpleNamespace(hidden=16, hidden_layers=2, siren_first_omega0=2.0,
                          siren_hidden_omega0=1.5)
    model = ModeModel(cfg, K=5, seed=9, inputs=7, outputs=3)
    rng = np.random.default_rng(1)
    W0 = [w.double().cpu().numpy() for w in model.W]
    b0 = [x.double().cpu().numpy() for x in model.b]
    gWn = [rng.normal(size=w.shape) * (1 + np.arange(5)).reshape(5, *([1] * (w.ndim - 1)))
           for w in W0]
    gbn = [rng.normal(size=x.shape) for x in b0]
    gW = [torch.tensor(g, dtype=torch.float32, device="cuda") for g in gWn]
    gb = [torch.tensor(g, dtype=torch.float32, device="cuda") for g in gbn]
    bad = [g.clone() for g in gW]
    bad[0][3, 0, 0] = float("nan")
    with pytest.raises(FloatingPointError):
        model.adam(bad, gb, 1e-3, clip=2.0)
    assert model.epoch == 0
    for w, r in zip(model.W, W0):
        assert np.array_equal(w.double().cpu().numpy(), r)
    norms = model.adam(gW, gb, 1e-3, clip=2.0).cpu().numpy()
    zW = [np.zeros_like(w) for w in W0]
    zb = [np.zeros_like(x) for x in b0]
    st, rn = O.mode_adam(W0, b0, zW, zW, zb, zb, gWn, gbn, 0, 1e-3, 2.0)
    np.testing.assert_allclose(norms, rn, rtol=1e-5)
    assert model.epoch == st[6] == 1
    for w, r in zip(model.W, st[0]):
        np.testing.assert_allclose(w.double().cpu().numpy(), r, rtol=2e-6, atol=2e-7)
    for x, r in zip(model.b, st[1]):
        np.testing.assert_allclose(x.double().cpu().numpy(), r, rtol=2e-6, atol=2e-7)


# --------------------------------------------------------------- the peel
def test_coefficient_peel_matches_oracle():
    _needs_gpu()
    rng = np.random.default_rng(5)
    K = 48
    X = rng.normal(size=(300, K))
    Y = rng.normal(size=(300, K)) * np.linspace(0.3, 4, K)
    M, S = X.T @ X / 100, Y.T @ Y / 100
    r = coefficient_peel(torch.tensor(M, device="cuda"), torch.tensor(S, device="cuda"))
    ref = O.coefficient_peel(M, S)
    np.testing.assert_array_equal(r.order.cpu().numpy(), ref["order"])
    np.testing.assert_allclose(r.losses.cpu().numpy(), ref["losses"], rtol=1e-10)
    for key in ("T", "Cu", "Cd"):
        got = getattr(r, key).cpu().numpy()
        np.testing.assert_allclose(got, ref[key], rtol=1e-9, atol=1e-11 * np.abs(ref[key]).max())
    np.testing.assert_allclose(r.relative_mass.cpu().numpy(), ref["relative_mass"], rtol=1e-10)
    assert float(r.gram_max) <= 1e-12
    # the gate: a duplicated mode leaves no relative mass for its copy
    M2 = M.copy(); S2 = S.copy()
    M2[:, 1] = M2[:, 0]; M2[1, :] = M2[0, :]
    with pytest.raises(FloatingPointError):
        coefficient_peel(torch.tensor(M2, device="cuda"), torch.tensor(S2, device="cuda"))


# ----------------------------------------------------- 3D velocity objective
@pytest.mark.parametrize("precision,tol", [("fp64", 1e-8), ("fp32", 2e-3), ("bf16x9", 2e-3)])
def test_velocity_step_matches_oracle(precision, tol):
    _needs_gpu()
    K, n = 12, 400
    cfg = SimpleNamespace(hidden=24, hidden_layers=2, siren_first_omega0=2.0,
                          siren_hidden_omega0=1.5)
    model = ModeModel(cfg, K=K, seed=2, inputs=5, outputs=3, dim=3, order=2, precision=precision)
    rng = np.random.default_rng(11)
    X0 = rng.normal(size=(10, n, 5)) * 0.6
    E = np.concatenate([rng.uniform(.5, 1, (1, n, 1)), rng.normal(size=(9, n, 1)) * 0.2])
    data = SimpleNamespace(features=_packed(X0, model), envelope=_packed(E, model))
    res = velocity_step(model, data, block=5)
    Wn = [w.double().cpu().numpy() for w in model.W]
    bn = [x.double().cpu().numpy() for x in model.b]
    ref = O.velocity_step(Wn, bn, X0, E, O.mode_omegas(3, 2.0, 1.5))
    np.testing.assert_array_equal(res["order"].cpu().numpy(), ref["order"])
    np.testing.assert_allclose(res["losses"].cpu().numpy(), ref["losses"], rtol=tol)
    gW, gb = res["grads"]
    num = den = 0.0
    for g, r in zip(gW + gb, ref["grads"][0] + ref["grads"][1]):
        d = g.double().cpu().numpy() - r
        num += float((d * d).sum())
        den += float((r * r).sum())
    assert (num / den) ** 0.5 <= tol, (num / den) ** 0.5


@pytest.mark.parametrize("dim,order", [(2, 1), (2, 2), (3, 1), (3, 2)])
def test_evaluation_forward_equals_taped_forward(dim, order):
    """The tape-free evaluation forward gives the same output jets, bit for
    bit, as the taped forward (same kernels, outputs kept in two alternating
    buffers)."""
    _needs_gpu()
    cfg = SimpleNamespace(hidden=40, hidden_layers=3, siren_first_omega0=2.0,
                          siren_hidden_omega0=1.5)
    model = ModeModel(cfg, K=6, seed=3, inputs=5, outputs=3, dim=dim, order=order)
    C = model.channels
    rng = np.random.default_rng(2)
    feats = torch.tensor(rng.normal(size=(300, C, 5)) * 0.5, dtype=torch.float32,
                         device="cuda").contiguous()
    env = torch.tensor(rng.normal(size=(300, C, 1)) * 0.3 + (np.arange(C) == 0)[None, :, None],
                       dtype=torch.float32, device="cuda").contiguous()
    a, _ = model.forward_packed(feats, env, 1, 5)
    b = model.forward_eval(feats, env, 1, 5)
    assert torch.equal(a, b)


def test_velocity_fields_evaluation_matches_oracle():
    """U and D of every mode (the reference's basis evaluation fields) from
    the evaluation forward, against the oracle."""
    _needs_gpu()
    from neb_gb300.modes import velocity_fields
    K, n = 5, 120
    cfg = SimpleNamespace(hidden=24, hidden_layers=2, siren_first_omega0=2.0,
                          siren_hidden_omega0=1.5)
    model = ModeModel(cfg, K=K, seed=2, inputs=5, outputs=3, dim=3, order=2, precision="fp64")
    rng = np.random.default_rng(11)
    X0 = rng.normal(size=(10, n, 5)) * 0.6
    E = np.concatenate([rng.uniform(.5, 1, (1, n, 1)), rng.normal(size=(9, n, 1)) * 0.2])
    data = SimpleNamespace(features=_packed(X0, model), envelope=_packed(E, model))
    U, D = velocity_fields(model, data, block=2)
    Wn = [w.double().cpu().numpy() for w in model.W]
    bn = [x.double().cpu().numpy() for x in model.b]
    om = O.mode_omegas(3, 2.0, 1.5)
    for k in range(K):
        _, _, out = O.mode_forward([w[k] for w in Wn], [x[k] for x in bn], X0, E, 3, 2, om)
        u, d = O.velocity_fields(out)
        np.testing.assert_allclose(U[:, k].cpu().numpy(), u.reshape(-1), rtol=1e-10, atol=1e-12)
        np.testing.assert_allclose(D[:, k].cpu().numpy(), d.reshape(-1), rtol=1e-10, atol=1e-12)
