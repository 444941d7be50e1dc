"""Envelopes on the shared network's reference-API forward / backward
(GB300 only): the output jets times a scalar envelope jet against the
product rule applied in NumPy to the envelope-free outputs, and the reverse
pass against a directional central difference of <adjoint, forward> (the
check of the reference's tests/test_network_backends.py:73-92), FP64."""
import numpy as np
import pytest
import torch

from neb_gb300 import CONFIGS, Jet, Model
from neb_gb300 import configs as CF

pytestmark = pytest.mark.gpu


def _needs_gpu():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def _envelope(dim, n, rng):
    v = rng.uniform(.3, .9, (n, 1))
    g = rng.normal(size=(n, 1, dim)) * 0.4
    if dim == 2:
        return Jet(torch.tensor(v), torch.tensor(g), lap=torch.tensor(rng.normal(size=(n, 1))))
    return Jet(torch.tensor(v), torch.tensor(g), hess=torch.tensor(rng.normal(size=(n, 1, 6))))


def _product(e, x, dim):
    """NumPy product rule; e [n, C], x [n, C, W]."""
    y = np.empty_like(x)
    y[:, 0] = e[:, :1] * x[:, 0]
    for a in range(dim):
        y[:, 1 + a] = e[:, :1] * x[:, 1 + a] + e[:, 1 + a:2 + a] * x[:, 0]
    if dim == 2:
        y[:, 3] = (e[:, :1] * x[:, 3] + e[:, 3:4] * x[:, 0]
                   + 2 * (e[:, 1:2] * x[:, 1] + e[:, 2:3] * x[:, 2]))
    else:
        pairs = [(0, 0), (0, 1), (0, 2), (1, 1), (1, 2), (2, 2)]
        for k, (i, j) in enumerate(pairs):
            q = 4 + k
            y[:, q] = (e[:, :1] * x[:, q] + e[:, q:q + 1] * x[:, 0]
                       + e[:, 1 + i:2 + i] * x[:, 1 + j] + e[:, 1 + j:2 + j] * x[:, 1 + i])
    return y


@pytest.mark.parametrize("dim", [2, 3])
def test_envelope_forward_and_reverse(dim):
    _needs_gpu()
    cfg = (CONFIGS["periodic_small"] if dim == 2 else CONFIGS["metaball3d"]).scaled(
        hidden=24, outputs=12, n_points=61, grid_n=8)
    pts, _ = CF.sample(cfg)
    model = Model(cfg, precision="fp64", seed=3)
    X0 = model.features(pts)
    n = X0.shape[0]
    rng = np.random.default_rng(5)
    env = _envelope(dim, n, rng)
    plain = type("D", (), {"features": X0})()
    data = type("D", (), {"features": X0, "envelope": env})()
    raw, _ = model.forward(plain, 2, 10)
    got, tape = model.forward(data, 2, 10, cache=True)
    from neb_gb300 import pack
    e = pack(env, dim).reshape(n, -1).numpy()
    ref = _product(e, pack(raw, dim).cpu().numpy(), dim)
    np.testing.assert_allclose(pack(got, dim).cpu().numpy(), ref, rtol=1e-12, atol=1e-12)
    C = 4 if dim == 2 else 10
    adj = torch.tensor(rng.normal(size=(n, C, 8)), device="cuda")
    gW, gb = model.backward(data, 2, 10, tape, adj)
    dirs = [torch.tensor(rng.normal(size=tuple(p.shape)), device="cuda")
            for p in [*model.W, *model.b]]
    exact = float(sum((g * d).sum() for g, d in zip([*gW, *gb], dirs)))
    params = [*model.W, *model.b]
    orig = [p.clone() for p in params]

    def objective(sign):
        for p, o, d in zip(params, orig, dirs):
            p.copy_(o + sign * 1e-6 * d)
        y, _ = model.forward(data, 2, 10)
        return float((pack(y, dim).to("cuda") * adj).sum())

    fd = (objective(1) - objective(-1)) / 2e-6
    for p, o in zip(params, orig):
        p.copy_(o)
    np.testing.assert_allclose(fd, exact, rtol=1e-6)
