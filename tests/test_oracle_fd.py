"""Oracle self-consistency: central finite differences in FP64 and the
direct-versus-factored Gram routes."""
import numpy as np
import pytest

from oracle import neb_oracle as O


def _fd(params, X0, w, dim, kind, grads, n_check=16, h=1e-5, seed=0):
    rng = np.random.default_rng(seed)
    worst = 0.0
    scale = max(np.abs(g).max() for pair in grads for g in pair)
    for _ in range(n_check):
        li, wi = rng.integers(len(params)), rng.integers(2)
        idx = tuple(rng.integers(s) for s in params[li][wi].shape)

        def loss(sign):
            p = [(W.copy(), b.copy()) for W, b in params]
            p[li][wi][idx] += sign * h
            return O.objective_and_grad(p, X0, w, dim, kind, want_grad=False).loss

        fd = (loss(1) - loss(-1)) / (2 * h)
        worst = max(worst, abs(fd - grads[li][wi][idx]) / scale)
    return worst


@pytest.mark.parametrize("kind", ["trace", "ordering"])
@pytest.mark.parametrize("widths", [[16, 12, 12, 8], [16, 10, 10, 24]])
def test_periodic_gradient_fd(kind, widths):
    pts, w = O.periodic_minibatch(300, 0, 0)
    X0 = O.features_periodic(pts, 4)
    params = O.glorot_init(widths, 0)
    r = O.objective_and_grad(params, X0, w, 2, kind)
    assert r.rank == min(widths[-1], widths[-2])
    assert _fd(params, X0, w, 2, kind, r.grads) < 1e-7


@pytest.mark.parametrize("kind", ["trace", "ordering"])
def test_3d_curl_gradient_fd(kind):
    pts = np.random.default_rng(3).random((200, 3))
    X0 = O.features_raw3d(pts)
    params = O.glorot_init([3, 10, 10, 15], 2)
    r = O.objective_and_grad(params, X0, 1 / 200, 3, kind)
    assert _fd(params, X0, 1 / 200, 3, kind, r.grads) < 1e-7


def test_multihole_gradient_fd():
    pts, w = O.multihole_points(300, 0)
    X0 = O.features_multihole(pts)
    params = O.glorot_init([5, 8, 8, 12], 4)
    r = O.objective_and_grad(params, X0, w, 2, "ordering")
    assert _fd(params, X0, w, 2, "ordering", r.grads) < 1e-7


@pytest.mark.parametrize("widths", [[16, 12, 12, 8], [16, 10, 10, 24], [16, 10, 10, 10]])
def test_factored_route_equals_direct_route(widths):
    pts, w = O.periodic_minibatch(256, 1, 0)
    X0 = O.features_periodic(pts, 4)
    params = O.glorot_init(widths, 5)
    a = O.objective_and_grad(params, X0, w, 2, "ordering")
    b = O.objective_and_grad_factored(params, X0, w, "ordering")
    np.testing.assert_allclose(b.lam, a.lam, rtol=1e-10)
    np.testing.assert_allclose(b.M, a.M, rtol=1e-10, atol=1e-10 * np.abs(a.M).max())
    scale = max(np.abs(g).max() for pair in a.grads for g in pair)
    for ga, gb in zip(a.grads, b.grads):
        for x, y in zip(ga, gb):
            assert np.abs(x - y).max() <= 1e-8 * scale


def test_rank_deficient_pencil_keeps_the_span():
    """K > last hidden width: M has rank H and the finite eigenvalues are
    independent of W_out."""
    pts, w = O.periodic_minibatch(400, 2, 0)
    X0 = O.features_periodic(pts, 4)
    params = O.glorot_init([16, 10, 10, 24], 7)
    a = O.objective_and_grad(params, X0, w, 2, "ordering", want_grad=False)
    params[-1] = (params[-1][0] @ np.random.default_rng(1).normal(size=(10, 10)), params[-1][1])
    b = O.objective_and_grad(params, X0, w, 2, "ordering", want_grad=False)
    assert a.rank == b.rank == 10
    np.testing.assert_allclose(a.lam, b.lam, rtol=1e-9)


def test_samplers_are_seeded_and_inside_their_domains():
    p, w = O.multihole_points(5000, 3)
    for (cx, cy), r in zip(O.MULTIHOLE_CENTRES, O.MULTIHOLE_RADII):
        assert np.all((p[:, 0] - cx) ** 2 + (p[:, 1] - cy) ** 2 > r * r)
    assert np.array_equal(p, O.multihole_points(5000, 3)[0])
    q, wq, c = O.metaball_points(4000, 0)
    d2 = ((q[:, None] - c[None]) ** 2).sum(-1)
    assert np.all(np.exp(-d2 / (2 * 0.08 ** 2)).sum(1) < 0.5)
    g, wg = O.periodic_grid(8)
    assert g.shape == (64, 2) and abs(wg * 64 - (2 * np.pi) ** 2) < 1e-12
