"""The oracle of the periodic evaluation pipeline against the reference's own
outputs (no GPU): third-order jets of the periodic backend's networks
(HardcodedModel.forward_stream) and the autonomous ETDRK4 Galerkin rollout
of experiments/periodic/paper_rollout.py (rollout) after its normalisation
and Ritz stage."""
import math

import numpy as np
import pytest

from oracle import neb_oracle as O

G = np.load(__file__.rsplit("/", 1)[0] + "/golden/reference_vectors.npz")
ROLLOUT_WAVES = ((1, 0), (0, 1), (1, 1), (2, 1))


def rollout_basis(coef, n):
    """Field f of mode k: sum over the wave vectors (m1, m2) of
    coef[k, t, f, 0] cos(m1 x + m2 y + coef[k, t, f, 1]) on the n x n grid,
    [3, n^2, K] (the construction of tests/golden/make_golden.py)."""
    axis = np.arange(n) * 2 * math.pi / n
    xg, yg = np.meshgrid(axis, axis)
    basis = np.zeros((3, n * n, len(coef)))
    for k in range(len(coef)):
        for t, (m1, m2) in enumerate(ROLLOUT_WAVES):
            for f in range(3):
                amp, phase = coef[k, t, f]
                basis[f, :, k] += (amp * np.cos(m1 * xg + m2 * yg + phase)).ravel()
    return basis


def rollout_case():
    """The golden rollout's basis, initial velocity and schedule."""
    basis = rollout_basis(G["roll_coef"], 128)
    u0 = basis[0, :, 0] - 0.7 * basis[0, :, 1] + 0.4 * basis[0, :, 3]
    v0 = basis[1, :, 0] - 0.7 * basis[1, :, 1] + 0.4 * basis[1, :, 3]
    return basis, u0, v0


def _hb_params(prefix):
    labels = ("l0", "l1", "output")
    return ([np.stack([G[f"{prefix}.m{k:03d}.{lab}.weight"] for k in range(4)]) for lab in labels],
            [np.stack([G[f"{prefix}.m{k:03d}.{lab}.bias"] for k in range(4)]) for lab in labels])


def test_third_order_jets_match_forward_stream():
    W, b = _hb_params("hb_in")
    X = O.features_periodic_jet(G["hb_points"], 3, 3)
    E = np.zeros((10, 48, 1)); E[0] = 1.0
    om = O.mode_omegas(3, 8.0, 30.0)
    for k in range(4):
        _, _, out = O.mode_forward([w[k] for w in W], [x[k] for x in b], X, E, 2, 3, om)
        o = out[:, :, 0]
        np.testing.assert_allclose(o[0], G["hb3_value"][k], rtol=1e-9, atol=1e-10)
        np.testing.assert_allclose(o[1:3].T, G["hb3_grad"][k], rtol=1e-9, atol=1e-9)
        np.testing.assert_allclose(o[3:6].T, G["hb3_hess"][k], rtol=1e-9,
                                   atol=1e-9 * np.abs(G["hb3_hess"][k]).max())
        np.testing.assert_allclose(o[6:10].T, G["hb3_third"][k], rtol=1e-9,
                                   atol=1e-9 * np.abs(G["hb3_third"][k]).max())


def test_feature_jets_are_consistent_across_orders():
    pts = np.random.default_rng(1).uniform(0, 2 * math.pi, (9, 2))
    f1 = O.features_periodic_jet(pts, 4, 1)
    f2 = O.features_periodic_jet(pts, 4, 2)
    f3 = O.features_periodic_jet(pts, 4, 3)
    assert np.array_equal(f1, f2[:3]) and np.array_equal(f2, f3[:6])
    lap = O.features_periodic(pts, 4)
    np.testing.assert_allclose(f2[3] + f2[5], lap[3], rtol=1e-14, atol=1e-12)


def test_rollout_matches_reference():
    """The oracle's Ritz stage and ETDRK4 rollout reproduce the reference's
    rollout states (the golden basis has simple Ritz values, so the states
    are fixed up to the sign of each eigenvector, which scipy's eigh fixes
    the same way on both sides)."""
    basis, u0, v0 = rollout_case()
    weight = (2 * math.pi / 128) ** 2
    vals, R, _ = O.ritz_basis(basis[0], basis[1], basis[2], weight)
    np.testing.assert_allclose(vals, G["roll_vals"], rtol=1e-10)
    gu, gv, gw = basis[0] @ R, basis[1] @ R, basis[2] @ R
    c0 = weight * (gu.T @ u0 + gv.T @ v0)
    states = O.etdrk4_rollout(gu, gv, gw, vals, float(G["roll_nu"]), c0, G["roll_times"],
                              float(G["roll_dt"]), weight)
    np.testing.assert_allclose(states, G["roll_states"], rtol=1e-9, atol=1e-11)
    np.testing.assert_allclose((states @ gu.T)[:, :64], G["roll_u_frames"], rtol=1e-9,
                               atol=1e-11)
    r = np.random.default_rng(42).normal(size=len(vals))
    skew = abs(r @ O.galerkin_rhs(gu, gv, gw, weight, r)) / np.linalg.norm(r) ** 3
    assert skew < 1e-9


def test_ritz_rank_gate():
    basis, _, _ = rollout_case()
    gu, gv, gw = basis[0].copy(), basis[1].copy(), basis[2].copy()
    gu[:, 1], gv[:, 1] = 2 * gu[:, 0], 2 * gv[:, 0]  # a dependent mode
    with pytest.raises(ArithmeticError):
        O.ritz_basis(gu, gv, gw, 1.0)
