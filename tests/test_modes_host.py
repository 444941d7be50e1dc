"""Host-side logic of the mode-stacked SIREN family (no GPU): the
initialisation equals the reference's, bit for bit, and the oracle's
reverse pass of the per-mode network and of the velocity objective passes
central finite differences."""
import math
from types import SimpleNamespace

import numpy as np
import pytest

from oracle import neb_oracle as O
from neb_gb300.modes import jet_channels, siren_init

G = np.load(__import__("os").path.join(__import__("os").path.dirname(__file__), "golden",
                                       "reference_vectors.npz"))


def test_siren_init_matches_reference_model():
    """native_cupy_core.Model(c, K=2, seed=31) with hidden 8 x 2 layers."""
    c = SimpleNamespace(hidden=8, hidden_layers=2, siren_first_omega0=2.3, siren_hidden_omega0=1.7)
    W, b = siren_init(c, 2, 31, 15, 3)
    for j in range(3):
        np.testing.assert_array_equal(W[j].astype(np.float64), G[f"env_W{j}"])
        np.testing.assert_array_equal(b[j].astype(np.float64), G[f"env_b{j}"])


def test_jet_channel_counts():
    assert [jet_channels(d, o) for d in (2, 3) for o in (1, 2)] == [3, 6, 4, 10]
    assert jet_channels(2, 3) == 10


def _velocity_case(seed=3, K=3, n=9):
    rng = np.random.default_rng(seed)
    c = SimpleNamespace(hidden=5, hidden_layers=2, siren_first_omega0=1.5, siren_hidden_omega0=1.2)
    W, b = siren_init(c, K, seed, 4, 3)
    W = [w.astype(np.float64) for w in W]
    b = [x.astype(np.float64) for x in b]
    X0 = rng.normal(size=(10, n, 4)) * 0.7
    E = np.concatenate([rng.uniform(.5, 1, (1, n, 1)), rng.normal(size=(9, n, 1)) * 0.2])
    return W, b, X0, E, O.mode_omegas(3, 1.5, 1.2)


def test_velocity_step_gradient_matches_central_differences():
    """The peel's gradient is causal: the loss of rank r is differentiated
    with the modes peeled before it frozen (velocity/verify.py
    frozen_prefix_tangent).  For the mode peeled last that is the full
    derivative of sum(losses), so central differences on its parameters
    must match (the reference's own check, tests/test_finite_gauge.py:30-35,
    perturbs the last column the same way)."""
    W, b, X0, E, om = _velocity_case()
    r = O.velocity_step(W, b, X0, E, om)
    last = int(r["order"][-1])
    gW, gb = r["grads"]
    rng = np.random.default_rng(0)
    h = 1e-6
    for _ in range(12):
        j = int(rng.integers(0, len(W)))
        use_w = bool(rng.integers(0, 2))
        arr = W[j] if use_w else b[j]
        idx = (last,) + tuple(int(rng.integers(0, s)) for s in arr.shape[1:])
        x0 = arr[idx]
        arr[idx] = x0 + h
        lp = O.velocity_step(W, b, X0, E, om, want_grad=False)
        arr[idx] = x0 - h
        lm = O.velocity_step(W, b, X0, E, om, want_grad=False)
        arr[idx] = x0
        assert int(lp["order"][-1]) == int(lm["order"][-1]) == last
        fd = (float(lp["losses"].sum()) - float(lm["losses"].sum())) / (2 * h)
        an = (gW if use_w else gb)[j][idx]
        assert abs(fd - an) <= 1e-6 * max(1.0, abs(an)), (j, use_w, idx, fd, an)


# ------------------------------------------- the periodic backend's facade
def test_hardcoded_trial_spaces_and_dispatch():
    """Host-side validation of the periodic backend's API: the supported
    trial spaces, the layer frequencies and the objective dispatch
    (hardcoded_backend.py:1250-1260, :3401-3427, :3796-3811)."""
    from types import SimpleNamespace
    from neb_gb300 import hardcoded as H
    periodic = SimpleNamespace(geometry_mode="periodic_box", envelope_mode="periodic_identity",
                               input_encoding="periodic_sincos_xy")
    assert H._trial_space(periodic) == H.PERIODIC
    airfoil = SimpleNamespace(geometry_mode="cinf_ellipse", envelope_mode="cinf_localized",
                              input_encoding="raw_xy")
    with pytest.raises(NotImplementedError):
        H._trial_space(airfoil)
    assert H.siren_layer_omega(SimpleNamespace(), 0) == 1.0
    c = SimpleNamespace(canonical_siren=True, siren_first_omega0=8.0)
    assert H.siren_layer_omega(c, 0) == 8.0 and H.siren_layer_omega(c, 1) == 30.0
    with pytest.raises(ValueError):
        H.peel_step(SimpleNamespace(basis_objective="nonsense"), None, [])
    with pytest.raises(ValueError):
        H.peel_step(SimpleNamespace(basis_objective="potential_rayleigh"), None, [],
                    reference_model=object())
    with pytest.raises(NotImplementedError):
        H.peel_step(SimpleNamespace(basis_objective="velocity_rayleigh"), None, [])


def test_fixed_order_peel_oracle():
    """With fixed_order the peel keeps network order: T orthonormalises M
    in that order and the losses are the diagonal of T^T S T."""
    rng = np.random.default_rng(2)
    X = rng.normal(size=(40, 6))
    Y = rng.normal(size=(40, 6)) * np.linspace(3, 0.5, 6)
    M, S = X.T @ X / 40, Y.T @ Y / 40
    r = O.coefficient_peel(M, S, sort=False)
    assert list(r["order"]) == list(range(6))
    T = r["T"]
    np.testing.assert_allclose(T.T @ M @ T, np.eye(6), atol=1e-10)
    np.testing.assert_allclose(np.diag(T.T @ S @ T), r["losses"], rtol=1e-10)
    s = O.coefficient_peel(M, S)
    assert list(s["order"]) != list(range(6))


def test_hardcoded_initial_arrays_and_points_match_reference():
    """initial_arrays and fluid_points against the reference trainer's own
    epoch-0 checkpoint and fixed validation points, bit for bit."""
    from neb_gb300 import hardcoded as H
    G = np.load(__file__.rsplit("/", 1)[0] + "/golden/reference_vectors.npz")
    cfg = SimpleNamespace(seed=3, modes=3, hidden=8, hidden_layers=2, frequencies=2,
                          input_features=8, xmin=0.0, xmax=2 * math.pi, ymin=0.0,
                          ymax=2 * math.pi, geometry_mode="periodic_box",
                          envelope_mode="periodic_identity", input_encoding="periodic_sincos_xy",
                          canonical_siren=True, siren_first_omega0=8.0, siren_hidden_omega0=30.0,
                          sampling_mode="uniform_random")
    arrays = H.initial_arrays(cfg)
    ref = {k[5:]: G[k] for k in G.files if k.startswith("init.")}
    assert set(arrays) == set(ref)
    for key, value in ref.items():
        assert np.array_equal(np.asarray(arrays[key], np.float64), value), key
    pts = H.fluid_points(cfg, 37, 0.0, 0.0, cfg.seed + 900000)
    assert pts.dtype == np.float32
    assert np.array_equal(pts.astype(np.float64), G["init_validation_points"])
