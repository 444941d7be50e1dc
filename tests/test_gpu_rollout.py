"""The periodic evaluation pipeline on the GPU (GB300 only), through the C ABI.

* Feature jets of order 1-3 and the third-order fields of the periodic
  backend's networks against the oracle and the reference's forward_stream.
* One Galerkin right-hand side against the oracle: FP64 fields, and FP32
  fields with compensated sums (checked against the oracle run on the same
  FP32-rounded fields, to FP64-class accuracy).
* The Ritz stage and the ETDRK4 rollout against the reference's own rollout
  states, and the whole pipeline (Jet3 sampling on a grid, Ritz, rollout)
  of a small network against the oracle.
"""
import math
from types import SimpleNamespace

import numpy as np
import pytest
import torch

from oracle import neb_oracle as O
from tests.test_rollout_host import G, rollout_case

pytestmark = pytest.mark.gpu


def _needs_gpu():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def _cfg(**kw):
    base = dict(modes=4, hidden=8, hidden_layers=2, frequencies=3, xmin=0.0, xmax=2 * math.pi,
                ymin=0.0, ymax=2 * math.pi, geometry_mode="periodic_box",
                envelope_mode="periodic_identity", input_encoding="periodic_sincos_xy",
                canonical_siren=True, siren_first_omega0=8.0, siren_hidden_omega0=30.0,
                mode_forward_batch=2, mlp_compute_dtype="float32")
    base.update(kw)
    return SimpleNamespace(**base)


def _golden_arrays(prefix):
    n = len(prefix) + 1
    return {k[n:]: G[k] for k in G.files if k.startswith(prefix + ".")}


@pytest.mark.parametrize("precision", ["fp32", "fp64"])
@pytest.mark.parametrize("order", [1, 2, 3])
def test_feature_jets(precision, order):
    _needs_gpu()
    from neb_gb300.hardcoded import HardcodedModel
    cfg = _cfg()
    model = HardcodedModel(cfg, _golden_arrays("hb_in"), precision=precision)
    pts = np.random.default_rng(3).uniform(0, 2 * math.pi, (50, 2))
    got = model.features(cfg, pts, order).double().cpu().numpy()
    ref = np.moveaxis(O.features_periodic_jet(pts, 3, order), 0, 1)
    tol = 1e-6 if precision == "fp32" else 1e-13
    np.testing.assert_allclose(got, ref, rtol=tol, atol=tol * np.abs(ref).max())


@pytest.mark.parametrize("precision,rtol", [("fp32", 3e-5), ("fp64", 1e-9)])
def test_forward_stream_third_order_matches_reference(precision, rtol):
    _needs_gpu()
    from neb_gb300.hardcoded import HardcodedModel
    cfg = _cfg()
    model = HardcodedModel(cfg, _golden_arrays("hb_in"), precision=precision)
    out = list(model.forward_stream(cfg, G["hb_points"]))
    assert [m.mode_index for m, _, _ in out] == [0, 1, 2, 3]
    for name in ("value", "grad", "hess", "third"):
        got = np.stack([getattr(f, name)[:, 0].double().cpu().numpy() for _, f, _ in out])
        ref = G["hb3_" + name]
        np.testing.assert_allclose(got, ref, rtol=rtol, atol=rtol * np.abs(ref).max(),
                                   err_msg=name)


def _rollout_objects(basis, precision, nu):
    """GridBasis / RitzBasis / Rollout of raw fields basis [3, n, K]."""
    from neb_gb300.rollout import GridBasis, Rollout, ritz
    dt = torch.float32 if precision == "fp32" else torch.float64
    n = basis.shape[1]
    UV = torch.tensor(np.stack([basis[0], basis[1]], 1), dtype=dt, device="cuda").contiguous()
    Om = torch.tensor(basis[2], dtype=dt, device="cuda").contiguous()
    gb = GridBasis(UV, Om, None, (2 * math.pi) ** 2 / n, precision)
    rb = ritz(gb)
    return gb, rb, Rollout(gb, rb, nu)


@pytest.mark.parametrize("precision", ["fp32", "fp64"])
def test_galerkin_rhs_matches_oracle(precision):
    """rhs of random Ritz coefficients against the oracle on the same
    fields; FP32 fields are summed with compensated FP32, so the relative
    error stays at the FP64 level."""
    _needs_gpu()
    basis, _, _ = rollout_case()
    if precision == "fp32":
        basis = basis.astype(np.float32).astype(np.float64)
    gb, rb, roll = _rollout_objects(basis, precision, 0.05)
    R = rb.R.cpu().numpy()
    weight = gb.weight
    x = np.random.default_rng(5).normal(size=gb.K)
    got = roll.rhs(torch.tensor(x, device="cuda")).cpu().numpy()
    ref = R.T @ O.galerkin_rhs(basis[0], basis[1], basis[2], weight, R @ x)
    np.testing.assert_allclose(got, ref, rtol=1e-11, atol=1e-12 * np.abs(ref).max())
    assert roll.energy_skew() < 1e-9
    f = roll.fields(torch.tensor(x, device="cuda")).cpu().numpy()
    np.testing.assert_allclose(f, basis @ (R @ x), rtol=1e-11, atol=1e-12 * np.abs(f).max())


@pytest.mark.parametrize("precision,tol", [("fp32", 2e-6), ("fp64", 1e-9)])
def test_rollout_matches_reference(precision, tol):
    """Ritz values and the reconstructed velocity of every frame against
    the reference's rollout (FP32 fields are the golden FP64 fields rounded
    to FP32, which moves the result by ~1e-7)."""
    _needs_gpu()
    basis, u0, v0 = rollout_case()
    gb, rb, roll = _rollout_objects(basis, precision, float(G["roll_nu"]))
    np.testing.assert_allclose(rb.lam.cpu().numpy(), G["roll_vals"], rtol=max(tol, 1e-10))
    c0 = roll.project(u0, v0)
    states = roll.run(c0, G["roll_times"], float(G["roll_dt"]))
    R = rb.R.cpu().numpy()
    u = (states @ R.T) @ basis[0].T  # raw-field coefficients -> u at every point
    ref = G["roll_u_frames"]
    np.testing.assert_allclose(u[:, :64], ref, rtol=tol, atol=tol * np.abs(ref).max())
    # the same states through the library's reconstruction
    f = roll.fields(torch.tensor(states[-1], device="cuda")).cpu().numpy()
    np.testing.assert_allclose(f[0, :64], ref[-1], rtol=tol, atol=tol * np.abs(ref).max())


def test_graph_replay_equals_launches():
    _needs_gpu()
    basis, u0, v0 = rollout_case()
    gb, rb, roll = _rollout_objects(basis, "fp64", 0.05)
    c0 = roll.project(u0, v0)
    a = roll.run(c0, [0.0, 0.1, 0.25], 0.02)
    roll.use_graph, roll._graph, roll.h = False, None, None
    b = roll.run(c0, [0.0, 0.1, 0.25], 0.02)
    np.testing.assert_array_equal(a, b)


def test_pipeline_on_a_network_matches_oracle():
    """Jet3 fields of a six-mode network on a 24 x 24 grid, Ritz stage and
    ten ETDRK4 steps, against the oracle (FP64)."""
    _needs_gpu()
    from neb_gb300.hardcoded import HardcodedModel, initial_arrays
    from neb_gb300.rollout import Rollout, grid_points, ritz, sample_basis
    cfg = _cfg(modes=6, hidden=16, hidden_layers=2, frequencies=2, input_features=8, seed=4,
               mode_forward_batch=6)
    arrays = initial_arrays(cfg)
    model = HardcodedModel(cfg, arrays, precision="fp64")
    gb = sample_basis(model, cfg, 24, diagnostics=True)
    pts = grid_points(24, cfg)
    X = O.features_periodic_jet(pts, 2, 3)
    E = np.zeros((10, len(pts), 1)); E[0] = 1.0
    labels = ("l0", "l1", "output")
    fields = []
    for k in range(6):
        Wk = [arrays[f"m{k:03d}.{lab}.weight"].astype(np.float64) for lab in labels]
        bk = [arrays[f"m{k:03d}.{lab}.bias"].astype(np.float64) for lab in labels]
        fields.append(O.stream_fields(O.mode_forward(Wk, bk, X, E, 2, 3,
                                                     O.mode_omegas(3, 8.0, 30.0))[2]))
    ref = np.stack(fields, -1)  # [6 channels, n, K]
    tol = 1e-9 * np.abs(ref).max()
    np.testing.assert_allclose(gb.UV[:, 0].cpu().numpy(), ref[1], atol=tol)
    np.testing.assert_allclose(gb.UV[:, 1].cpu().numpy(), ref[2], atol=tol)
    np.testing.assert_allclose(gb.Om.cpu().numpy(), ref[3], atol=tol)
    np.testing.assert_allclose(gb.diag.cpu().numpy(), ref[[0, 4, 5]].transpose(1, 0, 2),
                               atol=tol)
    rb = ritz(gb)
    vals, Rr, _ = O.ritz_basis(ref[1], ref[2], ref[3], gb.weight)
    np.testing.assert_allclose(rb.lam.cpu().numpy(), vals, rtol=1e-8)
    roll = Rollout(gb, rb, 0.01)
    c0 = roll.project(np.sin(pts[:, 1]), np.sin(pts[:, 0]))
    states = roll.run(c0, [0.0, 0.05], 0.005)
    gu, gv, gw = ref[1] @ Rr, ref[2] @ Rr, ref[3] @ Rr
    rc0 = gb.weight * (gu.T @ np.sin(pts[:, 1]) + gv.T @ np.sin(pts[:, 0]))
    rs = O.etdrk4_rollout(gu, gv, gw, vals, 0.01, rc0, [0.0, 0.05], 0.005, gb.weight)
    R = rb.R.cpu().numpy()
    # compare velocities (the Ritz vectors' signs may differ)
    np.testing.assert_allclose(ref[1] @ (R @ states[-1]), gu @ rs[-1], rtol=1e-8,
                               atol=1e-9 * np.abs(gu @ rs[-1]).max())
