"""The FP64 oracle against vectors produced by the reference's own functions.

The fixtures come from ``tests/golden/make_golden.py``, which runs the
reference's CuPy code on the CPU through a NumPy stand-in for ``cupy``.
"""
import math

import numpy as np
import pytest

from oracle import neb_oracle as O

G = np.load(__import__("os").path.join(__import__("os").path.dirname(__file__),
                                       "golden", "reference_vectors.npz"))
TOL = dict(rtol=1e-12, atol=1e-12)


def lap_of(hess):
    return hess[..., 0] + hess[..., 2]


def test_tanh_jet_forward_matches_unary2():
    Z = np.stack([G["act2d_z"], G["act2d_grad"][..., 0], G["act2d_grad"][..., 1],
                  lap_of(G["act2d_hess"])])
    Y = O.act_forward(Z, 2, "tanh")
    np.testing.assert_allclose(Y[0], G["act2d_y"], **TOL)
    np.testing.assert_allclose(Y[1], G["act2d_ygrad"][..., 0], **TOL)
    np.testing.assert_allclose(Y[2], G["act2d_ygrad"][..., 1], **TOL)
    np.testing.assert_allclose(Y[3], lap_of(G["act2d_yhess"]), **TOL)


def test_tanh_jet_transpose_matches_unary_backward_jet2():
    Z = np.stack([G["act2d_z"], G["act2d_grad"][..., 0], G["act2d_grad"][..., 1],
                  lap_of(G["act2d_hess"])])
    Yb = np.stack([G["act2d_av"], G["act2d_ag"][..., 0], G["act2d_ag"][..., 1], G["act2d_al"]])
    Zb = O.act_backward(Z, Yb, 2, "tanh")
    np.testing.assert_allclose(Zb[0], G["act2d_zb"], **TOL)
    np.testing.assert_allclose(Zb[1], G["act2d_gb"][..., 0], **TOL)
    np.testing.assert_allclose(Zb[2], G["act2d_gb"][..., 1], **TOL)
    # the Laplacian adjoint lands on hxx and hyy alike
    np.testing.assert_allclose(Zb[3], G["act2d_hb"][..., 0], **TOL)
    np.testing.assert_allclose(Zb[3], G["act2d_hb"][..., 2], **TOL)


def test_linear_jet_layer_and_transpose():
    X = np.stack([G["lin_x"], G["lin_xg"][..., 0], G["lin_xg"][..., 1], lap_of(G["lin_xh"])])
    Z = O.linear_forward(X, G["lin_W"], G["lin_b"])
    np.testing.assert_allclose(Z[0], G["lin_z"], **TOL)
    np.testing.assert_allclose(Z[1], G["lin_zg"][..., 0], **TOL)
    np.testing.assert_allclose(Z[3], lap_of(G["lin_zh"]), **TOL)
    # transpose on the full (value, grad, hess) channel set = 6 channels
    X6 = np.stack([G["lin_x"], G["lin_xg"][..., 0], G["lin_xg"][..., 1],
                   G["lin_xh"][..., 0], G["lin_xh"][..., 1], G["lin_xh"][..., 2]])
    A6 = np.stack([G["lin_av"], G["lin_ag"][..., 0], G["lin_ag"][..., 1],
                   G["lin_ah"][..., 0], G["lin_ah"][..., 1], G["lin_ah"][..., 2]])
    Xb, gW, gb = O.linear_backward(X6, A6, G["lin_W"])
    np.testing.assert_allclose(gW, G["lin_gW"], **TOL)
    np.testing.assert_allclose(gb, G["lin_gb"], **TOL)
    np.testing.assert_allclose(Xb[0], G["lin_xbv"], **TOL)
    np.testing.assert_allclose(Xb[4], G["lin_xbh"][..., 1], **TOL)


def test_periodic_features_match_encoding_jet2():
    F = int(G["enc_frequencies"])
    X = O.features_periodic(G["enc_points"], F)
    np.testing.assert_allclose(X[0], G["enc_value"], **TOL)
    np.testing.assert_allclose(X[1], G["enc_grad"][..., 0], **TOL)
    np.testing.assert_allclose(X[2], G["enc_grad"][..., 1], **TOL)
    np.testing.assert_allclose(X[3], lap_of(G["enc_hess"]), rtol=1e-12, atol=1e-10)


def _z3():
    return np.concatenate([G["act3d_z"][None], np.moveaxis(G["act3d_grad"], -1, 0),
                           np.moveaxis(G["act3d_hess"], -1, 0)])


def test_3d_jet_chain_rule_and_transpose_match_velocity_trace_jet2():
    Z = _z3()
    Y = O.act_forward(Z, 3, "sin")
    np.testing.assert_allclose(Y[0], G["act3d_y"], **TOL)
    np.testing.assert_allclose(np.moveaxis(Y[1:4], 0, -1), G["act3d_ygrad"], **TOL)
    np.testing.assert_allclose(np.moveaxis(Y[4:], 0, -1), G["act3d_yhess"], **TOL)
    Yb = np.concatenate([G["act3d_av"][None], np.moveaxis(G["act3d_ag"], -1, 0),
                         np.moveaxis(G["act3d_ah"], -1, 0)])
    Zb = O.act_backward(Z, Yb, 3, "sin")
    np.testing.assert_allclose(Zb[0], G["act3d_zb"], **TOL)
    np.testing.assert_allclose(np.moveaxis(Zb[1:4], 0, -1), G["act3d_gb"], **TOL)
    np.testing.assert_allclose(np.moveaxis(Zb[4:], 0, -1), G["act3d_hb"], **TOL)


def _psi3():
    k, n, _ = G["f3_value"].shape
    P = np.zeros((10, n, 3 * k))
    for m in range(k):
        for c in range(3):
            P[0, :, 3 * m + c] = G["f3_value"][m, :, c]
            P[1:4, :, 3 * m + c] = G["f3_grad"][m, :, c, :].T
            P[4:, :, 3 * m + c] = G["f3_hess"][m, :, c, :].T
    return P


def test_3d_fields_and_adjoint_match_velocity_trace_jet2():
    U, Om = O.fields_3d(_psi3())
    np.testing.assert_allclose(np.moveaxis(U, 0, -1).transpose(1, 0, 2), G["f3_u"], **TOL)
    np.testing.assert_allclose(np.moveaxis(Om, 0, -1).transpose(1, 0, 2), G["f3_w"], **TOL)
    k = G["f3_gu"].shape[0]
    Ub = np.moveaxis(G["f3_gu"], -1, 0).transpose(0, 2, 1)   # [3, n, k]
    Wb = np.moveaxis(G["f3_gw"], -1, 0).transpose(0, 2, 1)
    Pb = O.fields_adjoint(Ub, Wb, 3, 3 * k)
    for m in range(k):
        for c in range(3):
            np.testing.assert_allclose(Pb[1:4, :, 3 * m + c].T, G["f3_lift_grad"][m, :, c, :], **TOL)
            np.testing.assert_allclose(Pb[4:, :, 3 * m + c].T, G["f3_lift_hess"][m, :, c, :], **TOL)


def _stack3(A):
    n = A.shape[0] // 3
    return np.stack([A[a::3] for a in range(3)])    # rows are (point, component)


def test_grams_and_generalized_eigenpairs():
    U, D = _stack3(G["gram_U"]), _stack3(G["gram_D"])
    n = U.shape[1]
    M, S = O.grams(U, D, 1.0 / n)
    np.testing.assert_allclose(M, G["gram_M"], **TOL)
    np.testing.assert_allclose(S, G["gram_S"], **TOL)
    lam, V, r = O.finite_pencil(S, M)
    assert r == M.shape[0]
    np.testing.assert_allclose(lam, G["eig_lam"], rtol=1e-12)
    np.testing.assert_allclose(np.abs(V), np.abs(G["eig_V"]), rtol=1e-9, atol=1e-12)


def test_trace_objective_and_field_adjoints():
    U, D = _stack3(G["gram_U"]), _stack3(G["gram_D"])
    n, k = U.shape[1], U.shape[2]
    M, S = O.grams(U, D, 1.0 / n)
    obj = O.spectral_objective(M, S, "trace")
    np.testing.assert_allclose(obj["loss"] / k, float(G["trace_loss"]), rtol=1e-12)
    GU = np.stack([2.0 / n * U[a] @ obj["GM"] for a in range(3)]) / k
    GO = np.stack([2.0 / n * D[a] @ obj["GS"] for a in range(3)]) / k
    ref_GU, ref_GO = _stack3(G["trace_GU"]), _stack3(G["trace_GO"])
    np.testing.assert_allclose(GU, ref_GU, rtol=1e-10, atol=1e-13)
    np.testing.assert_allclose(GO, ref_GO, rtol=1e-10, atol=1e-13)


def _ncc_params():
    L = int(G["ncc_layers"])
    om = G["ncc_omega"]
    params = []
    for j in range(L):
        s = (om[0] if j == 0 else om[1]) if j < L - 1 else 1.0
        params.append((s * G[f"ncc_W{j}"], s * G[f"ncc_b{j}"]))
    return params, L, om


def test_network_forward_reverse_match_reference_model():
    """The reference Model with omega folded into W, b equals the oracle with
    act='sin' on the value/gradient channels (Hessian channels unused)."""
    params, L, om = _ncc_params()
    n = G["ncc_feat"].shape[0]
    X0 = np.zeros((10, n, 15))
    X0[0] = G["ncc_feat"]
    X0[1:4] = np.moveaxis(G["ncc_fgrad"], -1, 0)
    xs, zs, Psi = O.mlp_forward(params, X0, 3, "sin")
    np.testing.assert_allclose(Psi[0], G["ncc_value"], rtol=1e-11, atol=1e-12)
    np.testing.assert_allclose(np.moveaxis(Psi[1:4], 0, -1), G["ncc_grad"], rtol=1e-11, atol=1e-12)
    Pb = np.zeros_like(Psi)
    Pb[0] = G["ncc_av"]
    Pb[1:4] = np.moveaxis(G["ncc_ag"], -1, 0)
    grads = O.mlp_backward(params, xs, zs, Pb, 3, "sin")
    for j in range(L):
        s = (om[0] if j == 0 else om[1]) if j < L - 1 else 1.0
        # chain rule through W' = s W
        np.testing.assert_allclose(s * grads[j][0], G[f"ncc_gW{j}"], rtol=1e-10, atol=1e-11)
        np.testing.assert_allclose(s * grads[j][1], G[f"ncc_gb{j}"], rtol=1e-10, atol=1e-11)


def test_adam_matches_reference_model():
    L = int(G["ncc_layers"])
    params = [(G[f"ncc_W{j}"], G[f"ncc_b{j}"]) for j in range(L)]
    grads = [(G[f"ncc_gW{j}"], G[f"ncc_gb{j}"]) for j in range(L)]
    mom = O.zero_moments(params)
    params, mom, _ = O.adam_step(params, mom, grads, 0, 1e-3, clip=0.5)
    grads2 = [(2 * gw, -gb) for gw, gb in grads]
    params, mom, _ = O.adam_step(params, mom, grads2, 1, 1e-3, clip=0.5)
    # the reference Model keeps its parameters and moments in FP32
    # (native_cupy_core.py:121-127), hence FP32-level tolerances here
    for j in range(L):
        np.testing.assert_allclose(params[j][0], G[f"ncc_W{j}_after"], rtol=2e-6, atol=2e-8)
        np.testing.assert_allclose(params[j][1], G[f"ncc_b{j}_after"], rtol=2e-6, atol=2e-8)
        np.testing.assert_allclose(mom[j][0][0], G[f"ncc_mW{j}"], rtol=2e-6, atol=1e-10)
        np.testing.assert_allclose(mom[j][0][1], G[f"ncc_vW{j}"], rtol=2e-5, atol=1e-12)


def test_adam_rejects_invalid_gradients_without_change():
    params = [(np.ones((2, 2)), np.zeros(2))]
    mom = O.zero_moments(params)
    with pytest.raises(FloatingPointError):
        O.adam_step(params, mom, [(np.full((2, 2), np.nan), np.zeros(2))], 0, 1e-3)
    with pytest.raises(FloatingPointError):
        O.adam_step(params, mom, [(np.zeros((2, 2)), np.zeros(2))], 0, 1e-3)


# ------------------------------------------- mode-stacked SIREN networks
def _jet1(value, grad):
    """[n, F] value and [n, F, d] gradient -> channel-first [1 + d, n, F]."""
    return np.concatenate([value[None], np.moveaxis(grad, -1, 0)])


def _jet2(value, grad, hess):
    return np.concatenate([value[None], np.moveaxis(grad, -1, 0), np.moveaxis(hess, -1, 0)])


def test_mode_network_with_envelope_matches_reference_model():
    """Two modes, first-order jets, a random envelope: forward, reverse and
    two Adam steps with per-mode norms, against native_cupy_core.Model."""
    layers = 3
    W = [G[f"env_W{j}"] for j in range(layers)]
    b = [G[f"env_b{j}"] for j in range(layers)]
    X0 = _jet1(G["env_feat"], G["env_fgrad"])
    E = _jet1(G["env_ev"], G["env_eg"])
    om = O.mode_omegas(layers, 2.3, 1.7)
    gW = [np.zeros_like(w) for w in W]
    gb = [np.zeros_like(x) for x in b]
    for k in range(2):
        xs, pres, out = O.mode_forward([w[k] for w in W], [x[k] for x in b], X0, E, 3, 1, om)
        np.testing.assert_allclose(out[0], G["env_value"][k], rtol=1e-6, atol=1e-6)
        np.testing.assert_allclose(np.moveaxis(out[1:], 0, -1), G["env_grad"][k], rtol=1e-6,
                                   atol=1e-6)
        A = _jet1(G["env_av"][k], G["env_ag"][k])
        gwk, gbk = O.mode_backward([w[k] for w in W], xs, pres, E, A, 3, 1, om)
        for j in range(layers):
            gW[j][k], gb[j][k] = gwk[j], gbk[j]
    for j in range(layers):
        np.testing.assert_allclose(gW[j], G[f"env_gW{j}"], rtol=1e-6, atol=1e-6)
        np.testing.assert_allclose(gb[j], G[f"env_gb{j}"], rtol=1e-6, atol=1e-6)
    zeros = [np.zeros_like(w) for w in W], [np.zeros_like(x) for x in b]
    st, n1 = O.mode_adam(W, b, zeros[0], zeros[0], zeros[1], zeros[1], gW, gb, 0, 1e-3, 0.5)
    st, n2 = O.mode_adam(st[0], st[1], st[2], st[3], st[4], st[5], [2 * g for g in gW],
                         [-g for g in gb], st[6], 1e-3, 0.5)
    np.testing.assert_allclose(n1, G["env_norms1"], rtol=1e-6)
    np.testing.assert_allclose(n2, G["env_norms2"], rtol=1e-6)
    for j in range(layers):
        np.testing.assert_allclose(st[0][j], G[f"env_W{j}_after"], rtol=1e-6, atol=1e-7)
        np.testing.assert_allclose(st[1][j], G[f"env_b{j}_after"], rtol=1e-6, atol=1e-7)
    assert st[6] == 2


def test_gram_form_peel_matches_coefficient_peel():
    p = O.coefficient_peel(G["peel_M"], G["peel_S"])
    np.testing.assert_array_equal(p["order"], G["peel_order"])
    np.testing.assert_allclose(p["losses"], G["peel_losses"], rtol=1e-12)
    for key in ("T", "Cu", "Cd"):
        np.testing.assert_allclose(p[key], G[f"peel_{key}"], rtol=1e-10,
                                   atol=1e-12 * np.abs(G[f"peel_{key}"]).max())


def test_velocity_step_matches_reference_composition():
    """Second-order 3D mode network with envelope, velocity and velocity
    gradient fields, Grams, the Gram-form peel and the parameter gradient,
    against the reference's velocity_trace_jet2 / velocity/core.py functions
    composed as core.py compute composes them."""
    layers = int(G["vel_layers"])
    W = [G[f"vel_W{j}"] for j in range(layers)]
    b = [G[f"vel_b{j}"] for j in range(layers)]
    X0 = _jet2(G["vel_fv"], G["vel_fg"], G["vel_fh"])
    E = _jet2(G["vel_ev"], G["vel_eg"], G["vel_eh"])
    om = O.mode_omegas(layers, *G["vel_omega"])
    r = O.velocity_step(W, b, X0, E, om)
    np.testing.assert_allclose(r["U"], G["vel_U"], rtol=1e-10, atol=1e-12)
    np.testing.assert_allclose(r["D"], G["vel_D"], rtol=1e-10, atol=1e-12)
    np.testing.assert_allclose(r["M"], G["vel_M"], rtol=1e-10, atol=1e-12)
    np.testing.assert_allclose(r["S"], G["vel_S"], rtol=1e-10, atol=1e-12)
    np.testing.assert_array_equal(r["order"], G["vel_order"])
    np.testing.assert_allclose(r["losses"], G["vel_losses"], rtol=1e-9)
    gW, gb = r["grads"]
    for j in range(layers):
        np.testing.assert_allclose(gW[j], G[f"vel_gW{j}"], rtol=1e-8,
                                   atol=1e-10 * np.abs(G[f"vel_gW{j}"]).max())
        np.testing.assert_allclose(gb[j], G[f"vel_gb{j}"], rtol=1e-8,
                                   atol=1e-10 * np.abs(G[f"vel_gb{j}"]).max())


# ------------------------------------------- the periodic backend's peel step
def _hb_arrays(prefix):
    W = [np.stack([G[f"{prefix}.m{k:03d}.{lab}.weight"] for k in range(4)])
         for lab in ("l0", "l1", "output")]
    b = [np.stack([G[f"{prefix}.m{k:03d}.{lab}.bias"] for k in range(4)])
         for lab in ("l0", "l1", "output")]
    return W, b


def test_periodic_fields_match_forward_stream_jet1():
    W, b = _hb_arrays("hb_in")
    X0 = O.features_periodic(G["hb_points"], 3)[:3]
    E = np.zeros((3, 48, 1)); E[0] = 1.0
    om = O.mode_omegas(3, 8.0, 30.0)
    for k in range(4):
        _, _, out = O.mode_forward([w[k] for w in W], [x[k] for x in b], X0, E, 2, 1, om)
        np.testing.assert_allclose(out[0][:, 0], G["hb_value"][k], rtol=1e-9, atol=1e-10)
        np.testing.assert_allclose(np.stack([out[1][:, 0], out[2][:, 0]], -1), G["hb_grad"][k],
                                   rtol=1e-9, atol=1e-9)


def test_potential_peel_step_matches_reference_peel_step():
    """One training step of the reference's streamfunction Rayleigh peel
    (its loss, per-rank energies, causal order and the parameters after its
    device Adam) against the oracle's Gram-form restatement."""
    W, b = _hb_arrays("hb_in")
    X0 = O.features_periodic(G["hb_points"], 3)[:3]
    weight = (2 * math.pi) ** 2 / 48
    r = O.potential_peel_step(W, b, X0, weight, O.mode_omegas(3, 8.0, 30.0), lr=1e-3, clip=5.0)
    np.testing.assert_array_equal(r["order"], G["hb_order"])
    np.testing.assert_allclose(r["losses"], G["hb_energies"], rtol=1e-6)
    np.testing.assert_allclose(r["loss"], G["hb_loss"], rtol=1e-6)
    np.testing.assert_allclose([r["norms"].min(), r["norms"].max()],
                               [G["hb_norm_min"], G["hb_norm_max"]], rtol=1e-9)
    W2, b2 = _hb_arrays("hb_out")
    for j in range(3):
        np.testing.assert_allclose(r["state"][0][j], W2[j], rtol=1e-9, atol=1e-12)
        np.testing.assert_allclose(r["state"][1][j], b2[j], rtol=1e-9, atol=1e-12)


def test_fixed_order_and_free_box_peel_steps_match_reference():
    """The reference's peel step with fixed-order sorting (the same four
    periodic networks) and on the free box (raw_xy inputs, three networks):
    losses, energies, order and the parameters after its device Adam."""
    W, b = _hb_arrays("hb_in")
    X0 = O.features_periodic(G["hb_points"], 3)[:3]
    r = O.potential_peel_step(W, b, X0, (2 * math.pi) ** 2 / 48, O.mode_omegas(3, 8.0, 30.0),
                              lr=1e-3, clip=5.0, sort=False)
    np.testing.assert_array_equal(r["order"], G["hbf_order"])
    np.testing.assert_allclose(r["losses"], G["hbf_energies"], rtol=1e-6)
    W2, b2 = _hb_arrays("hbf_out")
    for j in range(3):
        np.testing.assert_allclose(r["state"][0][j], W2[j], rtol=1e-9, atol=1e-12)
    labels = ("l0", "l1", "output")
    Wf = [np.stack([G[f"hbfree_in.m{k:03d}.{lab}.weight"] for k in range(3)]) for lab in labels]
    bf = [np.stack([G[f"hbfree_in.m{k:03d}.{lab}.bias"] for k in range(3)]) for lab in labels]
    pts = G["hbfree_points"]
    X = np.zeros((3, len(pts), 2))
    X[0] = pts
    X[1, :, 0] = 1.0
    X[2, :, 1] = 1.0
    r = O.potential_peel_step(Wf, bf, X, 3.0 * 1.5 / len(pts), O.mode_omegas(3, 3.0, 2.0),
                              lr=1e-3, clip=5.0)
    np.testing.assert_array_equal(r["order"], G["hbfree_order"])
    np.testing.assert_allclose(r["losses"], G["hbfree_energies"], rtol=1e-6)
    for j, lab in enumerate(labels):
        ref = np.stack([G[f"hbfree_out.m{k:03d}.{lab}.weight"] for k in range(3)])
        np.testing.assert_allclose(r["state"][0][j], ref, rtol=1e-9, atol=1e-12)
