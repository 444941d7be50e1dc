"""FP64 NumPy oracle for the neural-eigenfluid hot path.

TEST INFRASTRUCTURE ONLY.  This module is the reference that the CUDA product
is compared against; the product (``neb_gb300``) never imports, links or calls it.
Only ``tests/``, ``__graft_entry__.smoke()`` and the ``cpu_baseline`` /
``--impl reference`` legs of ``bench.py`` may use it.

It restates, in plain FP64 NumPy, the algorithm of the reference
(baiming-zhang/NEB) for the path "jet MLP -> fields -> weighted Grams ->
generalized eigenproblem -> spectral objective -> hand-written reverse pass ->
Adam", specialised to the shared tanh network of the benchmark configurations:

* jet algebra (value / gradient / Laplacian in 2D, value / gradient / Hessian in
  3D) follows the reference's chain rule ``unary2``
  (experiments/2d/_backend/periodic_core/vortex_merger/src/eigenfluid/gen/
  vortex_merger2d/hardcoded_backend.py:252-271) and its transpose
  ``unary_backward_jet2`` (same file :1147-1173), and the 3D compact Jet2 of
  experiments/metaball/_backend/flow/cases/metaball/velocity_trace_jet2.py:31-55;
* the linear layer and its transpose follow ``linear_forward_batch_jet2`` /
  ``linear_backward_batch_jet2`` (hardcoded_backend.py:1005-1035, :1115-1144):
  one weight matrix for every jet channel, bias on the value channel only;
* periodic Fourier features follow ``encoding_jet2`` ``periodic_sincos_xy``
  (hardcoded_backend.py:576-588): for axis in (x, y), for n, (sin, cos);
* fields follow u = (d_y psi, -d_x psi), omega = -lap psi in 2D and
  u = curl A, omega = curl curl A in 3D (velocity_trace_jet2.py:93-98);
* Grams follow M = sum_p w u_i.u_j, S = sum_p w omega_i.omega_j
  (experiments/periodic/paper_rollout.py:171-179,
  experiments/metaball/_backend/flow/cases/metaball/velocity/core.py:40-46);
* the generalized eigenproblem follows ``scipy.linalg.eigh(S, M)``
  (paper_rollout.py:187) and the trace objective's adjoints follow
  ``trace_objective`` (velocity_trace_jet2.py:107-117);
* Adam follows ``Model.adam`` (experiments/metaball/_backend/flow/cases/
  metaball/native_cupy_core.py:156-171).

Array convention: a jet is one array ``[C, N, F]`` with the channel first.
2D channels (C=4): value, d/dx, d/dy, Laplacian.  3D channels (C=10): value,
d/dx, d/dy, d/dz, then the Hessian entries in the order
(xx, xy, xz, yy, yz, zz) of velocity_trace_jet2.py:9.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np
import scipy.linalg as sla

PAIRS = [(0, 0), (0, 1), (0, 2), (1, 1), (1, 2), (2, 2)]
_HI = {p: i for i, p in enumerate(PAIRS)}


def hid(a: int, b: int) -> int:
    """Hessian slot of the unordered pair (a, b) (velocity_trace_jet2.py:9-11)."""
    return _HI[tuple(sorted((a, b)))]


def channels(dim: int) -> int:
    return 4 if dim == 2 else 10


# --------------------------------------------------------------------------
# activations: value and first three derivatives
# --------------------------------------------------------------------------
def tanh_derivs(z):
    t = np.tanh(z)
    s1 = 1.0 - t * t
    s2 = -2.0 * t * s1
    s3 = -2.0 * s1 * (s1 - 2.0 * t * t)
    return t, s1, s2, s3


def sin_derivs(z):
    s, c = np.sin(z), np.cos(z)
    return s, c, -s, -c


ACTIVATIONS = {"tanh": tanh_derivs, "sin": sin_derivs}


# --------------------------------------------------------------------------
# jet chain rule and its transpose
# --------------------------------------------------------------------------
def act_forward(Z, dim, act="tanh"):
    """y = s(z); grad y = s' grad z; 2D: lap y = s' lap z + s'' |grad z|^2;
    3D: H y = s' H z + s'' grad z grad z^T  (hardcoded_backend.py:252-271)."""
    t, s1, s2, _ = ACTIVATIONS[act](Z[0])
    Y = np.empty_like(Z)
    Y[0] = t
    for a in range(dim):
        Y[1 + a] = s1 * Z[1 + a]
    if dim == 2:
        Y[3] = s1 * Z[3] + s2 * (Z[1] ** 2 + Z[2] ** 2)
    else:
        for k, (i, j) in enumerate(PAIRS):
            Y[4 + k] = s1 * Z[4 + k] + s2 * Z[1 + i] * Z[1 + j]
    return Y


def act_backward(Z, Ybar, dim, act="tanh"):
    """Transpose of :func:`act_forward` (hardcoded_backend.py:1147-1173,
    velocity_trace_jet2.py:35-41, with the tanh derivatives)."""
    t, s1, s2, s3 = ACTIVATIONS[act](Z[0])
    Zb = np.empty_like(Z)
    zb = Ybar[0] * s1
    for a in range(dim):
        zb = zb + Ybar[1 + a] * Z[1 + a] * s2
        Zb[1 + a] = s1 * Ybar[1 + a]
    if dim == 2:
        g2 = Z[1] ** 2 + Z[2] ** 2
        zb = zb + Ybar[3] * (s2 * Z[3] + s3 * g2)
        Zb[1] += 2.0 * s2 * Ybar[3] * Z[1]
        Zb[2] += 2.0 * s2 * Ybar[3] * Z[2]
        Zb[3] = s1 * Ybar[3]
    else:
        for k, (i, j) in enumerate(PAIRS):
            hb = Ybar[4 + k]
            zb = zb + hb * (s2 * Z[4 + k] + s3 * Z[1 + i] * Z[1 + j])
            Zb[1 + i] += s2 * hb * Z[1 + j]
            Zb[1 + j] += s2 * hb * Z[1 + i]
            Zb[4 + k] = s1 * hb
    Zb[0] = zb
    return Zb


def linear_forward(X, W, b):
    """z_c = W x_c for every channel c, + b on the value channel
    (hardcoded_backend.py:1005-1035)."""
    Z = X @ W.T
    Z[0] += b
    return Z


def linear_backward(X, Zbar, W):
    """Transpose (hardcoded_backend.py:1115-1144): Xbar_c = Zbar_c W,
    gW = sum_c Zbar_c^T X_c, gb = sum_points Zbar_value."""
    Xbar = Zbar @ W
    gW = np.tensordot(Zbar, X, axes=([0, 1], [0, 1]))
    gb = Zbar[0].sum(axis=0)
    return Xbar, gW, gb


# --------------------------------------------------------------------------
# input features with jets
# --------------------------------------------------------------------------
def features_periodic(points, frequencies=16, period=2 * math.pi):
    """Fourier features sin/cos(n s), s in (x, y), n = 1..F with value,
    gradient and Laplacian channels (hardcoded_backend.py:576-588 with
    xmin=0, xmax=period, so phase = 2 pi n s / period)."""
    points = np.asarray(points, dtype=np.float64)
    n_pts = len(points)
    out = np.zeros((4, n_pts, 4 * frequencies))
    col = 0
    for axis in range(2):
        s = points[:, axis]
        for n in range(1, frequencies + 1):
            k = 2.0 * math.pi * n / period
            sn, cs = np.sin(k * s), np.cos(k * s)
            out[0, :, col] = sn
            out[1 + axis, :, col] = k * cs
            out[3, :, col] = -k * k * sn
            col += 1
            out[0, :, col] = cs
            out[1 + axis, :, col] = -k * sn
            out[3, :, col] = -k * k * cs
            col += 1
    return out


MULTIHOLE_CENTRES = np.array([[0.3, 0.3], [0.7, 0.4], [0.45, 0.75]])
MULTIHOLE_RADII = np.array([0.10, 0.08, 0.09])


def features_multihole(points, centres=MULTIHOLE_CENTRES):
    """Raw (x, y) plus one atan2 angle about each hole centre.  The angle is
    harmonic, so its Laplacian channel is zero."""
    p = np.asarray(points, dtype=np.float64)
    n_pts = len(p)
    out = np.zeros((4, n_pts, 2 + len(centres)))
    out[0, :, 0], out[1, :, 0] = p[:, 0], 1.0
    out[0, :, 1], out[2, :, 1] = p[:, 1], 1.0
    for h, (cx, cy) in enumerate(centres):
        dx, dy = p[:, 0] - cx, p[:, 1] - cy
        r2 = dx * dx + dy * dy
        out[0, :, 2 + h] = np.arctan2(dy, dx)
        out[1, :, 2 + h] = -dy / r2
        out[2, :, 2 + h] = dx / r2
    return out


def features_raw3d(points):
    p = np.asarray(points, dtype=np.float64)
    out = np.zeros((10, len(p), 3))
    for a in range(3):
        out[0, :, a] = p[:, a]
        out[1 + a, :, a] = 1.0
    return out


# --------------------------------------------------------------------------
# network
# --------------------------------------------------------------------------
def glorot_init(widths, seed):
    """Glorot-normal weights, std sqrt(2/(fan_in+fan_out)), zero biases, drawn
    layer by layer from numpy.random.default_rng(seed)."""
    rng = np.random.default_rng(seed)
    params = []
    for fan_in, fan_out in zip(widths[:-1], widths[1:]):
        std = math.sqrt(2.0 / (fan_in + fan_out))
        params.append((rng.normal(0.0, std, (fan_out, fan_in)), np.zeros(fan_out)))
    return params


def mlp_forward(params, X0, dim, act="tanh"):
    """Hidden layers with the jet activation, then the linear output layer.
    Returns (inputs of every layer, pre-activations of hidden layers, output
    jet).  Matches ``forward`` of velocity_trace_jet2.py:65-76 without the
    envelope (identity envelope of the periodic and benchmark cases)."""
    X = X0
    xs, zs = [], []
    for W, b in params[:-1]:
        xs.append(X)
        Z = linear_forward(X, W, b)
        zs.append(Z)
        X = act_forward(Z, dim, act)
    xs.append(X)
    W, b = params[-1]
    return xs, zs, linear_forward(X, W, b)


def mlp_backward(params, xs, zs, Psibar, dim, act="tanh"):
    """Hand-written reverse of :func:`mlp_forward`
    (velocity_trace_jet2.py:77-82)."""
    grads = [None] * len(params)
    Xbar, gW, gb = linear_backward(xs[-1], Psibar, params[-1][0])
    grads[-1] = (gW, gb)
    for layer in range(len(params) - 2, -1, -1):
        Zbar = act_backward(zs[layer], Xbar, dim, act)
        Xbar, gW, gb = linear_backward(xs[layer], Zbar, params[layer][0])
        grads[layer] = (gW, gb)
    return grads


# --------------------------------------------------------------------------
# fields and Grams
# --------------------------------------------------------------------------
def fields_2d(Psi):
    """u = (d_y psi, -d_x psi), omega = -lap psi; U stacked [2, N, K]."""
    U = np.stack([Psi[2], -Psi[1]])
    Om = -Psi[3][None]
    return U, Om


def fields_3d(Psi):
    """A_k = (psi_{3k}, psi_{3k+1}, psi_{3k+2}); u = curl A, omega = curl u
    = grad div A - lap A (velocity_trace_jet2.py:93-98).  Returns [3, N, K]."""
    K = Psi.shape[2] // 3

    def g(comp, axis):  # d_axis A_comp  -> [N, K]
        return Psi[1 + axis][:, comp::3]

    def h(comp, a, b):
        return Psi[4 + hid(a, b)][:, comp::3]

    U = np.stack([g(2, 1) - g(1, 2), g(0, 2) - g(2, 0), g(1, 0) - g(0, 1)])
    Om = np.stack([sum(h(b, a, b) - h(a, b, b) for b in range(3)) for a in range(3)])
    assert U.shape[2] == K
    return U, Om


def fields(Psi, dim):
    return fields_2d(Psi) if dim == 2 else fields_3d(Psi)


def grams(U, Om, w):
    """M = sum_p w_p u_i.u_j, S = sum_p w_p omega_i.omega_j
    (paper_rollout.py:178-179)."""
    w = np.broadcast_to(np.asarray(w, dtype=np.float64), U.shape[1:2])
    M = sum((U[a] * w[:, None]).T @ U[a] for a in range(U.shape[0]))
    S = sum((Om[a] * w[:, None]).T @ Om[a] for a in range(Om.shape[0]))
    return 0.5 * (M + M.T), 0.5 * (S + S.T)


# --------------------------------------------------------------------------
# finite part of the pencil (S, M) and the spectral objectives
# --------------------------------------------------------------------------
def finite_pencil(S, M, rank_rtol=1e-10):
    """Finite generalized eigenpairs S v = lam M v, v^T M v = 1, ascending.

    When M has full rank this is ``scipy.linalg.eigh(S, M)`` (the recipe of
    paper_rollout.py:187).  When the K fields span fewer than K dimensions
    (a shared network whose last hidden width is below K), S and M share that
    null space; the finite eigenvalues are those of the pencil restricted to
    range(M), computed through M = Q diag(e) Q^T with the eigenvalues above
    ``rank_rtol * max(e)``.  The reference's rank gate
    (paper_rollout.py:180-186) uses the same eigenvalue-ratio test.
    """
    e, Q = np.linalg.eigh(M)
    keep = e > rank_rtol * e[-1]
    r = int(keep.sum())
    if r == len(M):
        lam, V = sla.eigh(S, M)
        return lam, V, r
    Qr = Q[:, keep] / np.sqrt(e[keep])
    C = Qr.T @ S @ Qr
    lam, Y = np.linalg.eigh(0.5 * (C + C.T))
    return lam, Qr @ Y, r


def objective_weights(kind, r):
    """c_k: 'trace' -> 1 (L = tr(M^-1 S) = sum lam), 'ordering' -> 1/k."""
    if kind == "trace":
        return np.ones(r)
    if kind == "ordering":
        return 1.0 / np.arange(1, r + 1)
    raise ValueError(kind)


def spectral_objective(M, S, kind, rank_rtol=1e-10):
    """L = sum_k c_k lam_k over the finite eigenvalues, and its matrix
    adjoints dL/dS = V diag(c) V^T, dL/dM = -V diag(c lam) V^T.  For
    kind='trace' these are M^-1 and -M^-1 S M^-1 (velocity_trace_jet2.py:
    114-116 up to its 1/k normalisation)."""
    lam, V, r = finite_pencil(S, M, rank_rtol)
    c = objective_weights(kind, r)
    GS = (V * c) @ V.T
    GM = -(V * (c * lam)) @ V.T
    return dict(loss=float(c @ lam), lam=lam, V=V, rank=r, GS=GS, GM=GM)


# --------------------------------------------------------------------------
# field adjoints (transpose of ``fields``)
# --------------------------------------------------------------------------
def fields_adjoint(Ubar, Ombar, dim, n_out):
    """Psi-bar from U-bar, Omega-bar (velocity_trace_jet2.py:102-106 and
    core.py:32-38 for 3D)."""
    C = channels(dim)
    n = Ubar.shape[1]
    Pb = np.zeros((C, n, n_out))
    if dim == 2:
        Pb[2] += Ubar[0]
        Pb[1] -= Ubar[1]
        Pb[3] -= Ombar[0]
        return Pb

    def addg(comp, axis, val):
        Pb[1 + axis][:, comp::3] += val

    def addh(comp, a, b, val):
        Pb[4 + hid(a, b)][:, comp::3] += val

    addg(2, 1, Ubar[0]); addg(1, 2, -Ubar[0])
    addg(0, 2, Ubar[1]); addg(2, 0, -Ubar[1])
    addg(1, 0, Ubar[2]); addg(0, 1, -Ubar[2])
    for a in range(3):
        for b in range(3):
            addh(b, a, b, Ombar[a])
            addh(a, b, b, -Ombar[a])
    return Pb


# --------------------------------------------------------------------------
# one objective + gradient step
# --------------------------------------------------------------------------
@dataclass
class StepResult:
    loss: float
    lam: np.ndarray
    M: np.ndarray
    S: np.ndarray
    rank: int
    grads: list = field(default_factory=list)


def objective_and_grad(params, X0, w, dim, kind, act="tanh", want_grad=True,
                       rank_rtol=1e-10):
    """Direct route: full output layer, U and Omega, K x K Grams, the finite
    pencil, the objective and its parameter gradient."""
    xs, zs, Psi = mlp_forward(params, X0, dim, act)
    U, Om = fields(Psi, dim)
    M, S = grams(U, Om, w)
    obj = spectral_objective(M, S, kind, rank_rtol)
    res = StepResult(obj["loss"], obj["lam"], M, S, obj["rank"])
    if want_grad:
        wv = np.broadcast_to(np.asarray(w, dtype=np.float64), (U.shape[1],))[:, None]
        Ubar = np.stack([2.0 * wv * (U[a] @ obj["GM"]) for a in range(U.shape[0])])
        Obar = np.stack([2.0 * wv * (Om[a] @ obj["GS"]) for a in range(Om.shape[0])])
        Psibar = fields_adjoint(Ubar, Obar, dim, Psi.shape[2])
        res.grads = mlp_backward(params, xs, zs, Psibar, dim, act)
    return res


def hidden_grams_2d(H, w):
    """Grams of the last hidden layer's field channels, 2D scalar potential:
    A_M = sum_p w (h_x h_x^T + h_y h_y^T), A_S = sum_p w h_lap h_lap^T.
    With psi = W_out h + b:  M = W_out A_M W_out^T, S = W_out A_S W_out^T."""
    wv = np.broadcast_to(np.asarray(w, dtype=np.float64), (H.shape[1],))[:, None]
    AM = (H[1] * wv).T @ H[1] + (H[2] * wv).T @ H[2]
    AS = (H[3] * wv).T @ H[3]
    return 0.5 * (AM + AM.T), 0.5 * (AS + AS.T)


def objective_and_grad_factored(params, X0, w, kind, act="tanh", want_grad=True,
                                rank_rtol=1e-10):
    """Factored route for the 2D scalar potential: Grams in the span of the
    last hidden layer.  When K >= H the finite eigenvalues of (S, M) are those
    of (A_S, A_M) (W_out of full column rank) and dL/dW_out = 0; otherwise the
    K x K pencil W A W^T is solved.  Identical results to
    :func:`objective_and_grad` (checked by the tests)."""
    dim = 2
    xs, zs, _ = mlp_forward(params, X0, dim, act)
    H = xs[-1]
    W_out = params[-1][0]
    K, Hn = W_out.shape
    AM, AS = hidden_grams_2d(H, w)
    if K >= Hn:
        obj = spectral_objective(AM, AS, kind, rank_rtol)
        GMh, GSh = obj["GM"], obj["GS"]
        M = W_out @ AM @ W_out.T
        S = W_out @ AS @ W_out.T
        gWout = np.zeros_like(W_out)
    else:
        M = W_out @ AM @ W_out.T
        S = W_out @ AS @ W_out.T
        obj = spectral_objective(M, S, kind, rank_rtol)
        GMh = W_out.T @ obj["GM"] @ W_out
        GSh = W_out.T @ obj["GS"] @ W_out
        gWout = 2.0 * (obj["GM"] @ W_out @ AM + obj["GS"] @ W_out @ AS)
    res = StepResult(obj["loss"], obj["lam"], 0.5 * (M + M.T), 0.5 * (S + S.T), obj["rank"])
    if want_grad:
        wv = np.broadcast_to(np.asarray(w, dtype=np.float64), (H.shape[1],))[:, None]
        Hbar = np.zeros_like(H)
        Hbar[1] = 2.0 * wv * (H[1] @ GMh)
        Hbar[2] = 2.0 * wv * (H[2] @ GMh)
        Hbar[3] = 2.0 * wv * (H[3] @ GSh)
        grads = [None] * len(params)
        grads[-1] = (gWout, np.zeros(K))
        Xbar = Hbar
        for layer in range(len(params) - 2, -1, -1):
            Zbar = act_backward(zs[layer], Xbar, dim, act)
            Xbar, gW, gb = linear_backward(xs[layer], Zbar, params[layer][0])
            grads[layer] = (gW, gb)
        res.grads = grads
    return res


# --------------------------------------------------------------------------
# Adam (native_cupy_core.py:156-171, one shared network: one global norm)
# --------------------------------------------------------------------------
def adam_step(params, moments, grads, step, lr, clip=8.0, beta1=0.9, beta2=0.999,
              eps=1e-8):
    """One Adam transaction.  Raises FloatingPointError and changes nothing
    when the global gradient norm is not finite and positive."""
    flat = [g for pair in grads for g in pair]
    norm = math.sqrt(sum(float(np.sum(np.asarray(g, dtype=np.float64) ** 2)) for g in flat))
    if not (math.isfinite(norm) and norm > 0):
        raise FloatingPointError("Invalid parameter gradients; no optimizer update")
    scale = min(1.0, clip / max(norm, 1e-30))
    t = step + 1
    new_params, new_moments = [], []
    for (W, b), (gW, gb), ((mW, vW), (mb, vb)) in zip(params, grads, moments):
        out = []
        for p, g, m, v in ((W, gW, mW, vW), (b, gb, mb, vb)):
            g = g * scale
            m = beta1 * m + (1 - beta1) * g
            v = beta2 * v + (1 - beta2) * g * g
            p = p - lr * (m / (1 - beta1 ** t)) / (np.sqrt(v / (1 - beta2 ** t)) + eps)
            out.append((p, m, v))
        new_params.append((out[0][0], out[1][0]))
        new_moments.append(((out[0][1], out[0][2]), (out[1][1], out[1][2])))
    return new_params, new_moments, norm


def zero_moments(params):
    return [((np.zeros_like(W), np.zeros_like(W)), (np.zeros_like(b), np.zeros_like(b)))
            for W, b in params]


# --------------------------------------------------------------------------
# quadrature points
# --------------------------------------------------------------------------
def periodic_grid(n, period=2 * math.pi):
    g = np.arange(n) * (period / n)
    X, Y = np.meshgrid(g, g, indexing="ij")
    return np.stack([X.ravel(), Y.ravel()], axis=1), (period / n) ** 2


def periodic_minibatch(count, seed, step, period=2 * math.pi):
    """Points ~ U[0, period)^2 from default_rng((seed, step)); equal weights."""
    rng = np.random.default_rng([seed, step])
    return rng.uniform(0.0, period, (count, 2)), period * period / count


def multihole_points(count, seed, centres=MULTIHOLE_CENTRES, radii=MULTIHOLE_RADII):
    """Seeded rejection sampling of the unit square minus the disks; equal
    weights area / N."""
    rng = np.random.default_rng(seed)
    pieces, remain = [], count
    while remain:
        cand = rng.random((max(2 * remain, 256), 2))
        ok = np.ones(len(cand), bool)
        for (cx, cy), r in zip(centres, radii):
            ok &= (cand[:, 0] - cx) ** 2 + (cand[:, 1] - cy) ** 2 > r * r
        acc = cand[ok][:remain]
        pieces.append(acc)
        remain -= len(acc)
    area = 1.0 - math.pi * float(np.sum(np.asarray(radii) ** 2))
    return np.concatenate(pieces), area / count


def metaball_points(count, seed, n_centres=8, sigma=0.08, level=0.5, chunk=1 << 20):
    """Seeded rejection sampling of {x in [0,1]^3 : sum_i exp(-|x-c_i|^2 /
    (2 sigma^2)) < level}, centres ~ U[0.2, 0.8]^3 drawn first from the same
    generator; equal weights 1/N."""
    rng = np.random.default_rng(seed)
    centres = rng.uniform(0.2, 0.8, (n_centres, 3))
    pieces, remain = [], count
    while remain:
        cand = rng.random((min(max(2 * remain, 256), chunk), 3))
        d2 = ((cand[:, None, :] - centres[None]) ** 2).sum(-1)
        ok = np.exp(-d2 / (2 * sigma * sigma)).sum(1) < level
        acc = cand[ok][:remain]
        pieces.append(acc)
        remain -= len(acc)
    return np.concatenate(pieces), 1.0 / count, centres


# --------------------------------------------------------------------------
# benchmark configurations
# --------------------------------------------------------------------------
CONFIGS = {
    "c1": dict(dim=2, features="periodic", frequencies=16, widths=[64, 128, 128, 128, 64],
               kind="trace"),
    "c2": dict(dim=2, features="periodic", frequencies=16,
               widths=[64, 512, 512, 512, 512, 1024], kind="ordering"),
    "c3": dict(dim=2, features="periodic", frequencies=16,
               widths=[64, 512, 512, 512, 512, 1024], kind="ordering"),
    "c4": dict(dim=2, features="multihole", widths=[5, 256, 256, 256, 256, 1024],
               kind="ordering"),
    "c5": dict(dim=3, features="raw3d", widths=[3, 512, 512, 512, 512, 1536],
               kind="ordering"),
}


def features(kind, points, frequencies=16):
    if kind == "periodic":
        return features_periodic(points, frequencies)
    if kind == "multihole":
        return features_multihole(points)
    if kind == "raw3d":
        return features_raw3d(points)
    raise ValueError(kind)


def scaled_widths(widths, hidden=None, outputs=None):
    """Shrink a configuration's hidden width / output count for small tests."""
    w = list(widths)
    if hidden is not None:
        w = [w[0]] + [hidden] * (len(w) - 2) + [w[-1]]
    if outputs is not None:
        w[-1] = outputs
    return w


# ==========================================================================
# Mode-stacked SIREN networks: the reference's own per-mode architecture
# ==========================================================================
# K independent networks, one per mode, with weights stacked [K, out, in]:
# hidden layers y = sin(omega (W x + b)) (omega_first on layer 0,
# omega_hidden after), a linear output layer, and the output multiplied by an
# envelope jet (native_cupy_core.py:111-154 for first-order jets,
# velocity_trace_jet2.py:26-82 for second-order jets in 3D).  Jets here are
# channel-first arrays [C, n, F]: value, the dim gradient channels, and for
# order 2 the compact Hessian (2D: xx, xy, yy; 3D: xx, xy, xz, yy, yz, zz).
PAIRS_2D = [(0, 0), (0, 1), (1, 1)]


def jet_pairs(dim):
    return PAIRS_2D if dim == 2 else PAIRS


def jet_channels_of(dim, order):
    return 1 + dim + (len(jet_pairs(dim)) if order >= 2 else 0) + (4 if order == 3 else 0)


def sine_jet_forward(Z, dim, order):
    """y = sin z, grad y = cos z grad z, H y = cos z H z - sin z grad z grad z^T
    (velocity_trace_jet2.py:31-34; hardcoded_backend.py sine_forward_jet1);
    order 3 (2D): third derivatives (xxx, xxy, xyy, yyy), the chain rule of
    the reference's Jet3 unary (hardcoded_backend.py:58-152)."""
    s, c = np.sin(Z[0]), np.cos(Z[0])
    Y = np.empty_like(Z)
    Y[0] = s
    for a in range(dim):
        Y[1 + a] = c * Z[1 + a]
    if order >= 2:
        for k, (i, j) in enumerate(jet_pairs(dim)):
            Y[1 + dim + k] = c * Z[1 + dim + k] - s * Z[1 + i] * Z[1 + j]
    if order == 3:
        zx, zy, hxx, hxy, hyy = Z[1], Z[2], Z[3], Z[4], Z[5]
        Y[6] = c * Z[6] - s * 3 * hxx * zx - c * zx ** 3
        Y[7] = c * Z[7] - s * (hxx * zy + 2 * hxy * zx) - c * zx * zx * zy
        Y[8] = c * Z[8] - s * (hyy * zx + 2 * hxy * zy) - c * zx * zy * zy
        Y[9] = c * Z[9] - s * 3 * hyy * zy - c * zy ** 3
    return Y


def sine_jet_backward(Z, A, dim, order):
    """Transpose of :func:`sine_jet_forward` (velocity_trace_jet2.py:35-41,
    sine_backward_jet1 of the analytic-jets backend)."""
    s, c = np.sin(Z[0]), np.cos(Z[0])
    B = np.empty_like(Z)
    zb = c * A[0]
    for a in range(dim):
        zb = zb - s * A[1 + a] * Z[1 + a]
        B[1 + a] = c * A[1 + a]
    if order == 2:
        for k, (i, j) in enumerate(jet_pairs(dim)):
            ah = A[1 + dim + k]
            zb = zb + ah * (-s * Z[1 + dim + k] - c * Z[1 + i] * Z[1 + j])
            B[1 + i] -= s * ah * Z[1 + j]
            B[1 + j] -= s * ah * Z[1 + i]
            B[1 + dim + k] = c * ah
    B[0] = zb
    return B


def envelope_product(E, X, dim, order):
    """Product of the envelope jet E [C, n, 1] with X [C, n, F]
    (native_cupy_core.py product1, velocity_trace_jet2.py product)."""
    Y = np.empty_like(X)
    Y[0] = E[0] * X[0]
    for a in range(dim):
        Y[1 + a] = E[0] * X[1 + a] + E[1 + a] * X[0]
    if order >= 2:
        for k, (i, j) in enumerate(jet_pairs(dim)):
            q = 1 + dim + k
            Y[q] = E[0] * X[q] + E[q] * X[0] + E[1 + i] * X[1 + j] + E[1 + j] * X[1 + i]
    if order == 3:
        # d_ijk (e x) = sum over the subsets S of {i, j, k} of d_S e d_(rest) x
        for q, idx in zip(range(6, 10), ((0, 0, 0), (0, 0, 1), (0, 1, 1), (1, 1, 1))):
            acc = 0.0
            for mask in range(8):
                left = tuple(idx[t] for t in range(3) if mask >> t & 1)
                right = tuple(idx[t] for t in range(3) if not mask >> t & 1)
                acc = acc + E[_jet3_slot(left)] * X[_jet3_slot(right)]
            Y[q] = acc
    return Y


def _jet3_slot(multi):
    """Channel of the 2D derivative d_multi in a third-order jet."""
    m = tuple(sorted(multi))
    return {(): 0, (0,): 1, (1,): 2, (0, 0): 3, (0, 1): 4, (1, 1): 5, (0, 0, 0): 6,
            (0, 0, 1): 7, (0, 1, 1): 8, (1, 1, 1): 9}[m]


def envelope_product_backward(E, A, dim, order):
    """Adjoint of X in :func:`envelope_product` (envelope_product_backward_jet1,
    velocity_trace_jet2.py product_reverse)."""
    B = np.empty_like(A)
    xb = E[0] * A[0]
    for a in range(dim):
        xb = xb + E[1 + a] * A[1 + a]
        B[1 + a] = E[0] * A[1 + a]
    if order == 2:
        for k, (i, j) in enumerate(jet_pairs(dim)):
            q = 1 + dim + k
            xb = xb + E[q] * A[q]
            B[1 + i] += E[1 + j] * A[q]
            B[1 + j] += E[1 + i] * A[q]
            B[q] = E[0] * A[q]
    B[0] = xb
    return B


def mode_omegas(n_layers, omega_first, omega_hidden):
    """omega of every hidden layer (the output layer has none)."""
    return [omega_first if j == 0 else omega_hidden for j in range(n_layers - 1)]


def mode_forward(W, b, X0, E, dim, order, omegas):
    """One mode: W, b lists of [out, in], [out]; X0 the shared feature jet.
    Returns (layer inputs, scaled pre-activations, envelope * output)."""
    X, xs, pres = X0, [], []
    for j in range(len(W) - 1):
        xs.append(X)
        P = omegas[j] * linear_forward(X, W[j], b[j])
        pres.append(P)
        X = sine_jet_forward(P, dim, order)
    xs.append(X)
    raw = linear_forward(X, W[-1], b[-1])
    return xs, pres, envelope_product(E, raw, dim, order)


def mode_backward(W, xs, pres, E, A, dim, order, omegas):
    """Hand-written reverse of :func:`mode_forward` for one mode
    (native_cupy_core.py:142-154, velocity_trace_jet2.py:77-82)."""
    a = envelope_product_backward(E, A, dim, order)
    gW, gb = [None] * len(W), [None] * len(W)
    a, gW[-1], gb[-1] = linear_backward(xs[-1], a, W[-1])
    for j in range(len(W) - 2, -1, -1):
        a = omegas[j] * sine_jet_backward(pres[j], a, dim, order)
        a, gW[j], gb[j] = linear_backward(xs[j], a, W[j])
    return gW, gb


def mode_adam(W, b, mW, vW, mb, vb, gW, gb, epoch, lr, clip=8.0):
    """Per-mode Adam (native_cupy_core.py:156-171): the clip norm of mode k
    runs over that mode's slice of every tensor; any non-finite or zero norm
    raises with nothing changed.  Arrays are stacked [K, ...].  Returns the
    new (W, b, mW, vW, mb, vb, epoch) and the per-mode norms."""
    K = W[0].shape[0]
    norms = np.sqrt(sum(np.sum(np.asarray(g, dtype=np.float64).reshape(K, -1) ** 2, axis=1)
                        for g in [*gW, *gb]))
    if not np.all(np.isfinite(norms) & (norms > 0)):
        raise FloatingPointError("Invalid parameter gradients; no optimizer update")
    scales = np.minimum(1.0, clip / np.maximum(norms, 1e-30))
    t = epoch + 1
    out = []
    for pars, ms, vs, gs in ((W, mW, vW, gW), (b, mb, vb, gb)):
        np_, nm, nv = [], [], []
        for p, m, v, g in zip(pars, ms, vs, gs):
            g = g * scales.reshape((K,) + (1,) * (g.ndim - 1))
            m = 0.9 * m + 0.1 * g
            v = 0.999 * v + 0.001 * g * g
            np_.append(p - lr * (m / (1 - 0.9 ** t)) / (np.sqrt(v / (1 - 0.999 ** t)) + 1e-8))
            nm.append(m)
            nv.append(v)
        out.append((np_, nm, nv))
    (W2, mW2, vW2), (b2, mb2, vb2) = out
    return (W2, b2, mW2, vW2, mb2, vb2, t), norms


def velocity_fields(out):
    """Velocity u = curl A and its gradient D[a][j] = d_j u_a of a 3D
    vector potential jet out [10, n, 3] (velocity_trace_jet2.py:93-101):
    returns U [n, 3], D [n, 3, 3]."""
    def g(comp, axis):
        return out[1 + axis][:, comp]

    def h(comp, a, b):
        return out[4 + hid(a, b)][:, comp]

    U = np.stack([g(2, 1) - g(1, 2), g(0, 2) - g(2, 0), g(1, 0) - g(0, 1)], -1)
    D = np.stack([np.stack([h((a + 2) % 3, j, (a + 1) % 3) - h((a + 1) % 3, j, (a + 2) % 3)
                            for j in range(3)], -1) for a in range(3)], -2)
    return U, D


def velocity_lift(GU, GD):
    """Adjoint of :func:`velocity_fields`: GU [n, 3], GD [n, 3, 3] -> output
    jet adjoint [10, n, 3] (core.py:32-38 lift)."""
    n = GU.shape[0]
    A = np.zeros((10, n, 3))
    A[1 + 1][:, 2] += GU[:, 0]; A[1 + 2][:, 1] -= GU[:, 0]
    A[1 + 2][:, 0] += GU[:, 1]; A[1 + 0][:, 2] -= GU[:, 1]
    A[1 + 0][:, 1] += GU[:, 2]; A[1 + 1][:, 0] -= GU[:, 2]
    for a in range(3):
        for j in range(3):
            A[4 + hid(j, (a + 1) % 3)][:, (a + 2) % 3] += GD[:, a, j]
            A[4 + hid(j, (a + 2) % 3)][:, (a + 1) % 3] -= GD[:, a, j]
    return A


def coefficient_peel(M, S, sort=True):
    """Causal Rayleigh peel in Gram form (core.py:48-69): modes sorted by
    their raw quotients S_kk / M_kk (stable; with ``sort`` False the network
    order, the 2D peel's fixed_order, hardcoded_backend.py:3471-3475), the
    sorted mass matrix
    orthonormalised by a scaled Cholesky factor applied twice (the Gram form
    of two-pass modified Gram-Schmidt), losses = diag(T^T S T).  Returns the
    losses in causal order, the order, the transform T (rows in mode order),
    and the coefficient adjoints Cu, Cd with dL/dU = U Cu / n and
    dL/dD = D Cd / n for L = sum(losses).  Raises FloatingPointError where
    the reference's rank / relative-mass / orthogonality gate fails."""
    K = len(M)
    raw = np.diag(S) / np.diag(M)
    order = np.argsort(raw, kind="stable") if sort else np.arange(K)
    ms = M[np.ix_(order, order)]
    ss = S[np.ix_(order, order)]
    scale = np.sqrt(np.diag(ms))
    L = np.linalg.cholesky(ms / scale[:, None] / scale[None, :])
    T = sla.solve_triangular(L.T, np.eye(K), lower=False) / scale[:, None]
    H2 = T.T @ ms @ T
    L2 = np.linalg.cholesky(0.5 * (H2 + H2.T))
    T = T @ sla.solve_triangular(L2.T, np.eye(K), lower=False)
    error = float(np.max(np.abs(T.T @ ms @ T - np.eye(K))))
    norm = 1.0 / np.diag(T)
    relative = norm * norm / np.diag(ms)
    F = T.T @ ss @ T
    loss = np.diag(F).copy()
    if not (np.all(np.isfinite(loss) & (loss > 0) & (relative >= 1e-4)) and error <= 1e-5):
        raise FloatingPointError("Velocity rank/relative mass/orthogonality gate failed")
    C = -2.0 * (T * loss[None, :] + T @ np.triu(F, 1)) / norm[None, :]
    B = 2.0 * T / norm[None, :]
    Cu = np.empty_like(C); Cd = np.empty_like(B); Tm = np.empty_like(T)
    Cu[np.ix_(order, order)] = C
    Cd[np.ix_(order, order)] = B
    Tm[order] = T
    return dict(losses=loss, order=order, T=Tm, Cu=Cu, Cd=Cd, relative_mass=relative,
                gram_max=error, raw=raw)


def velocity_step(W, b, X0, E, omegas, want_grad=True):
    """The 3D velocity objective of the mode-stacked network (core.py:79-103):
    every mode's vector potential (3 outputs, second-order jets), U [3n, K]
    and D [9n, K], M = U^T U / n, S = D^T D / n, the Gram-form peel, and the
    parameter gradient of sum(losses).  W, b: lists of stacked [K, out, in],
    [K, out] arrays."""
    K = W[0].shape[0]
    n = X0.shape[1]
    per, Us, Ds = [], [], []
    for k in range(K):
        Wk = [w[k] for w in W]
        bk = [x[k] for x in b]
        xs, pres, out = mode_forward(Wk, bk, X0, E, 3, 2, omegas)
        u, d = velocity_fields(out)
        per.append((Wk, xs, pres))
        Us.append(u.reshape(-1))
        Ds.append(d.reshape(-1))
    U = np.stack(Us, 1)
    D = np.stack(Ds, 1)
    M = U.T @ U / n
    S = D.T @ D / n
    obj = coefficient_peel(M, S)
    obj.update(M=M, S=S, U=U, D=D)
    if want_grad:
        gu = U @ obj["Cu"] / n
        gd = D @ obj["Cd"] / n
        gW = [np.zeros_like(w) for w in W]
        gb = [np.zeros_like(x) for x in b]
        for k, (Wk, xs, pres) in enumerate(per):
            A = velocity_lift(gu[:, k].reshape(n, 3), gd[:, k].reshape(n, 3, 3))
            gwk, gbk = mode_backward(Wk, xs, pres, E, A, 3, 2, omegas)
            for j in range(len(W)):
                gW[j][k] = gwk[j]
                gb[j][k] = gbk[j]
        obj["grads"] = (gW, gb)
    return obj


def potential_peel_step(W, b, X0, weight, omegas, lr=None, clip=8.0, moments=None, epoch=0,
                        sort=True):
    """The periodic 2D streamfunction Rayleigh peel (hardcoded_backend.py:
    3383-3771) on the mode-stacked network with first-order jets and the
    identity envelope: raw values (mean removed, the constant gauge) and
    gradients of every mode, M = w V^T V, S = w G^T G (w = area / n), the
    Gram-form causal peel, the gradient of sum(losses) (detached prefix) and,
    when ``lr`` is given, the all-mode Adam transaction.  X0: [3, n, F]
    feature jet.  Returns the peel dict with ``loss`` = mean of the peeled
    quotients and ``grads``; with ``lr`` also ``state`` (mode_adam's)."""
    K = W[0].shape[0]
    n = X0.shape[1]
    E = np.zeros((3, n, 1))
    E[0] = 1.0
    per, vals, grads = [], [], []
    for k in range(K):
        Wk = [w[k] for w in W]
        bk = [x[k] for x in b]
        xs, pres, out = mode_forward(Wk, bk, X0, E, 2, 1, omegas)
        per.append((Wk, xs, pres))
        vals.append(out[0][:, 0])
        grads.append(np.stack([out[1][:, 0], out[2][:, 0]], -1).reshape(-1))
    V = np.stack(vals, 1)
    V = V - V.mean(axis=0, keepdims=True)
    G = np.stack(grads, 1)
    M = weight * V.T @ V
    S = weight * G.T @ G
    obj = coefficient_peel(M, S, sort)
    obj.update(M=M, S=S, loss=float(np.mean(obj["losses"])))
    dV = weight * V @ obj["Cu"]
    dG = weight * G @ obj["Cd"]
    dV = dV - dV.mean(axis=0, keepdims=True)
    gW = [np.zeros_like(w) for w in W]
    gb = [np.zeros_like(x) for x in b]
    for k, (Wk, xs, pres) in enumerate(per):
        A = np.zeros((3, n, 1))
        A[0, :, 0] = dV[:, k]
        A[1, :, 0] = dG[0::2, k]
        A[2, :, 0] = dG[1::2, k]
        gwk, gbk = mode_backward(Wk, xs, pres, E, A, 2, 1, omegas)
        for j in range(len(W)):
            gW[j][k] = gwk[j]
            gb[j][k] = gbk[j]
    obj["grads"] = (gW, gb)
    if lr is not None:
        if moments is None:
            moments = ([np.zeros_like(w) for w in W], [np.zeros_like(w) for w in W],
                       [np.zeros_like(x) for x in b], [np.zeros_like(x) for x in b])
        mW, vW, mb, vb = moments
        obj["state"], obj["norms"] = mode_adam(W, b, mW, vW, mb, vb, gW, gb, epoch, lr, clip)
    return obj


# --------------------------------------------------------------------------
# periodic evaluation: Jet3 fields, Ritz basis, ETDRK4 Galerkin rollout
# --------------------------------------------------------------------------
def features_periodic_jet(points, frequencies, order, length=2 * math.pi):
    """Fourier feature jets of order 1, 2 or 3, [C, n, 4F] with channels
    (value, x, y[, xx, xy, yy[, xxx, xxy, xyy, yyy]]) (hardcoded_backend.py:
    418-438 and its Jet3 encoding): sin, cos of 2 pi h s / L, s = x then y."""
    points = np.asarray(points, dtype=np.float64)
    n = len(points)
    C = jet_channels_of(2, order)
    out = np.zeros((C, n, 4 * frequencies))
    col = 0
    for axis in range(2):
        s = points[:, axis]
        for h in range(1, frequencies + 1):
            k = 2.0 * math.pi * h / length
            for fn, d1 in ((np.sin(k * s), k * np.cos(k * s)), (np.cos(k * s), -k * np.sin(k * s))):
                out[0, :, col] = fn
                out[1 + axis, :, col] = d1
                if order >= 2:
                    out[3 if axis == 0 else 5, :, col] = -k * k * fn
                if order == 3:
                    out[6 if axis == 0 else 9, :, col] = -k * k * d1
                col += 1
    return out


def stream_fields(out):
    """The six channels of evaluate_large_comparison.py:29-35 from a mode's
    third-order output jet [10, n, 1]: psi, u = psi_y, v = -psi_x,
    omega = -lap psi, -lap u, -lap v."""
    o = out[:, :, 0]
    return np.stack([o[0], o[2], -o[1], -(o[3] + o[5]), -(o[7] + o[9]), o[6] + o[8]])


def ritz_basis(gu, gv, gw, weight, rank_rtol=1e-12):
    """Normalisation and Ritz stage of paper_rollout.py:171-192: columns
    scaled to unit velocity norm, M = w (gu^T gu + gv^T gv), S = w gw^T gw,
    the full-rank gate on eig(M) (rank = #(e > rtol e_max)), eigh(S, M).
    Returns (vals, R, norm) with R = D^-1 T mapping Ritz coefficients to
    coefficients of the raw fields."""
    norm = np.sqrt(weight * np.sum(gu * gu + gv * gv, axis=0))
    if not np.all(norm > 0):
        raise ArithmeticError("a mode with zero velocity")
    U, V, W = gu / norm, gv / norm, gw / norm
    mass = weight * (U.T @ U + V.T @ V)
    stiff = weight * (W.T @ W)
    mh, sh = (mass + mass.T) / 2, (stiff + stiff.T) / 2
    ev = np.linalg.eigvalsh(mh)
    rank = int(np.sum(ev > ev[-1] * rank_rtol))
    if rank != len(mh):
        raise ArithmeticError("Full-K rank gate")
    vals, T = sla.eigh(sh, mh)
    return vals, T / norm[:, None], norm


def etdrk4_weights(lam, nu, h):
    """(e, e2, q, f1, f2, f3) of paper_rollout.py:56-64."""
    linear = -nu * lam
    e = np.exp(h * linear)
    e2 = np.exp(0.5 * h * linear)
    roots = np.exp(1j * np.pi * (np.arange(1, 33) - 0.5) / 32)
    lr = h * linear[:, None] + roots
    q = h * np.real(np.mean((np.exp(lr / 2) - 1) / lr, axis=-1))
    f1 = h * np.real(np.mean((-4 - lr + np.exp(lr) * (4 - 3 * lr + lr * lr)) / lr ** 3, axis=-1))
    f2 = h * np.real(np.mean((2 + lr + np.exp(lr) * (-2 + lr)) / lr ** 3, axis=-1))
    f3 = h * np.real(np.mean((-4 - 3 * lr - lr * lr + np.exp(lr) * (4 - lr)) / lr ** 3, axis=-1))
    return e, e2, q, f1, f2, f3


def galerkin_rhs(gu, gv, gw, weight, a):
    """rhs(a) = gu^T (w omega v) - gv^T (w omega u), (u, v, omega) = g a
    (paper_rollout.py:37-41)."""
    u, v, w = gu @ a, gv @ a, gw @ a
    return gu.T @ (weight * w * v) - gv.T @ (weight * w * u)


def etdrk4_rollout(gu, gv, gw, lam, nu, c0, times, dt, weight):
    """The autonomous ETDRK4 rollout of paper_rollout.py:31-79 in the (Ritz)
    basis gu, gv, gw: for every target time, ceil((t - t_prev) / dt) equal
    steps; returns the coefficient states [frames, K]."""
    c = np.asarray(c0, dtype=np.float64).copy()
    current = 0.0
    states = []
    for target in times:
        steps = max(0, int(np.ceil((target - current) / dt - 1e-10)))
        if steps:
            h = (target - current) / steps
            e, e2, q, f1, f2, f3 = etdrk4_weights(lam, nu, h)
            rhs = lambda x: galerkin_rhs(gu, gv, gw, weight, x)  # noqa: E731
            for _ in range(steps):
                nv = rhs(c)
                a = e2 * c + q * nv
                na = rhs(a)
                b = e2 * c + q * na
                nb = rhs(b)
                z = e2 * a + q * (2 * nb - nv)
                c = e * c + f1 * nv + 2 * f2 * (na + nb) + f3 * rhs(z)
        current = target
        states.append(c.copy())
    return np.array(states)
