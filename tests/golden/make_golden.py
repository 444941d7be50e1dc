"""Generate the golden fixtures that pin the oracle to the reference.

Runs the reference's own (CuPy) functions on the CPU by installing a NumPy
stand-in for ``cupy`` / ``cupyx`` (the pattern of the reference's
tests/test_finite_gauge.py:10-16) and records small seeded input/output
vectors in ``tests/golden/reference_vectors.npz``.  It needs the reference
checkout named by ``$NEB_REFERENCE`` (required), which exists only
where the fixtures are made; the tests read the committed ``.npz`` alone.

Reference functions exercised (paths relative to the reference project):

* experiments/2d/_backend/periodic_core/vortex_merger/src/eigenfluid/gen/
  vortex_merger2d/hardcoded_backend.py: ``unary2`` (:252), ``xy_jets2`` (:496),
  ``encoding_jet2`` periodic branch (:576), ``linear_forward_batch_jet2``
  (:1005), ``linear_backward_batch_jet2`` (:1115), ``unary_backward_jet2`` (:1147);
* experiments/metaball/_backend/flow/cases/metaball/velocity_trace_jet2.py:
  ``sine`` (:31), ``sine_reverse`` (:35), ``velocity`` (:93), ``vorticity`` (:96),
  ``lift_reverse`` (:102), ``trace_objective`` (:107);
* experiments/metaball/_backend/flow/cases/metaball/velocity/core.py: ``grams`` (:40),
  ``coefficient_peel`` (:48), ``lift`` (:32), composed as ``compute`` (:79) composes them;
* experiments/metaball/_backend/flow/cases/metaball/native_cupy_core.py:
  ``Model`` forward / backward / adam (:111-171), with one mode and the
  identity envelope, and with two modes and a random envelope;
* experiments/metaball/_backend/flow/cases/metaball/velocity_trace_jet2.py:
  ``forward`` / ``backward`` (:65-82) of a four-mode second-order network;
* experiments/periodic/paper_rollout.py:178-187 recipe (Grams, then
  ``scipy.linalg.eigh(S, M)``);
* hardcoded_backend.py ``HardcodedModel`` (:1705) ``forward_stream_jet1``
  (:1716), ``forward_stream`` (third-order jets, :1882), ``arrays`` (:1987)
  and ``peel_step`` (:3774) with the streamfunction Rayleigh peel (:3383) on
  a four-mode periodic network;
* experiments/2d/_backend/flow/cases/vortex_merger/neural_training/
  prepare_gauge_canonical.py ``main`` (the trainer's epoch-0 arrays and its
  fixed validation points);
* experiments/periodic/paper_rollout.py ``rollout`` (:31), the autonomous
  ETDRK4 Galerkin rollout, on a six-mode basis of the 128^2 grid.

Usage:  NEB_REFERENCE=<reference checkout> python tests/golden/make_golden.py
"""
from __future__ import annotations

import importlib.util
import math
import os
import sys
import types
from pathlib import Path
from types import SimpleNamespace

import numpy as np
import scipy.linalg as sla

def reference_root() -> Path:
    """The reference checkout, named by $NEB_REFERENCE (required)."""
    root = os.environ.get("NEB_REFERENCE")
    if not root:
        raise SystemExit("set NEB_REFERENCE to the reference checkout (baiming-zhang/NEB)")
    return Path(root)
OUT = Path(__file__).resolve().parent / "reference_vectors.npz"


class _NumpyCupy(types.ModuleType):
    """Module that answers every ``cupy`` attribute from NumPy."""

    def __init__(self):
        super().__init__("cupy")
        self.cuda = SimpleNamespace(
            Stream=SimpleNamespace(null=SimpleNamespace(synchronize=lambda: None)))
        self.linalg = np.linalg

    def __getattr__(self, name):
        return getattr(np, name)

    @staticmethod
    def asnumpy(a):
        return np.asarray(a)

    @staticmethod
    def get_default_memory_pool():
        return SimpleNamespace(free_all_blocks=lambda: None, set_limit=lambda **k: None)


def install_shim():
    cp = _NumpyCupy()
    sys.modules["cupy"] = cp
    cupyx = types.ModuleType("cupyx")
    cupyx_scipy = types.ModuleType("cupyx.scipy")
    cupyx_linalg = types.ModuleType("cupyx.scipy.linalg")
    cupyx_linalg.solve_triangular = sla.solve_triangular
    cupyx.scipy = cupyx_scipy
    cupyx_scipy.linalg = cupyx_linalg
    sys.modules["cupyx"] = cupyx
    sys.modules["cupyx.scipy"] = cupyx_scipy
    sys.modules["cupyx.scipy.linalg"] = cupyx_linalg
    return cp


ROLLOUT_WAVES = ((1, 0), (0, 1), (1, 1), (2, 1))


def rollout_basis(coef, n):
    """Smooth periodic (u, v, omega) fields of len(coef) modes on the n x n
    grid, [3, n^2, K]: field f of mode k is sum over the wave vectors (m1, m2)
    of coef[k, t, f, 0] cos(m1 x + m2 y + coef[k, t, f, 1]) (the same
    construction as tests/test_rollout_host.py)."""
    axis = np.arange(n) * 2 * math.pi / n
    xg, yg = np.meshgrid(axis, axis)
    basis = np.zeros((3, n * n, len(coef)))
    for k in range(len(coef)):
        for t, (m1, m2) in enumerate(ROLLOUT_WAVES):
            for f in range(3):
                amp, phase = coef[k, t, f]
                basis[f, :, k] += (amp * np.cos(m1 * xg + m2 * yg + phase)).ravel()
    return basis


def load(path, name):
    spec = importlib.util.spec_from_file_location(name, path)
    module = importlib.util.module_from_spec(spec)
    sys.modules[name] = module
    spec.loader.exec_module(module)
    return module


def main():
    install_shim()
    hb_src = reference_root() / "experiments/2d/_backend/periodic_core/vortex_merger/src"
    sys.path.insert(0, str(hb_src))
    from eigenfluid.gen.vortex_merger2d import hardcoded_backend as HB
    HB.F32 = np.float64  # run the reference's FP32-typed GEMMs in FP64
    vendor = reference_root() / "experiments/metaball/_backend"
    metaball = vendor / "flow/cases/metaball"
    sys.path[:0] = [str(vendor), str(metaball)]
    ncc = load(metaball / "native_cupy_core.py", "native_cupy_core")
    ncc.old.F32 = np.float64  # the analytic_jets transposes NCC calls
    vtj2 = load(metaball / "velocity_trace_jet2.py", "velocity_trace_jet2")
    vcore = load(metaball / "velocity/core.py", "velocity_core")

    rng = np.random.default_rng(20261203)
    g = {}

    # --- 2D tanh jet chain rule and its transpose (unary2 / unary_backward_jet2)
    n, f = 9, 6
    z = rng.normal(size=(n, f))
    grad = rng.normal(size=(n, f, 2))
    hess = rng.normal(size=(n, f, 3))
    t = np.tanh(z); s1 = 1 - t * t; s2 = -2 * t * s1; s3 = -2 * s1 * (s1 - 2 * t * t)
    y = HB.unary2(HB.Jet2(z, grad, hess), t, s1, s2)
    g.update(act2d_z=z, act2d_grad=grad, act2d_hess=hess,
             act2d_y=y.value, act2d_ygrad=y.grad, act2d_yhess=y.hess)
    av, ag, al = rng.normal(size=(n, f)), rng.normal(size=(n, f, 2)), rng.normal(size=(n, f))
    adj = HB.Jet2(av, ag, np.stack([al, np.zeros_like(al), al], -1))
    back = HB.unary_backward_jet2(HB.Jet2(z, grad, hess), adj, s1, s2, s3)
    g.update(act2d_av=av, act2d_ag=ag, act2d_al=al,
             act2d_zb=back.value, act2d_gb=back.grad, act2d_hb=back.hess)

    # --- 2D linear jet layer and its transpose (shared source, one mode)
    n, fi, fo = 7, 5, 4
    src = HB.Jet2(rng.normal(size=(n, fi)), rng.normal(size=(n, fi, 2)), rng.normal(size=(n, fi, 3)))
    W = rng.normal(size=(1, fo, fi)); b = rng.normal(size=(1, fo))
    out = HB.linear_forward_batch_jet2(src, W, b, np.float64)
    ad = HB.Jet2(rng.normal(size=(1, n, fo)), rng.normal(size=(1, n, fo, 2)), rng.normal(size=(1, n, fo, 3)))
    xb, gW, gb = HB.linear_backward_batch_jet2(src, ad, W)
    g.update(lin_x=src.value, lin_xg=src.grad, lin_xh=src.hess, lin_W=W[0], lin_b=b[0],
             lin_z=out.value[0], lin_zg=out.grad[0], lin_zh=out.hess[0],
             lin_av=ad.value[0], lin_ag=ad.grad[0], lin_ah=ad.hess[0],
             lin_xbv=xb.value[0], lin_xbg=xb.grad[0], lin_xbh=xb.hess[0], lin_gW=gW[0], lin_gb=gb[0])

    # --- periodic Fourier encoding with second-order jets
    cfg = SimpleNamespace(input_encoding="periodic_sincos_xy", xmin=0.0, xmax=2 * math.pi,
                          ymin=0.0, ymax=2 * math.pi, frequencies=5)
    pts = rng.uniform(0, 2 * math.pi, size=(11, 2))
    x, yj = HB.xy_jets2(pts, np.float64)
    enc = HB.encoding_jet2(cfg, x, yj, 0.0, 0.0)
    g.update(enc_points=pts, enc_value=enc.value, enc_grad=enc.grad, enc_hess=enc.hess,
             enc_frequencies=np.asarray(5))

    # --- 3D compact Jet2 sine chain rule and transpose
    n, f = 6, 4
    z3 = rng.normal(size=(n, f)); g3 = rng.normal(size=(n, f, 3)); h3 = rng.normal(size=(n, f, 6))
    y3 = vtj2.sine(vtj2.J2(z3, g3, h3))
    a3 = vtj2.J2(rng.normal(size=(n, f)), rng.normal(size=(n, f, 3)), rng.normal(size=(n, f, 6)))
    b3 = vtj2.sine_reverse(vtj2.J2(z3, g3, h3), a3)
    g.update(act3d_z=z3, act3d_grad=g3, act3d_hess=h3, act3d_y=y3.value, act3d_ygrad=y3.grad,
             act3d_yhess=y3.hess, act3d_av=a3.value, act3d_ag=a3.grad, act3d_ah=a3.hess,
             act3d_zb=b3.value, act3d_gb=b3.grad, act3d_hb=b3.hess)

    # --- 3D fields (curl, curl curl) and their transpose
    k, n = 3, 5
    fj = vtj2.J2(rng.normal(size=(k, n, 3)), rng.normal(size=(k, n, 3, 3)), rng.normal(size=(k, n, 3, 6)))
    gu, gw = rng.normal(size=(k, n, 3)), rng.normal(size=(k, n, 3))
    lifted = vtj2.lift_reverse(gu, gw)
    g.update(f3_value=fj.value, f3_grad=fj.grad, f3_hess=fj.hess, f3_u=vtj2.velocity(fj),
             f3_w=vtj2.vorticity(fj), f3_gu=gu, f3_gw=gw, f3_lift_grad=lifted.grad,
             f3_lift_hess=lifted.hess)

    # --- Grams (core.py:40-46) and the eigen recipe (paper_rollout.py:178-187)
    n, k = 40, 6
    U = rng.normal(size=(3 * n, k)); D = rng.normal(size=(3 * n, k))
    M, S = vcore.grams(U, D)
    lam, V = sla.eigh(S, M)
    g.update(gram_U=U, gram_D=D, gram_M=M, gram_S=S, eig_lam=lam, eig_V=V)

    # --- trace objective with adjoints (velocity_trace_jet2.py:107-117)
    tr = vtj2.trace_objective(U, D, adjoints=True)
    g.update(trace_loss=np.asarray(float(tr["loss"])), trace_GU=tr["GU"], trace_GO=tr["GO"])

    # --- the reference's own network-backend Model: forward, reverse, Adam
    c = SimpleNamespace(hidden=8, hidden_layers=2, siren_first_omega0=2.3, siren_hidden_omega0=1.7)
    model = ncc.Model(c, K=1, seed=31)
    n = 5
    feat = rng.normal(size=(n, 15)); fgrad = rng.normal(size=(n, 15, 3))
    env = ncc.Jet1(np.ones((n, 1)), np.zeros((n, 1, 3)))
    data = SimpleNamespace(features=ncc.Jet1(feat, fgrad), envelope=env)
    W0 = [w.copy() for w in model.W]; b0 = [bb.copy() for bb in model.b]
    val, tape = model.forward(data, 0, 1, True)
    av = rng.normal(size=val.value.shape); agr = rng.normal(size=val.grad.shape)
    gw, gbias = model.backward(data, 0, 1, tape, ncc.Jet1(av, agr))
    model.adam(gw, gbias, 1e-3, clip=0.5)
    model.adam([2 * x for x in gw], [-x for x in gbias], 1e-3, clip=0.5)
    for j in range(len(W0)):
        g[f"ncc_W{j}"] = W0[j][0]; g[f"ncc_b{j}"] = b0[j][0]
        g[f"ncc_gW{j}"] = gw[j][0]; g[f"ncc_gb{j}"] = gbias[j][0]
        g[f"ncc_W{j}_after"] = model.W[j][0]; g[f"ncc_b{j}_after"] = model.b[j][0]
        g[f"ncc_mW{j}"] = model.mW[j][0]; g[f"ncc_vW{j}"] = model.vW[j][0]
    g.update(ncc_feat=feat, ncc_fgrad=fgrad, ncc_value=val.value[0], ncc_grad=val.grad[0],
             ncc_av=av[0], ncc_ag=agr[0], ncc_omega=np.asarray([2.3, 1.7]),
             ncc_layers=np.asarray(len(W0)))
    # --- the per-mode network with a non-trivial envelope (the shape of the
    # reference's backend test, tests/test_network_backends.py:37-98): two
    # modes, first-order jets, two Adam steps
    model = ncc.Model(c, K=2, seed=31)
    n = 5
    feat = rng.normal(size=(n, 15)); fgrad = rng.normal(size=(n, 15, 3))
    env_v = rng.uniform(.3, .8, size=(n, 1)); env_g = rng.normal(size=(n, 1, 3))
    data = SimpleNamespace(features=ncc.Jet1(feat, fgrad), envelope=ncc.Jet1(env_v, env_g))
    W0 = [w.copy() for w in model.W]; b0 = [bb.copy() for bb in model.b]
    val, tape = model.forward(data, 0, 2, True)
    av = rng.normal(size=val.value.shape); agr = rng.normal(size=val.grad.shape)
    gw, gbias = model.backward(data, 0, 2, tape, ncc.Jet1(av, agr))
    norms1 = model.adam(gw, gbias, 1e-3, clip=0.5)
    norms2 = model.adam([2 * x for x in gw], [-x for x in gbias], 1e-3, clip=0.5)
    for j in range(len(W0)):
        g[f"env_W{j}"] = W0[j]; g[f"env_b{j}"] = b0[j]
        g[f"env_gW{j}"] = gw[j]; g[f"env_gb{j}"] = gbias[j]
        g[f"env_W{j}_after"] = model.W[j]; g[f"env_b{j}_after"] = model.b[j]
    g.update(env_feat=feat, env_fgrad=fgrad, env_ev=env_v, env_eg=env_g, env_value=val.value,
             env_grad=val.grad, env_av=av, env_ag=agr, env_norms1=norms1, env_norms2=norms2)

    # --- 3D second-order per-mode network with envelope, velocity fields,
    # Grams, the Gram-form causal peel and the gradient, composed from the
    # reference's own functions as velocity/core.py:79-103 composes them
    K3, n3 = 4, 7
    c3 = SimpleNamespace(hidden=6, hidden_layers=2, siren_first_omega0=1.9,
                         siren_hidden_omega0=1.3)
    m3 = ncc.Model(c3, K=K3, seed=5)
    f3 = vtj2.J2(rng.normal(size=(n3, 15)) * 0.5, rng.normal(size=(n3, 15, 3)) * 0.5,
                 rng.normal(size=(n3, 15, 6)) * 0.5)
    e3 = vtj2.J2(rng.uniform(.3, .8, size=(n3, 1)), rng.normal(size=(n3, 1, 3)) * 0.3,
                 rng.normal(size=(n3, 1, 6)) * 0.3)
    d3 = SimpleNamespace(features=f3, envelope=e3, n=n3)
    out3, hist3 = vtj2.forward(m3, d3, 0, K3, True)
    U3 = vtj2.velocity(out3).reshape(K3, -1).T
    D3 = vtj2.velocity_grad(out3).reshape(K3, -1).T
    M3, S3 = vcore.grams(U3, D3)
    pk = vcore.coefficient_peel(M3, S3)
    gu3 = (U3 @ pk["Cu"] / n3).T.reshape(K3, n3, 3)
    gd3 = (D3 @ pk["Cd"] / n3).T.reshape(K3, n3, 3, 3)
    gw3, gb3 = vtj2.backward(m3, d3, hist3, vcore.lift(gu3, gd3))
    for j in range(len(m3.W)):
        g[f"vel_W{j}"] = m3.W[j]; g[f"vel_b{j}"] = m3.b[j]
        g[f"vel_gW{j}"] = gw3[j]; g[f"vel_gb{j}"] = gb3[j]
    g.update(vel_fv=f3.value, vel_fg=f3.grad, vel_fh=f3.hess, vel_ev=e3.value, vel_eg=e3.grad,
             vel_eh=e3.hess, vel_out_v=out3.value, vel_out_g=out3.grad, vel_out_h=out3.hess,
             vel_U=U3, vel_D=D3, vel_M=M3, vel_S=S3, vel_losses=pk["losses"],
             vel_order=pk["order"], vel_T=pk["T"], vel_Cu=pk["Cu"], vel_Cd=pk["Cd"],
             vel_omega=np.asarray([1.9, 1.3]), vel_layers=np.asarray(len(m3.W)))

    # --- the Gram-form peel alone on a larger, well-conditioned pencil
    Kp = 12
    X = rng.normal(size=(60, Kp)); Y = rng.normal(size=(60, Kp)) * np.linspace(0.5, 3, Kp)
    Mp, Sp = X.T @ X / 20, Y.T @ Y / 20
    pp = vcore.coefficient_peel(Mp, Sp)
    g.update(peel_M=Mp, peel_S=Sp, peel_losses=pp["losses"], peel_order=pp["order"],
             peel_T=pp["T"], peel_Cu=pp["Cu"], peel_Cd=pp["Cd"])

    # --- the periodic backend's HardcodedModel: first-order fields of every
    # mode, then one training step of the streamfunction Rayleigh peel
    # (hardcoded_backend.py:3383-3771) with its all-mode device Adam
    hcfg = HB.cfg_namespace(dict(
        modes=4, hidden=8, hidden_layers=2, frequencies=3, xmin=0.0, xmax=2 * math.pi,
        ymin=0.0, ymax=2 * math.pi, geometry_mode="periodic_box",
        envelope_mode="periodic_identity", input_encoding="periodic_sincos_xy",
        canonical_siren=True, siren_first_omega0=8.0, siren_hidden_omega0=30.0,
        basis_objective="streamfunction_dirichlet_rayleigh", causal_sorting="geometry_rayleigh",
        reorthogonalization_passes=2, mass_floor=1e-14, learning_rate=1e-3, grad_clip=5.0,
        spatial_derivative_order=1, mode_forward_batch=2, mode_backward_batch=2,
        mlp_compute_dtype="float32", master_weight_dtype="float32"))
    harr = {}
    for mode in range(4):
        for layer, (inside, outside) in enumerate(((12, 8), (8, 8), (8, 1))):
            label = f"l{layer}" if layer < 2 else "output"
            for offset, (kind, shape) in enumerate((("weight", (outside, inside)),
                                                    ("bias", (outside,)))):
                harr[f"m{mode:03d}.{label}.{kind}"] = rng.normal(0, .15, size=shape)
                stem = f"m{mode:03d}.adam.p{2 * layer + offset:02d}"
                harr[stem + ".exp_avg"] = np.zeros(shape)
                harr[stem + ".exp_avg_sq"] = np.zeros(shape)
                harr[stem + ".step"] = np.asarray(0, "i8")
    hmodel = HB.HardcodedModel(hcfg, harr)
    hpts = rng.uniform(0, 2 * math.pi, size=(48, 2))
    fields = list(hmodel.forward_stream_jet1(hcfg, hpts, 0.0, 0.0, False))
    g.update(hb_points=hpts,
             hb_value=np.stack([np.asarray(f.value[:, 0]) for _, f, _ in fields]),
             hb_grad=np.stack([np.asarray(f.grad[:, 0]) for _, f, _ in fields]))
    # third-order jets of the same networks (forward_stream, HB:1882-1986)
    fields3 = list(hmodel.forward_stream(hcfg, hpts, 0.0, 0.0, False))
    for name in ("value", "grad", "hess", "third"):
        g["hb3_" + name] = np.stack([np.asarray(getattr(f, name)[:, 0]) for _, f, _ in fields3])
    for key, value in harr.items():
        g["hb_in." + key] = np.asarray(value)
    res = HB.peel_step(hcfg, hmodel, hpts, 0.0, 0.0, True)
    g.update(hb_loss=np.asarray(res["loss"]), hb_energies=np.asarray(res["mode_energies"]),
             hb_order=np.asarray(res["causal_order"]),
             hb_norm_min=np.asarray(res["gradient_norm_min"]),
             hb_norm_max=np.asarray(res["gradient_norm_max"]))
    for key, value in hmodel.arrays().items():
        g["hb_out." + key] = np.asarray(value)

    # the same networks with fixed-order sorting, and a three-mode network on
    # the free box (raw_xy inputs, free_identity envelope): one training step
    hcfg_fixed = HB.cfg_namespace(dict(vars(hcfg), causal_sorting="fixed_order"))
    fmodel = HB.HardcodedModel(hcfg_fixed, {k[6:]: v for k, v in g.items()
                                            if k.startswith("hb_in.")})
    res = HB.peel_step(hcfg_fixed, fmodel, hpts, 0.0, 0.0, True)
    g.update(hbf_loss=np.asarray(res["loss"]), hbf_energies=np.asarray(res["mode_energies"]),
             hbf_order=np.asarray(res["causal_order"]))
    for key, value in fmodel.arrays().items():
        g["hbf_out." + key] = np.asarray(value)
    free = HB.cfg_namespace(dict(
        modes=3, hidden=8, hidden_layers=2, xmin=-1.0, xmax=2.0, ymin=0.0, ymax=1.5,
        geometry_mode="free_box", envelope_mode="free_identity", input_encoding="raw_xy",
        canonical_siren=True, siren_first_omega0=3.0, siren_hidden_omega0=2.0,
        basis_objective="potential_rayleigh", causal_sorting="geometry_rayleigh",
        reorthogonalization_passes=2, mass_floor=1e-14, learning_rate=1e-3, grad_clip=5.0,
        spatial_derivative_order=1, mode_forward_batch=3, mode_backward_batch=3,
        mlp_compute_dtype="float32", master_weight_dtype="float32"))
    farr = {}
    for mode in range(3):
        for layer, (inside, outside) in enumerate(((2, 8), (8, 8), (8, 1))):
            label = f"l{layer}" if layer < 2 else "output"
            for offset, (kind, shape) in enumerate((("weight", (outside, inside)),
                                                    ("bias", (outside,)))):
                farr[f"m{mode:03d}.{label}.{kind}"] = rng.normal(0, .5, size=shape)
                stem = f"m{mode:03d}.adam.p{2 * layer + offset:02d}"
                farr[stem + ".exp_avg"] = np.zeros(shape)
                farr[stem + ".exp_avg_sq"] = np.zeros(shape)
                farr[stem + ".step"] = np.asarray(0, "i8")
    fpts = np.column_stack((rng.uniform(-1.0, 2.0, 40), rng.uniform(0.0, 1.5, 40)))
    fm = HB.HardcodedModel(free, farr)
    res = HB.peel_step(free, fm, fpts, 0.0, 0.0, True)
    g.update(hbfree_points=fpts, hbfree_loss=np.asarray(res["loss"]),
             hbfree_energies=np.asarray(res["mode_energies"]),
             hbfree_order=np.asarray(res["causal_order"]))
    for key, value in farr.items():
        g["hbfree_in." + key] = np.asarray(value)
    for key, value in fm.arrays().items():
        g["hbfree_out." + key] = np.asarray(value)

    # --- the trainer's epoch-0 arrays and fixed validation points
    # (prepare_gauge_canonical.py main, run on a three-mode configuration)
    import json
    import tempfile
    os.environ["NEB_2D_VENDOR_ROOT"] = str(reference_root() / "experiments/2d/_backend")
    prep = load(reference_root() / "experiments/2d/_backend/flow/cases/vortex_merger/"
                "neural_training/prepare_gauge_canonical.py", "prepare_gauge_canonical")
    pcfg = dict(seed=3, modes=3, hidden=8, hidden_layers=2, frequencies=2, input_features=8,
                xmin=0.0, xmax=2 * math.pi, ymin=0.0, ymax=2 * math.pi,
                geometry_mode="periodic_box", envelope_mode="periodic_identity",
                input_encoding="periodic_sincos_xy", canonical_siren=True,
                siren_first_omega0=8.0, siren_hidden_omega0=30.0,
                basis_objective="potential_rayleigh", spatial_derivative_order=1,
                sampling_mode="uniform_random", mlp_compute_dtype="float32",
                mlp_accumulation_dtype="float32", jet_dtype="float32",
                parameter_backward_dtype="float32", quadrature_dtype="float32",
                ritz_dtype="float32", master_weight_dtype="float32", optimizer_dtype="float32",
                validation_points=37, validation_beta_samples=1, validation_alpha_samples=1,
                alpha_min_deg=0.0, alpha_max_deg=0.0, probe_beta=0.0, probe_alpha_deg=0.0,
                learning_rate=1e-3)
    with tempfile.TemporaryDirectory() as tmp:
        conf = Path(tmp) / "config.json"
        conf.write_text(json.dumps(pcfg))
        saved = sys.argv
        sys.argv = ["prepare", "--config", str(conf), "--output-dir", str(Path(tmp) / "run")]
        try:
            prep.main()
        finally:
            sys.argv = saved
        with np.load(Path(tmp) / "run/initial_epoch0000.npz") as z:
            for key in z.files:
                g["init." + key] = np.asarray(z[key])
        with np.load(Path(tmp) / "run/fixed_validation_iid_uniform_v1.npz") as z:
            g["init_validation_points"] = np.asarray(z["validation_points"][0], np.float64)

    # --- the autonomous ETDRK4 Galerkin rollout (paper_rollout.py rollout) on
    # a random six-mode basis of the 128^2 grid
    roll = load(reference_root() / "experiments/periodic/paper_rollout.py", "paper_rollout")
    nr, kr = 128, 6
    coef = rng.normal(size=(kr, len(ROLLOUT_WAVES), 3, 2))
    basis = rollout_basis(coef, nr)  # [3, n^2, K]
    u0 = (basis[0, :, 0] - 0.7 * basis[0, :, 1] + 0.4 * basis[0, :, 3]).reshape(nr, nr)
    v0 = (basis[1, :, 0] - 0.7 * basis[1, :, 1] + 0.4 * basis[1, :, 3]).reshape(nr, nr)
    # the normalisation and Ritz stage of paper_rollout.py:171-192, then the
    # rollout in the rotated basis
    weight = (2 * math.pi / nr) ** 2
    gu, gv, gw = basis
    norm = np.sqrt(weight * np.sum(gu * gu + gv * gv, axis=0))
    gu, gv, gw = gu / norm, gv / norm, gw / norm
    mass = weight * (gu.T @ gu + gv.T @ gv)
    stiff = weight * (gw.T @ gw)
    vals, transform = sla.eigh((stiff + stiff.T) / 2, (mass + mass.T) / 2)
    rtimes = np.linspace(0.0, 0.3, 7)
    gt = dict(time=rtimes, velocity_u=u0[None], velocity_v=v0[None], nu=0.05)
    with tempfile.TemporaryDirectory() as tmp:
        fields_r, states_r, skew_r, _, _ = roll.rollout(gu @ transform, gv @ transform,
                                                        gw @ transform, vals, gt, 0.02,
                                                        Path(tmp), "golden")
    g.update(roll_coef=coef, roll_vals=vals,
             roll_times=rtimes, roll_nu=np.asarray(0.05), roll_dt=np.asarray(0.02),
             roll_states=states_r, roll_u_frames=fields_r[0].reshape(len(rtimes), -1)[:, :64],
             roll_skew=np.asarray(skew_r))

    g = {key: np.asarray(v, dtype=np.float64) if np.asarray(v).dtype.kind == "f" else np.asarray(v)
         for key, v in g.items()}
    np.savez_compressed(OUT, **g)
    print(f"wrote {OUT} ({len(g)} arrays)")


if __name__ == "__main__":
    main()
