"""The periodic backend's API on the mode-stacked kernels.

``HardcodedModel`` keeps the interface of the reference's 2D backend
(experiments/2d/_backend/periodic_core/vortex_merger/src/eigenfluid/gen/
vortex_merger2d/hardcoded_backend.py): ``HardcodedModel(cfg, arrays)`` from
the checkpoint key schema ``m{k:03d}.l{i}.{weight,bias}``,
``m{k:03d}.output.{weight,bias}`` and ``m{k:03d}.adam.pNN.{exp_avg,
exp_avg_sq,step}`` (:1435-1474, :1596-1714, :1987-2032); ``modes`` with
per-mode ``weights``, ``biases``, ``steps`` and ``adam_step(gradients,
cfg)`` (:1548-1587); the generators ``forward_stream_jet1`` /
``forward_stream_jet2`` yielding ``(mode, field, cache)`` with fields
value [n, 1], grad [n, 1, 2] (and hess [n, 1, 3], order xx, xy, yy)
(:1716-1880); ``backward_gradients_block_jet1`` / ``_jet2`` (:2034-2139);
``adam_step_jet1_device`` with its active-mode mask and physical validity
flag (:2184-2277); ``arrays()``; and ``peel_step`` (:3774-3811) for the
streamfunction Rayleigh objective (:3383-3771).

The peel step runs in Gram form: the modes' mean-removed values V [n, K] and
gradients G [2n, K], M = w V^T V and S = w G^T G in FP64 (w = area / n), the
causal peel (``coefficient_peel``, two orthonormalisation passes), the
detached-prefix gradient of the summed peeled quotients, the all-mode device
Adam transaction gated by the peel's status, and one host read of the
diagnostics per step.

Supported trial spaces: the periodic box (``periodic_sincos_xy`` features,
``periodic_identity`` envelope) and the free box (``raw_xy``,
``free_identity``); the airfoil / C2 geometries are outside this path.
Master parameters are FP32 as in the reference (``precision="fp64"`` for
checks); ``mlp_compute_dtype="float16"`` computes in FP32.  Parameters live on
the GPU as mode-stacked tensors (one ``ModeModel``); the per-mode views alias
them.
"""
from __future__ import annotations

import ctypes
from contextlib import contextmanager
from types import SimpleNamespace

import numpy as np
import torch

from . import _native as N
from .jets import Jet
from .modes import ModeModel, ModeNet, ModeTape, column_apply, column_gram, coefficient_peel

PERIODIC = ("periodic_box", "periodic_identity", "periodic_sincos_xy")
FREE = ("free_box", "free_identity", "raw_xy")


def _stream() -> int:
    return torch.cuda.current_stream().cuda_stream


def siren_layer_omega(cfg, layer: int) -> float:
    """The sine frequency of hidden layer ``layer`` (hardcoded_backend.py:
    1250-1260): 1 for legacy networks, else the configured omega0."""
    if not bool(getattr(cfg, "canonical_siren", False)):
        return 1.0
    return float(getattr(cfg, "siren_first_omega0" if layer == 0 else "siren_hidden_omega0", 30.0))


def _trial_space(cfg):
    space = (str(getattr(cfg, "geometry_mode", "")), str(getattr(cfg, "envelope_mode", "")),
             str(getattr(cfg, "input_encoding", "")))
    if space not in (PERIODIC, FREE):
        raise NotImplementedError(
            "the periodic (periodic_box, periodic_identity, periodic_sincos_xy) and free "
            "(free_box, free_identity, raw_xy) trial spaces are supported")
    return space


class HardcodedMode:
    """One mode's view of the stacked parameters (the reference's per-mode
    object); ``weights`` / ``biases`` alias rows of the stacks."""

    def __init__(self, model: "HardcodedModel", index: int):
        self.model = model
        self.mode_index = index

    @property
    def weights(self):
        return [w[self.mode_index] for w in self.model.core.W]

    @property
    def biases(self):
        return [b[self.mode_index] for b in self.model.core.b]

    @property
    def exp_avg(self):
        c = self.model.core
        return [t[self.mode_index] for pair in zip(c.mW, c.mb) for t in pair]

    @property
    def exp_avg_sq(self):
        c = self.model.core
        return [t[self.mode_index] for pair in zip(c.vW, c.vb) for t in pair]

    @property
    def steps(self):
        """Adam step count of every parameter tensor of this mode (one device
        read)."""
        return [int(self.model.steps[self.mode_index].item())] * (2 * len(self.model.core.W))

    @steps.setter
    def steps(self, value) -> None:
        counts = {int(v) for v in value}
        if len(counts) != 1:
            raise ValueError("every parameter tensor of a mode shares one Adam step count")
        self.model.steps[self.mode_index] = counts.pop()

    def adam_step(self, gradients, cfg) -> None:
        """Adam on this mode alone (hardcoded_backend.py:1548-1587): the
        gradients [W_0, b_0, W_1, b_1, ...]; raises FloatingPointError with
        nothing changed unless every tensor is finite and the total norm is
        positive; clip at cfg.grad_clip, lr cfg.learning_rate."""
        core = self.model.core
        k = self.mode_index
        if len(gradients) != 2 * len(core.W):
            raise RuntimeError("hardcoded reverse pass returned the wrong gradient count")
        params, m, v = [], [], []
        for j in range(len(core.W)):
            params += [core.W[j][k], core.b[j][k]]
            m += [core.mW[j][k], core.mb[j][k]]
            v += [core.vW[j][k], core.vb[j][k]]
        grads = [torch.as_tensor(g, device=core.device).to(core.dtype).contiguous()
                 for g in gradients]
        for p, g in zip(params, grads):
            if p.shape != g.shape:
                raise ValueError(f"gradient shape {tuple(g.shape)} != parameter {tuple(p.shape)}")
        sizes = (ctypes.c_int64 * len(params))(*[p.numel() for p in params])
        committed = torch.empty((), dtype=torch.int32, device=core.device)
        lib = N.load()
        ws = core._buf("adam1", lib.neb_modes_adam_workspace_bytes(1))
        N.call("neb_modes_adam", 1 if core.dtype == torch.float64 else 0, 1, len(params),
               N.ptr_array(params), N.ptr_array(m), N.ptr_array(v), N.ptr_array(grads), sizes,
               self.model.steps[k:k + 1].data_ptr(), 1, 0, 0, float(cfg.learning_rate),
               float(cfg.grad_clip), 0, committed.data_ptr(), ws.data_ptr(), ws.numel(),
               _stream())
        if not bool(committed.item()):
            raise FloatingPointError("zero or non-finite total hardcoded gradient")


class HardcodedModel:
    """cfg.modes per-mode SIRENs of the periodic / free 2D backend."""

    def __init__(self, cfg, arrays: dict, precision: str = "fp32",
                 device: str | torch.device = "cuda"):
        _trial_space(cfg)
        K = int(cfg.modes)
        layers = int(cfg.hidden_layers)
        labels = [f"l{i}" for i in range(layers)] + ["output"]
        W = [np.stack([np.asarray(arrays[f"m{k:03d}.{lab}.weight"]) for k in range(K)])
             for lab in labels]
        b = [np.stack([np.asarray(arrays[f"m{k:03d}.{lab}.bias"]) for k in range(K)])
             for lab in labels]
        if str(getattr(cfg, "mlp_compute_dtype", "float32")).lower() not in ("float16", "float32", "float64"):
            raise ValueError(f"Unsupported MLP compute dtype: {cfg.mlp_compute_dtype}")
        widths = [W[0].shape[2]] + [w.shape[1] for w in W]
        if any(w != widths[1] for w in widths[1:-1]):
            raise ValueError("hidden layers of different widths are not supported")
        shape = SimpleNamespace(hidden=widths[1], hidden_layers=layers,
                                siren_first_omega0=siren_layer_omega(cfg, 0),
                                siren_hidden_omega0=siren_layer_omega(cfg, 1))
        self.core = ModeModel(shape, K=K, seed=0, inputs=widths[0], outputs=widths[-1],
                              dim=2, order=1, precision=precision, device=device)
        core = self.core
        for j in range(len(W)):
            core.W[j].copy_(torch.as_tensor(W[j], dtype=core.dtype))
            core.b[j].copy_(torch.as_tensor(b[j], dtype=core.dtype))
            for name, (wt, bt) in (("exp_avg", (core.mW, core.mb)),
                                   ("exp_avg_sq", (core.vW, core.vb))):
                for which, target in enumerate((wt, bt)):
                    target[j].copy_(torch.as_tensor(np.stack([
                        np.asarray(arrays[f"m{k:03d}.adam.p{2 * j + which:02d}.{name}"])
                        for k in range(K)]), dtype=core.dtype))
        steps = []
        for k in range(K):
            s = {int(np.asarray(arrays[f"m{k:03d}.adam.p{i:02d}.step"]))
                 for i in range(2 * len(W))}
            if len(s) != 1:
                raise ValueError(f"mode {k}: parameter tensors with different Adam step counts")
            steps.append(s.pop())
        self.steps = torch.tensor(steps, dtype=torch.int32, device=core.device)
        self.modes = [HardcodedMode(self, k) for k in range(K)]
        self._nets = {1: core.net}

    def _net(self, order: int):
        """The stacked network's shape with jets of ``order`` (1, 2 or 3)."""
        if order not in self._nets:
            n1 = self._nets[1]
            self._nets[order] = ModeNet(2, order, n1.n_layers, n1.widths, self.core.K,
                                        n1.precision, n1.omega_first, n1.omega_hidden)
        return self._nets[order]

    @contextmanager
    def _order(self, order: int):
        """The stacked network with jets of ``order`` (1, 2 or 3) for the
        duration of one call."""
        core = self.core
        saved = core.net, core.order
        core.net, core.order = self._net(order), order
        try:
            yield core
        finally:
            core.net, core.order = saved

    # ------------------------------------------------------------ features
    def features(self, cfg, points, order: int = 1) -> torch.Tensor:
        """Input feature jets [n, C, F] (C = 3, 6, 10 for order 1, 2, 3:
        value, x, y[, xx, xy, yy[, xxx, xxy, xyy, yyy]]) of points [n, 2]:
        sin / cos of pi h (s_n + 1) for the coordinate s_n normalised to
        [-1, 1], h = 1..cfg.frequencies, x then y (hardcoded_backend.py:
        418-438 and the Jet2 / Jet3 encodings), or the raw coordinates."""
        core = self.core
        pts = torch.as_tensor(points, device=core.device).to(torch.float64).contiguous()
        if pts.ndim != 2 or pts.shape[1] != 2:
            raise ValueError("points must be [n, 2]")
        if order not in (1, 2, 3):
            raise ValueError("jet order 1, 2 or 3")
        n = pts.shape[0]
        C = (3, 6, 10)[order - 1]
        if _trial_space(cfg) == FREE:
            f = torch.zeros((n, C, 2), dtype=core.dtype, device=core.device)
            f[:, 0] = pts.to(core.dtype)
            f[:, 1, 0] = 1.0
            f[:, 2, 1] = 1.0
            return f
        Fq = int(cfg.frequencies)
        if core.widths[0] != 4 * Fq:
            raise ValueError(f"first layer takes {core.widths[0]} inputs, the encoding "
                             f"{4 * Fq}")
        origin = torch.tensor([cfg.xmin, cfg.ymin], dtype=torch.float64, device=core.device)
        shifted = (pts - origin).contiguous()
        out = torch.empty((n, C, 4 * Fq), dtype=core.dtype, device=core.device)
        N.call("neb_periodic_features", core.storage_prec, order, Fq,
               float(cfg.xmax - cfg.xmin), float(cfg.ymax - cfg.ymin), shifted.data_ptr(), n,
               out.data_ptr(), _stream())
        return out

    # ------------------------------------------------------------- forward
    def _forward_block(self, feats, start, stop, cache, order):
        with self._order(order) as core:
            return core.forward_packed(feats, None, start, stop, cache)

    def _stream_fields(self, cfg, points, cache: bool, order: int):
        feats = self.features(cfg, points, order)
        K = self.core.K
        block = max(1, int(getattr(cfg, "mode_forward_batch", 1)))
        for start in range(0, K, block):
            stop = min(K, start + block)
            out, tape = self._forward_block(feats, start, stop, cache, order)
            for local in range(stop - start):
                o = out[local]  # [n, C, 1]
                hess = o[:, 3:6].permute(0, 2, 1) if order == 2 else None
                field = Jet(o[:, 0], o[:, 1:3].permute(0, 2, 1), hess=hess)
                yield self.modes[start + local], field, ((tape, order) if cache else None)

    def forward_stream_jet1(self, cfg, points, beta: float = 0.0, alpha: float = 0.0,
                            cache: bool = False):
        """(mode, Jet(value [n, 1], grad [n, 1, 2]), cache) for every mode,
        evaluated in blocks of cfg.mode_forward_batch modes."""
        yield from self._stream_fields(cfg, points, cache, 1)

    def forward_stream_jet2(self, cfg, points, beta: float = 0.0, alpha: float = 0.0,
                            cache: bool = False):
        """(mode, Jet(value, grad, hess [n, 1, 3] = xx, xy, yy), cache)."""
        yield from self._stream_fields(cfg, points, cache, 2)

    def forward_stream(self, cfg, points, beta: float = 0.0, alpha: float = 0.0,
                       cache: bool = False, mode_indices=None):
        """(mode, Jet(value, grad, hess, third [n, 1, 4] = xxx, xxy, xyy,
        yyy), None) for every mode: the reference's third-order evaluation
        stream (hardcoded_backend.py:1882-1986), in network order (a given
        mode_indices must be a permutation of all modes and sets the order).
        Evaluation only: no reverse pass of third-order jets."""
        if cache:
            raise NotImplementedError("third-order jets are evaluation only (cache=False)")
        K = self.core.K
        order = list(range(K)) if mode_indices is None else [int(i) for i in mode_indices]
        if sorted(order) != list(range(K)):
            raise ValueError("mode_indices must be a permutation of all modes")
        feats = self.features(cfg, points, 3)
        block = max(1, int(getattr(cfg, "mode_forward_batch", 1)))
        cached = {}
        for start in range(0, K, block):
            stop = min(K, start + block)
            for k in order[start:stop]:
                if k not in cached:
                    cached.clear()
                    a = (k // block) * block
                    out, _ = self._forward_block(feats, a, min(K, a + block), False, 3)
                    for j in range(a, min(K, a + block)):
                        cached[j] = out[j - a]
                o = cached[k]  # [n, 10, 1]
                yield self.modes[k], Jet(o[:, 0], o[:, 1:3].permute(0, 2, 1),
                                         hess=o[:, 3:6].permute(0, 2, 1),
                                         third=o[:, 6:10].permute(0, 2, 1)), None

    # ------------------------------------------------------------- reverse
    def _backward_block(self, modes, caches, field_adjoints, order):
        if not modes:
            return [], []
        idx = [m.mode_index for m in modes]
        start, stop = idx[0], idx[0] + len(idx)
        if idx != list(range(start, stop)):
            raise RuntimeError(f"Jet{order} backward mode block must be contiguous")
        if len(caches) != len(idx) or len(field_adjoints) != len(idx):
            raise ValueError("one cache and one field adjoint per mode")
        if any(c is None or c[1] != order for c in caches):
            raise ValueError(f"backward needs the caches of forward_stream_jet{order}(cache=True)")
        tape: ModeTape = caches[0][0]
        if (tape.start, tape.stop) != (start, stop) or any(c[0] is not tape for c in caches):
            # the block differs from the forward block: recompute its tape
            _, tape = self._forward_block(tape.features, start, stop, True, order)
        core = self.core
        chans = []
        for a in field_adjoints:
            parts = [torch.as_tensor(a.value, device=core.device).reshape(-1, 1, 1),
                     torch.as_tensor(a.grad, device=core.device).reshape(-1, 1, 2).permute(0, 2, 1)]
            if order == 2:
                parts.append(torch.as_tensor(a.hess, device=core.device)
                             .reshape(-1, 1, 3).permute(0, 2, 1))
            chans.append(torch.cat(parts, dim=1))
        adj = torch.stack(chans).to(core.dtype).contiguous()
        with self._order(order):
            return core.backward_packed(tape, adj)

    def backward_gradients_block_jet1(self, cfg, modes, caches, field_adjoints):
        """Parameter gradients ([B, out, in] and [B, out] per layer) of a
        contiguous block of modes from their first-order field adjoints."""
        return self._backward_block(modes, caches, field_adjoints, 1)

    def backward_gradients_block_jet2(self, cfg, modes, caches, field_adjoints):
        """As backward_gradients_block_jet1 with second-order adjoints."""
        return self._backward_block(modes, caches, field_adjoints, 2)

    # -------------------------------------------------------------- optimiser
    def adam_step_jet1_device(self, cfg, weight_grads, bias_grads, active_modes=None,
                              physical_valid=None):
        """One all-mode Adam transaction on the device (hardcoded_backend.py:
        2184-2277): per-mode clip at cfg.grad_clip, lr cfg.learning_rate.  It
        commits only when physical_valid holds and every active mode's
        gradient is finite with a positive norm; on commit the active modes
        update and their step counts advance.  ``physical_valid``: a device
        bool, or an int32 status word (0 = valid).  Returns device (norms,
        committed); no host synchronisation."""
        core = self.core
        if len(weight_grads) != len(core.W) or len(bias_grads) != len(core.b):
            raise RuntimeError("Jet1 reverse pass returned the wrong gradient count")
        params = [*core.W, *core.b]
        grads = [torch.as_tensor(g, device=core.device).to(core.dtype).contiguous()
                 for g in [*weight_grads, *bias_grads]]
        for p, g in zip(params, grads):
            if p.shape != g.shape:
                raise ValueError(f"gradient shape {tuple(g.shape)} != parameter {tuple(p.shape)}")
        sizes = (ctypes.c_int64 * len(params))(*[p.numel() for p in params])
        norms = torch.empty(core.K, dtype=torch.float64, device=core.device)
        committed = torch.empty((), dtype=torch.int32, device=core.device)
        active = None if active_modes is None else \
            torch.as_tensor(active_modes, device=core.device).to(torch.int32).contiguous()
        gate = None
        if physical_valid is not None:
            if isinstance(physical_valid, torch.Tensor) and physical_valid.dtype == torch.int32:
                gate = physical_valid
            else:
                gate = (~torch.as_tensor(physical_valid, device=core.device)
                        .to(torch.bool)).to(torch.int32)
        lib = N.load()
        ws = core._buf("adam", lib.neb_modes_adam_workspace_bytes(core.K))
        N.call("neb_modes_adam", 1 if core.dtype == torch.float64 else 0, core.K, len(params),
               N.ptr_array(params), N.ptr_array([*core.mW, *core.mb]),
               N.ptr_array([*core.vW, *core.vb]), N.ptr_array(grads), sizes,
               self.steps.data_ptr(), 1, 0 if active is None else active.data_ptr(),
               0 if gate is None else gate.data_ptr(), float(cfg.learning_rate),
               float(cfg.grad_clip), norms.data_ptr(), committed.data_ptr(), ws.data_ptr(),
               ws.numel(), _stream())
        return norms, committed

    # ----------------------------------------------------------- checkpoint
    def save(self, path) -> None:
        """``arrays()`` to an .npz, written to a temporary file and then moved
        into place (the reference's save_npz)."""
        from pathlib import Path
        path = Path(path)
        tmp = path.with_suffix(path.suffix + ".tmp")
        with tmp.open("wb") as stream:
            np.savez(stream, **self.arrays())
        tmp.replace(path)

    def arrays(self) -> dict:
        """Checkpoint arrays under the reference's key schema, one device to
        host copy per stacked tensor."""
        core = self.core
        L = len(core.W)
        host = {name: [t.detach().cpu().numpy() for t in getattr(core, name)]
                for name in ("W", "b", "mW", "mb", "vW", "vb")}
        steps = self.steps.cpu().numpy()
        out = {}
        for k in range(core.K):
            p = f"m{k:03d}"
            for j in range(L):
                lab = f"l{j}" if j < L - 1 else "output"
                out[f"{p}.{lab}.weight"] = host["W"][j][k]
                out[f"{p}.{lab}.bias"] = host["b"][j][k]
                for which, (m_name, v_name) in enumerate((("mW", "vW"), ("mb", "vb"))):
                    stem = f"{p}.adam.p{2 * j + which:02d}"
                    out[f"{stem}.exp_avg"] = host[m_name][j][k]
                    out[f"{stem}.exp_avg_sq"] = host[v_name][j][k]
                    out[f"{stem}.step"] = np.asarray(steps[k], dtype=np.int64)
        return out


# ------------------------------------------------------------------ peel step
TAPE_BUDGET = 16 << 30  # bytes of activation tape one block of modes may hold


def _block(core: ModeModel, n: int) -> int:
    """Modes per block of the peel step: as many as keep the block's tape
    within TAPE_BUDGET (the reference's mode_forward_batch bounds its own
    memory; the results do not depend on the blocking)."""
    per_mode = max(1, N.load().neb_modes_tape_bytes(ctypes.byref(core.net), 1, n))
    return max(1, min(core.K, TAPE_BUDGET // per_mode))


def _streamfunction_peel_step(cfg, model: HardcodedModel, points, training: bool) -> dict:
    """The streamfunction (potential) Rayleigh peel step of the periodic
    backend (hardcoded_backend.py:3383-3771) in Gram form on the device."""
    core = model.core
    _trial_space(cfg)
    if int(getattr(cfg, "spatial_derivative_order", 0)) < 1:
        raise ValueError("Dirichlet streamfunction Rayleigh requires spatial gradients")
    sorting = str(getattr(cfg, "causal_sorting", "fixed_order"))
    if sorting not in ("fixed_order", "geometry_rayleigh"):
        raise ValueError(f"unsupported causal_sorting {sorting!r}")
    if int(getattr(cfg, "freeze_prefix_modes", 0)) != 0:
        raise NotImplementedError("freeze_prefix_modes > 0 is not supported")
    if max(1, int(getattr(cfg, "reorthogonalization_passes", 2))) != 2:
        raise NotImplementedError("the Gram-form peel applies two orthonormalisation passes")
    n = len(points)
    if n == 0:
        raise ValueError("Dirichlet streamfunction Rayleigh received no points")
    K = core.K
    if int(cfg.modes) != K:
        raise ValueError("configuration/model mode count mismatch")
    weight = float(np.float32((cfg.xmax - cfg.xmin) * (cfg.ymax - cfg.ymin)) / np.float32(n))
    mass_floor = float(cfg.mass_floor)
    prec = core.storage_prec
    s = _stream()
    feats = model.features(cfg, points, 1)
    V = torch.empty((n, K), dtype=core.dtype, device=core.device)
    G = torch.empty((2 * n, K), dtype=core.dtype, device=core.device)
    block = _block(core, n)
    blocks = [(a, min(K, a + block)) for a in range(0, K, block)]
    # one block holds every mode: keep its tape for the reverse pass instead
    # of recomputing it (the reference recomputes each block, HB:3614-3629)
    keep = training and len(blocks) == 1
    tapes = {}
    for a, b in blocks:
        out, tape = core.forward_packed(feats, None, a, b, cache=keep)
        if keep:
            tapes[a] = tape
        N.call("neb_potential_fields", prec, out.data_ptr(), a, b, n, K, V.data_ptr(),
               G.data_ptr(), s)
    # the additive streamfunction constant is a gauge: project it out
    N.call("neb_column_center", prec, n, K, V.data_ptr(), s)
    M = column_gram(V, weight)
    S = column_gram(G, weight)
    peel = coefficient_peel(M, S, check=False, mass_floor=mass_floor,
                            sort=sorting == "geometry_rayleigh")
    f64 = dict(dtype=torch.float64, device=core.device)
    norms = torch.full((K,), float("nan"), **f64)
    committed = torch.zeros((), dtype=torch.int32, device=core.device)
    if training:
        dV = column_apply(V, peel.Cu, weight, core.precision)
        dG = column_apply(G, peel.Cd, weight, core.precision)
        N.call("neb_column_center", prec, n, K, dV.data_ptr(), s)
        gW = [torch.empty_like(w) for w in core.W]
        gb = [torch.empty_like(x) for x in core.b]
        for a, b in blocks:
            tape = tapes.pop(a, None) or core.forward_packed(feats, None, a, b, cache=True)[1]
            adj = torch.empty((b - a, n, 3, 1), dtype=core.dtype, device=core.device)
            N.call("neb_potential_lift", prec, dV.data_ptr(), dG.data_ptr(), a, b, n, K,
                   adj.data_ptr(), s)
            core.backward_packed(tape, adj, [g[a:b] for g in gW], [g[a:b] for g in gb])
        norms, committed = model.adam_step_jet1_device(cfg, gW, gb, None, peel.info)
    # the step's one host read: the diagnostic table
    ones = torch.ones(K, **f64)
    table = torch.stack((
        peel.losses, peel.order.to(torch.float64), peel.relative_mass, torch.diagonal(M),
        torch.diagonal(S), norms, ones * committed.to(torch.float64),
        ones * peel.info.to(torch.float64), ones * peel.gram_max)).cpu().numpy()
    losses, order_f, relative, rmass, rstiff, gnorms, done, info, orth = table
    order = order_f.astype(np.int64)
    with np.errstate(divide="ignore", invalid="ignore"):
        sorting_rayleigh = rstiff / rmass
    bad = ~(np.isfinite(rmass) & np.isfinite(rstiff) & np.isfinite(sorting_rayleigh)) | \
        (rmass <= mass_floor)
    if np.any(bad):
        net = int(np.flatnonzero(bad)[0])
        raise FloatingPointError(
            "causal sorting received an invalid streamfunction candidate "
            f"{net + 1}: M={rmass[net]:.8e}, K={rstiff[net]:.8e}")
    if info[0] != 0:
        raise FloatingPointError("a peeled streamfunction candidate is invalid (non-finite, or "
                                 "its mass at or below mass_floor); no update")
    if training and not bool(done[0]):
        bad = ~np.isfinite(gnorms) | (gnorms <= 0.0)
        net = int(np.flatnonzero(bad)[0]) if np.any(bad) else -1
        raise FloatingPointError("zero or non-finite total hardcoded gradient"
                                 + (f" for network mode {net + 1}" if net >= 0 else ""))
    projection = np.where(np.arange(K) > 0, 1.0 / relative - 1.0, 0.0)
    by_network = np.empty(K)
    by_network[order] = losses
    mean = float(np.mean(losses))
    resident = isinstance(points, torch.Tensor) and points.is_cuda
    return {
        "loss": mean, "base_loss": mean, "streamfunction_rayleigh": mean, "mean_energy": mean,
        "max_energy": float(np.max(losses)), "min_energy": float(np.min(losses)),
        "mean_projection_ratio": float(np.mean(projection)), "orth_error": float(orth[0]),
        "peeled_rank": K, "requested_modes": K, "mode_energies": losses.tolist(),
        "mode_energies_by_network": by_network.tolist(), "causal_sorting": sorting,
        "causal_order": order.tolist(), "causal_order_1based": (order + 1).tolist(),
        "sorting_rayleigh_by_network": sorting_rayleigh.tolist(),
        "spatial_jet_order_used": 1, "causal_sort_device": "gpu",
        "diagnostic_host_transfers_per_step": 1, "optimizer_device": "gpu_batched_all_modes",
        "optimizer_host_transfers_per_step": 0,
        "input_host_to_device_transfers_per_step": int(not resident),
        "sample_pack_device": "gpu_resident" if resident else "host_per_step",
        "gradient_norm_min": float(np.min(gnorms)) if training else float("nan"),
        "gradient_norm_max": float(np.max(gnorms)) if training else float("nan"),
    }


def peel_step(cfg, model: HardcodedModel, points, beta: float = 0.0, alpha: float = 0.0,
              training: bool = True, reference_model=None, full_diagnostics: bool = True) -> dict:
    """Dispatch on cfg.basis_objective (hardcoded_backend.py:3774-3811); the
    streamfunction (potential) Rayleigh objective is built on this path."""
    objective = str(getattr(cfg, "basis_objective", ""))
    if reference_model is not None:
        raise ValueError("Rayleigh training uses no reference model")
    if objective in {"potential_rayleigh", "streamfunction_dirichlet_rayleigh"}:
        return _streamfunction_peel_step(cfg, model, points, training)
    if objective in {"pure_vorticity_rayleigh", "velocity_rayleigh"}:
        raise NotImplementedError(f"basis_objective={objective!r} is not built on this path")
    raise ValueError(f"unsupported basis_objective={objective!r}")


# ----------------------------------------------------- initialisation, points
def initial_arrays(cfg) -> dict:
    """Epoch-0 checkpoint arrays of the reference's trainer preparation
    (experiments/2d/_backend/flow/cases/vortex_merger/neural_training/
    prepare_gauge_canonical.py:51-86): one PCG64 generator seeded cfg.seed
    drawn mode after mode, layer after layer, weight then bias, uniform in
    +-bound (canonical SIREN: 1 / fan_in on the first layer, sqrt(6 / fan_in)
    / omega_hidden after and on the output layer, bias bound 1 / sqrt(fan_in);
    otherwise gain / sqrt(fan_in)), float32; zero Adam moments, step 0."""
    import math
    rng = np.random.default_rng(int(cfg.seed))
    encoding = str(getattr(cfg, "input_encoding", ""))
    fan0 = int(getattr(cfg, "input_features", 2 if encoding == "raw_xy" else 0))
    siren = bool(getattr(cfg, "canonical_siren", False))
    g_first = float(getattr(cfg, "initial_first_layer_gain", 1.0))
    g_hidden = float(getattr(cfg, "initial_hidden_layer_gain", 1.0))
    g_out = float(getattr(cfg, "initial_output_layer_gain", 1.0))
    arrays = {}
    for mode in range(int(cfg.modes)):
        prefix = f"m{mode:03d}"
        names = []
        fan_in = fan0
        for layer in range(int(cfg.hidden_layers)):
            if siren:
                bound = 1.0 / fan_in if layer == 0 else \
                    math.sqrt(6.0 / fan_in) / float(cfg.siren_hidden_omega0)
                bias_bound = 1.0 / math.sqrt(fan_in)
            else:
                bound = (g_first if layer == 0 else g_hidden) / math.sqrt(fan_in)
                bias_bound = bound
            w, b = f"{prefix}.l{layer}.weight", f"{prefix}.l{layer}.bias"
            arrays[w] = rng.uniform(-bound, bound, (int(cfg.hidden), fan_in)).astype(np.float32)
            arrays[b] = rng.uniform(-bias_bound, bias_bound, int(cfg.hidden)).astype(np.float32)
            names += [w, b]
            fan_in = int(cfg.hidden)
        bound = math.sqrt(6.0 / fan_in) / float(cfg.siren_hidden_omega0) if siren else \
            g_out / math.sqrt(fan_in)
        bias_bound = 1.0 / math.sqrt(fan_in)
        w, b = f"{prefix}.output.weight", f"{prefix}.output.bias"
        arrays[w] = rng.uniform(-bound, bound, (1, fan_in)).astype(np.float32)
        arrays[b] = rng.uniform(-bias_bound, bias_bound, 1).astype(np.float32)
        names += [w, b]
        for index, name in enumerate(names):
            stem = f"{prefix}.adam.p{index:02d}"
            arrays[f"{stem}.exp_avg"] = np.zeros_like(arrays[name])
            arrays[f"{stem}.exp_avg_sq"] = np.zeros_like(arrays[name])
            arrays[f"{stem}.step"] = np.asarray(0, dtype=np.int64)
    return arrays


def fluid_points(cfg, count: int, beta: float, alpha: float, seed: int) -> np.ndarray:
    """Quadrature points of one step in the periodic or free box
    (hardcoded_backend.py:2425-2447, sampling_mode uniform_random; the box
    has no body, so every candidate is accepted): PCG64 seeded ``seed``,
    max(2 count, 128) x-draws, then as many y-draws, the first ``count``
    pairs, float32."""
    if str(getattr(cfg, "sampling_mode", "")) != "uniform_random":
        raise NotImplementedError("sampling_mode uniform_random is supported")
    _trial_space(cfg)
    rng = np.random.default_rng(seed)
    draws = max(2 * count, 128)
    x = rng.uniform(cfg.xmin, cfg.xmax, draws)
    y = rng.uniform(cfg.ymin, cfg.ymax, draws)
    return np.column_stack((x, y))[:count].astype(np.float32, copy=False)
