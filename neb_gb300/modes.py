"""Mode-stacked SIREN networks: the reference's own per-mode architecture.

``ModeModel`` keeps the interface of the reference's native network backend
(experiments/metaball/_backend/flow/cases/metaball/native_cupy_core.py:
111-185): ``Model(c, K, seed)`` with the configuration fields ``hidden``,
``hidden_layers``, ``siren_first_omega0``, ``siren_hidden_omega0``; stacked
parameters ``W[j]`` [K, out, in] and ``b[j]`` [K, out]; Adam moments
``mW, vW, mb, vb``; ``epoch``; ``forward(data, start, stop, cache)`` returning
the output jet of modes [start, stop) times the envelope, and the tape;
``backward(data, start, stop, cache, adj)`` returning that block's parameter
gradients; ``adam(gW, gb, lr, clip)`` returning per-mode gradient norms and
raising ``FloatingPointError`` with nothing changed; ``save`` / ``load`` with
the keys ``W_j, b_j, mW_j, vW_j, mb_j, vb_j, epoch``.  ``data`` carries
``features`` and ``envelope`` jets with ``value`` [n, F], ``grad`` [n, F, dim]
(and ``hess`` [n, F, dim (dim + 1) / 2] for second-order jets), as the
reference's Jet1 / J2 objects do; ``envelope`` may be None (identity).

``velocity_step`` is the 3D velocity objective of velocity/core.py:79-103
on the same network with second-order jets: velocity and velocity gradient
of every mode's vector potential, the FP64 Grams, the causal peel in Gram
form (``coefficient_peel``) and the hand-written parameter gradient.

Every computation runs in the library's CUDA kernels (``neb_modes_*``,
``neb_coefficient_peel``, ``neb_column_*``); PyTorch provides device memory
and the current stream.
"""
from __future__ import annotations

import ctypes
import math
from dataclasses import dataclass
from pathlib import Path

import numpy as np
import torch

from . import _native as N
from .jets import Jet


def _stream() -> int:
    return torch.cuda.current_stream().cuda_stream


ModeNet = N.ModeNet


def siren_init(c, K: int, seed: int, inputs: int, outputs: int):
    """Per-mode SIREN initialisation of the reference (native_cupy_core.py:
    116-124): one PCG64 generator per mode, seeded seed + 7919 (k + 1);
    layer j draws W, then b, uniform in +-bound with bound = 1 / fan_in on
    the first layer and sqrt(6 / fan_in) / siren_hidden_omega0 after, in
    float32.  Returns lists of stacked [K, out, in] and [K, out] arrays."""
    shapes = [inputs] + [c.hidden] * c.hidden_layers + [outputs]
    gens = [np.random.Generator(np.random.PCG64(seed + 7919 * (i + 1))) for i in range(K)]
    W, b = [], []
    for j, (inp, out) in enumerate(zip(shapes[:-1], shapes[1:])):
        bound = 1 / inp if j == 0 else math.sqrt(6 / inp) / c.siren_hidden_omega0
        W.append(np.stack([r.uniform(-bound, bound, (out, inp)).astype("f4") for r in gens]))
        b.append(np.stack([r.uniform(-bound, bound, out).astype("f4") for r in gens]))
    return W, b


def jet_channels(dim: int, order: int) -> int:
    """Channels of a jet: value, gradient, compact Hessian (order >= 2) and
    the four third derivatives of a 2D third-order jet."""
    return 1 + dim + (dim * (dim + 1) // 2 if order >= 2 else 0) + (4 if order == 3 else 0)


def _field(j, name):
    v = getattr(j, name, None)
    return None if v is None else torch.as_tensor(v)


def pack_jet(j, dim: int, order: int, dtype, device) -> torch.Tensor:
    """A jet with value [n, F], grad [n, F, dim] (and hess [n, F, h]) as the
    device layout [n, C, F]."""
    v = _field(j, "value")
    g = _field(j, "grad")
    chans = [v, *[g[..., a] for a in range(dim)]]
    if order == 2:
        h = _field(j, "hess")
        if h is None:
            h = torch.zeros((*v.shape, dim * (dim + 1) // 2), dtype=v.dtype, device=v.device)
        chans += [h[..., k] for k in range(h.shape[-1])]
    return torch.stack([x.to(device=device, dtype=dtype) for x in chans], dim=1).contiguous()


def unpack_block(out: torch.Tensor, dim: int, order: int) -> Jet:
    """[B, n, C, F] -> Jet(value [B, n, F], grad [B, n, F, dim][, hess])."""
    value = out[:, :, 0]
    grad = out[:, :, 1:1 + dim].permute(0, 1, 3, 2)
    hess = out[:, :, 1 + dim:].permute(0, 1, 3, 2) if order == 2 else None
    return Jet(value, grad, hess=hess)


def pack_block(adj, dim: int, order: int, dtype, device) -> torch.Tensor:
    """Adjoint jet of a block (value [B, n, F], grad [B, n, F, dim] ...) ->
    [B, n, C, F]."""
    v = _field(adj, "value")
    g = _field(adj, "grad")
    chans = [v, *[g[..., a] for a in range(dim)]]
    if order == 2:
        h = _field(adj, "hess")
        chans += [h[..., k] for k in range(h.shape[-1])]
    return torch.stack([x.to(device=device, dtype=dtype) for x in chans], dim=2).contiguous()


@dataclass
class ModeTape:
    """Tape of one block of modes (scaled pre-activations and outputs of the
    hidden layers), with the block and the packed inputs it was made from."""
    buffer: torch.Tensor
    start: int
    stop: int
    features: torch.Tensor
    envelope: torch.Tensor | None


class ModeModel:
    """K per-mode SIREN networks with analytic spatial jets (the reference's
    Model API; first-order jets by default, ``order=2`` for the velocity
    objective's second derivatives)."""

    def __init__(self, c, K: int = 32, seed: int = 0, inputs: int = 15, outputs: int = 3,
                 dim: int = 3, order: int = 1, precision: str = "fp32",
                 device: str | torch.device = "cuda"):
        if precision not in ("fp32", "fp64", "tf32", "bf16x9"):
            raise ValueError("precision must be 'fp32', 'fp64', 'tf32' or 'bf16x9' (FP32 "
                             "parameters with the per-mode GEMMs on the tensor cores)")
        if dim not in (2, 3) or order not in (1, 2):
            raise ValueError("dim must be 2 or 3 and order 1 or 2")
        self.c, self.K, self.dim, self.order = c, K, dim, order
        self.precision = precision
        self.device = torch.device(device)
        self.dtype = torch.float64 if precision == "fp64" else torch.float32
        W, b = siren_init(c, K, seed, inputs, outputs)
        self.W = [torch.tensor(w, dtype=self.dtype, device=self.device) for w in W]
        self.b = [torch.tensor(x, dtype=self.dtype, device=self.device) for x in b]
        self.mW = [torch.zeros_like(w) for w in self.W]
        self.vW = [torch.zeros_like(w) for w in self.W]
        self.mb = [torch.zeros_like(x) for x in self.b]
        self.vb = [torch.zeros_like(x) for x in self.b]
        self._steps = torch.zeros((), dtype=torch.int32, device=self.device)
        widths = [inputs] + [c.hidden] * c.hidden_layers + [outputs]
        if len(widths) - 1 > N.MAX_HIDDEN + 1:
            raise ValueError(f"at most {N.MAX_HIDDEN + 1} layers")
        arr = (ctypes.c_int32 * (N.MAX_HIDDEN + 2))(*(widths + [0] * (N.MAX_HIDDEN + 2 - len(widths))))
        self.net = ModeNet(dim, order, len(widths) - 1, arr, K, N.PREC[precision],
                           float(c.siren_first_omega0), float(c.siren_hidden_omega0))
        self.widths = widths
        self._bufs: dict[str, torch.Tensor] = {}
        N.load()

    # --------------------------------------------------------------- helpers
    @property
    def epoch(self) -> int:
        """Committed optimizer steps (reads the device counter)."""
        return int(self._steps.item())

    @epoch.setter
    def epoch(self, value: int) -> None:
        self._steps.fill_(int(value))

    @property
    def storage_prec(self) -> int:
        """Precision code of the stored arrays (FP32 for the tensor-core forms)."""
        return N.PREC["fp64" if self.dtype == torch.float64 else "fp32"]

    @property
    def channels(self) -> int:
        return jet_channels(self.dim, self.order)

    def _buf(self, key: str, nbytes: int) -> torch.Tensor:
        nbytes = max(int(nbytes), 256)
        b = self._bufs.get(key)
        if b is None or b.numel() < nbytes:
            b = torch.empty(nbytes, dtype=torch.uint8, device=self.device)
            self._bufs[key] = b
        return b

    def _inputs(self, data):
        feats = data.features
        if not (isinstance(feats, torch.Tensor) and feats.dim() == 3):
            feats = pack_jet(feats, self.dim, self.order, self.dtype, self.device)
        env = getattr(data, "envelope", None)
        if env is not None and not (isinstance(env, torch.Tensor) and env.dim() == 3):
            env = pack_jet(env, self.dim, self.order, self.dtype, self.device)
        if env is not None and env.shape[2] != 1:
            raise ValueError("the envelope is one scalar jet per point")
        return feats.to(self.dtype).contiguous(), None if env is None else env.to(self.dtype).contiguous()

    # ------------------------------------------------- reference backend API
    def forward_packed(self, feats: torch.Tensor, env, start: int, stop: int, cache: bool = False):
        """Output jets [stop-start, n, C, outputs] of modes [start, stop) from
        packed inputs, and the tape (kept when ``cache``)."""
        n = feats.shape[0]
        B = stop - start
        C = jet_channels(self.net.dim, self.net.order)
        if C != self.channels or feats.shape[1] != C:
            raise ValueError(f"jets of {C} channels expected, features carry {feats.shape[1]}")
        lib = N.load()
        tb = lib.neb_modes_tape_bytes(ctypes.byref(self.net), B, n)
        tape = torch.empty(max(tb, 256), dtype=torch.uint8, device=self.device) if cache else \
            self._buf("tape", tb)
        out = torch.empty((B, n, self.channels, self.widths[-1]), dtype=self.dtype,
                          device=self.device)
        N.call("neb_modes_forward", ctypes.byref(self.net), start, stop, N.ptr_array(self.W),
               N.ptr_array(self.b), feats.data_ptr(), 0 if env is None else env.data_ptr(), n,
               tape.data_ptr(), tape.numel(), out.data_ptr(), _stream())
        return out, (ModeTape(tape, start, stop, feats, env) if cache else None)

    def forward_eval(self, feats: torch.Tensor, env, start: int, stop: int) -> torch.Tensor:
        """Output jets [stop-start, n, C, outputs] of modes [start, stop)
        without a tape (evaluation only: two alternating activation buffers)."""
        n = feats.shape[0]
        B = stop - start
        lib = N.load()
        scratch = self._buf("eval", lib.neb_modes_eval_scratch_bytes(ctypes.byref(self.net), B, n))
        out = torch.empty((B, n, self.channels, self.widths[-1]), dtype=self.dtype,
                          device=self.device)
        N.call("neb_modes_forward_eval", ctypes.byref(self.net), start, stop,
               N.ptr_array(self.W), N.ptr_array(self.b), feats.data_ptr(),
               0 if env is None else env.data_ptr(), n, scratch.data_ptr(), scratch.numel(),
               out.data_ptr(), _stream())
        return out

    def forward(self, data, start: int, stop: int, cache: bool = False):
        """(output jet of modes [start, stop) times the envelope, tape)."""
        feats, env = self._inputs(data)
        out, tape = self.forward_packed(feats, env, start, stop, cache)
        return unpack_block(out, self.dim, self.order), tape

    def backward_packed(self, tape: ModeTape, adj: torch.Tensor, gW=None, gb=None,
                        accumulate: bool = False):
        B = tape.stop - tape.start
        n = tape.features.shape[0]
        if adj.shape != (B, n, self.channels, self.widths[-1]):
            raise ValueError(f"adjoint shape {tuple(adj.shape)} does not match the block")
        if gW is None:
            gW = [torch.empty((B, *w.shape[1:]), dtype=self.dtype, device=self.device)
                  for w in self.W]
            gb = [torch.empty((B, *x.shape[1:]), dtype=self.dtype, device=self.device)
                  for x in self.b]
        lib = N.load()
        ws = self._buf("ws", lib.neb_modes_workspace_bytes(ctypes.byref(self.net), B, n))
        N.call("neb_modes_backward", ctypes.byref(self.net), tape.start, tape.stop,
               N.ptr_array(self.W), tape.features.data_ptr(),
               0 if tape.envelope is None else tape.envelope.data_ptr(), n,
               tape.buffer.data_ptr(), adj.contiguous().data_ptr(), N.ptr_array(gW),
               N.ptr_array(gb), int(accumulate), ws.data_ptr(), ws.numel(), _stream())
        return gW, gb

    def backward(self, data, start: int, stop: int, cache: ModeTape, adj):
        """Gradients (lists shaped [stop-start, ...]) of <adj, forward(...)>."""
        if cache is None or (cache.start, cache.stop) != (start, stop):
            raise ValueError("backward needs the tape of forward(data, start, stop, cache=True)")
        a = adj if isinstance(adj, torch.Tensor) and adj.dim() == 4 else \
            pack_block(adj, self.dim, self.order, self.dtype, self.device)
        return self.backward_packed(cache, a)

    def adam_async(self, gW, gb, lr: float, clip: float = 8.0, gate=None):
        """Per-mode Adam without a host synchronisation: device (norms [K],
        committed) tensors; the epoch counter advances on commit only.
        ``gate``: a device int status of the objective (the peel's ``info``);
        the update commits only when it is 0."""
        params = [*self.W, *self.b]
        grads = [g.to(self.dtype).contiguous() for g in [*gW, *gb]]
        for p, g in zip(params, grads):
            if p.shape != g.shape:
                raise ValueError(f"gradient shape {tuple(g.shape)} != parameter {tuple(p.shape)}")
        sizes = (ctypes.c_int64 * len(params))(*[p.numel() for p in params])
        norms = torch.empty(self.K, dtype=torch.float64, device=self.device)
        committed = torch.empty((), dtype=torch.int32, device=self.device)
        lib = N.load()
        ws = self._buf("adam", lib.neb_modes_adam_workspace_bytes(self.K))
        N.call("neb_modes_adam", 1 if self.dtype == torch.float64 else 0, self.K, len(params),
               N.ptr_array(params), N.ptr_array([*self.mW, *self.mb]),
               N.ptr_array([*self.vW, *self.vb]), N.ptr_array(grads), sizes,
               self._steps.data_ptr(), 0, 0, 0 if gate is None else gate.data_ptr(), lr, clip,
               norms.data_ptr(), committed.data_ptr(),
               ws.data_ptr(), ws.numel(), _stream())
        return norms, committed

    def adam(self, gW, gb, lr: float, clip: float = 8.0) -> torch.Tensor:
        """One Adam step with per-mode clipping; returns the per-mode norms.
        Raises FloatingPointError, with nothing changed, when any mode's
        gradient norm is not finite and positive."""
        norms, committed = self.adam_async(gW, gb, lr, clip)
        if not bool(committed.item()):
            raise FloatingPointError("Invalid parameter gradients; no optimizer update")
        return norms

    def save(self, path, configuration=None) -> None:
        arrays = {f"{name}_{j}": a.detach().cpu().numpy()
                  for name in ("W", "b", "mW", "vW", "mb", "vb")
                  for j, a in enumerate(getattr(self, name))}
        arrays["epoch"] = np.asarray(self.epoch)
        path = Path(path)
        tmp = path.with_suffix(".tmp.npz")
        np.savez(tmp, **arrays)
        tmp.replace(path)

    def load(self, path, configuration=None) -> None:
        with np.load(path) as z:
            self.epoch = int(z["epoch"])
            for name in ("W", "b", "mW", "vW", "mb", "vb"):
                for j, a in enumerate(getattr(self, name)):
                    a.copy_(torch.as_tensor(z[f"{name}_{j}"], dtype=self.dtype))


# ------------------------------------------------------ velocity objective
@dataclass
class PeelResult:
    losses: torch.Tensor       # [K] in causal order
    order: torch.Tensor        # [K] mode index of each causal rank
    T: torch.Tensor            # [K, K], rows in mode order
    Cu: torch.Tensor           # [K, K]: dL/dU = U Cu / n
    Cd: torch.Tensor           # [K, K]: dL/dD = D Cd / n
    relative_mass: torch.Tensor
    gram_max: torch.Tensor     # orthogonality error of the peeled basis
    info: torch.Tensor         # 0 ok, 1 rank (Cholesky), 2 gate


def coefficient_peel(M: torch.Tensor, S: torch.Tensor, check: bool = True,
                     mass_floor: float = 0.0, sort: bool = True) -> PeelResult:
    """Causal Rayleigh peel in Gram form on the device (velocity/core.py:48-69);
    ``check`` reads the status back and raises FloatingPointError where the
    reference's gate fails (``mass_floor`` > 0: the 2D peel's gate,
    hardcoded_backend.py:3555-3567, instead of velocity/core.py:60-62);
    ``sort`` False keeps the modes in network order (the 2D peel's
    fixed_order, hardcoded_backend.py:3471-3475)."""
    K = M.shape[0]
    dev = M.device
    M = M.to(torch.float64).contiguous()
    S = S.to(torch.float64).contiguous()
    f64 = dict(dtype=torch.float64, device=dev)
    r = PeelResult(torch.empty(K, **f64), torch.empty(K, dtype=torch.int32, device=dev),
                   torch.empty((K, K), **f64), torch.empty((K, K), **f64),
                   torch.empty((K, K), **f64), torch.empty(K, **f64), torch.empty((), **f64),
                   torch.zeros((), dtype=torch.int32, device=dev))
    lib = N.load()
    ws = torch.empty(max(lib.neb_peel_workspace_bytes(K), 256), dtype=torch.uint8, device=dev)
    N.call("neb_coefficient_peel", K, M.data_ptr(), S.data_ptr(), float(mass_floor), int(sort),
           r.losses.data_ptr(),
           r.order.data_ptr(), r.T.data_ptr(), r.Cu.data_ptr(), r.Cd.data_ptr(),
           r.relative_mass.data_ptr(), r.gram_max.data_ptr(), r.info.data_ptr(), ws.data_ptr(),
           ws.numel(), _stream())
    if check and int(r.info.item()) != 0:
        raise FloatingPointError("Velocity rank/relative mass/orthogonality gate failed before Adam")
    return r


def column_gram(A: torch.Tensor, scale: float, compensated: bool = True) -> torch.Tensor:
    """scale A^T A in FP64 for A [rows, K] (FP32 sums compensated)."""
    rows, K = A.shape
    lib = N.load()
    G = torch.empty((K, K), dtype=torch.float64, device=A.device)
    ws = torch.empty(max(lib.neb_column_gram_workspace_bytes(rows, K), 256), dtype=torch.uint8,
                     device=A.device)
    N.call("neb_column_gram", N.PREC["fp64" if A.dtype == torch.float64 else "fp32"], rows, K,
           A.data_ptr(), scale, int(compensated), G.data_ptr(), ws.data_ptr(), ws.numel(),
           _stream())
    return G


def column_apply(A: torch.Tensor, C: torch.Tensor, scale: float,
                 form: str | None = None) -> torch.Tensor:
    """scale A C (A [rows, K], C [K, K] FP64) in A's type: FP64 GEMM for
    FP64 A; for FP32 A, scale C split into two floats and FP32 GEMMs (on the
    tensor cores for ``form`` "tf32" / "bf16x9")."""
    rows, K = A.shape
    lib = N.load()
    out = torch.empty_like(A)
    ws = torch.empty(max(lib.neb_column_apply_workspace_bytes(rows, K), 256), dtype=torch.uint8,
                     device=A.device)
    code = N.PREC["fp64" if A.dtype == torch.float64 else
                  (form if form in ("tf32", "bf16x9") else "fp32")]
    N.call("neb_column_apply", code, rows, K,
           A.data_ptr(), C.to(torch.float64).contiguous().data_ptr(), scale, out.data_ptr(),
           ws.data_ptr(), ws.numel(), _stream())
    return out


def velocity_fields(model: ModeModel, data, block: int = 32, gradient: bool = True):
    """Velocity U [3n, K] (rows p*3 + a) and, with ``gradient``, its
    gradient D [9n, K] of every mode at the data's points: the evaluation
    of velocity/core.py:71-77 (fields), with the evaluation-only forward."""
    if model.dim != 3 or model.order != 2 or model.widths[-1] != 3:
        raise ValueError("velocity fields need a 3D second-order model with 3 outputs per mode")
    feats, env = model._inputs(data)
    n, K = feats.shape[0], model.K
    U = torch.empty((3 * n, K), dtype=model.dtype, device=model.device)
    D = torch.empty((9 * n, K), dtype=model.dtype, device=model.device)
    prec = model.storage_prec
    for a in range(0, K, block):
        b = min(K, a + block)
        out = model.forward_eval(feats, env, a, b)
        N.call("neb_velocity_fields", prec, out.data_ptr(), a, b, n, K, U.data_ptr(),
               D.data_ptr(), _stream())
    return (U, D) if gradient else U


def velocity_step(model: ModeModel, data, training: bool = True, block: int = 32,
                  check: bool = True) -> dict:
    """The 3D velocity objective of velocity/core.py:79-103 on a second-order
    mode network with three outputs (a vector potential per mode): U [3n, K]
    velocities and D [9n, K] velocity gradients, M = U^T U / n, S = D^T D / n
    in FP64, the Gram-form peel, and with ``training`` the parameter
    gradient of sum(losses), recomputing each block's activations in the
    reverse pass as the reference does."""
    if model.dim != 3 or model.order != 2 or model.widths[-1] != 3:
        raise ValueError("velocity_step needs a 3D second-order model with 3 outputs per mode")
    feats, env = model._inputs(data)
    n, K = feats.shape[0], model.K
    dt = model.dtype
    U = torch.empty((3 * n, K), dtype=dt, device=model.device)
    D = torch.empty((9 * n, K), dtype=dt, device=model.device)
    prec = model.storage_prec
    blocks = [(a, min(K, a + block)) for a in range(0, K, block)]
    for a, b in blocks:
        out, _ = model.forward_packed(feats, env, a, b)
        N.call("neb_velocity_fields", prec, out.data_ptr(), a, b, n, K, U.data_ptr(),
               D.data_ptr(), _stream())
    M = column_gram(U, 1.0 / n)
    S = column_gram(D, 1.0 / n)
    peel = coefficient_peel(M, S, check=check)
    res = dict(losses=peel.losses, order=peel.order, T=peel.T, Cu=peel.Cu, Cd=peel.Cd,
               relative_mass=peel.relative_mass, gram_max=peel.gram_max, info=peel.info,
               M=M, S=S)
    if training:
        gu = column_apply(U, peel.Cu, 1.0 / n, model.precision)
        gd = column_apply(D, peel.Cd, 1.0 / n, model.precision)
        gW = [torch.empty_like(w) for w in model.W]
        gb = [torch.empty_like(x) for x in model.b]
        for a, b in blocks:
            _, tape = model.forward_packed(feats, env, a, b, cache=True)
            adj = torch.empty((b - a, n, 10, 3), dtype=dt, device=model.device)
            N.call("neb_velocity_lift", prec, gu.data_ptr(), gd.data_ptr(), a, b, n, K,
                   adj.data_ptr(), _stream())
            model.backward_packed(tape, adj, [g[a:b] for g in gW], [g[a:b] for g in gb])
        res["grads"] = (gW, gb)
    return res
