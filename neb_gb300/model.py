"""Host side of the hot path: the network-backend API over the C ABI.

``Model`` keeps the method names and meaning of the reference's native
network backend (experiments/metaball/_backend/flow/cases/metaball/
native_cupy_core.py:111-185): ``W``/``b`` parameter lists, Adam moments
``mW, vW, mb, vb``, ``epoch``, ``forward(data, start, stop, cache)``,
``backward(data, start, stop, tape, adj)``, ``adam(gW, gb, lr, clip)``,
``save``/``load`` with the keys ``W_j, b_j, mW_j, vW_j, mb_j, vb_j, epoch``.
It differs in the network: one shared tanh MLP whose K outputs are the
modes, instead of K per-mode SIREN networks.

``spectral_step`` is the new entry of the hot path: features -> jet MLP ->
weighted Grams -> FP64 generalized eigensolve -> objective -> hand-written
reverse pass, with ``SpectralObjective`` as its ``torch.autograd.Function``.

All device memory comes from PyTorch; kernels run on the current CUDA stream.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass
from pathlib import Path

import numpy as np
import torch

from . import _native as N
from .configs import NebConfig, glorot_params, objective_weights
from .jets import Jet, pack, unpack


def _stream() -> int:
    return torch.cuda.current_stream().cuda_stream


class _Buffers:
    """Grow-only device byte buffers keyed by role."""

    def __init__(self, device):
        self.device = device
        self.bufs: dict[str, torch.Tensor] = {}

    def get(self, key: str, nbytes: int) -> torch.Tensor:
        nbytes = max(int(nbytes), 256)
        b = self.bufs.get(key)
        if b is None or b.numel() < nbytes:
            b = torch.empty(nbytes, dtype=torch.uint8, device=self.device)
            self.bufs[key] = b
        return b


@dataclass
class Tape:
    """Activation tape of one forward pass (inputs and pre-activations of
    every hidden layer, in the library's storage format)."""
    buffer: torch.Tensor
    n_points: int
    features: torch.Tensor


class Model:
    """Shared tanh MLP with analytic spatial jets (reference backend API)."""

    def __init__(self, cfg: NebConfig, K: int | None = None, seed: int = 0,
                 precision: str | None = None, device: str | torch.device = "cuda",
                 spectral: str | None = None, gram: str | None = None):
        # split-BF16 tensor cores for the 2D hidden-layer route; the 3D curl
        # fields take the direct route, which runs the FP32 kernels
        precision = precision or ("bf16x3" if cfg.dim == 2 else "fp32")
        if precision not in N.PREC:
            raise ValueError(f"precision must be one of {tuple(N.PREC)}")
        # spectral stage: "mixed" (compensated-FP32 Cholesky and reduction,
        # FP32 tridiagonalisation and tridiagonal eigenvectors, FP64
        # Rayleigh-quotient eigenvalues) or "fp64" (cuSOLVER sygvd); the FP64
        # form defaults to "fp64"
        # "range" (cuSOLVER syevd on M, FP64 finite pencil on range(M)) for
        # configurations whose mass matrix may be numerically singular
        if spectral is None:
            spectral = cfg.spectral if cfg.spectral == "range" else \
                ("fp64" if precision == "fp64" else "mixed")
        if spectral not in ("mixed", "fp64", "range"):
            raise ValueError("spectral must be 'mixed', 'fp64' or 'range'")
        self.spectral = spectral
        # range solves keep the eigen-directions of M above rank_rtol * max:
        # the tolerance at which the finite pencil is determined by the
        # fields to the working precision (RANK_RTOL)
        self.rank_rtol = RANK_RTOL[precision]
        if K is not None:
            cfg = cfg.scaled(outputs=K * (3 if cfg.dim == 3 else 1))
        self.c = cfg
        self.K = cfg.K
        self.precision = precision
        self.device = torch.device(device)
        self.dtype = torch.float64 if precision == "fp64" else torch.float32
        # committed Adam steps, kept on the device: the update advances it
        # only when it commits, so a rejected step on the asynchronous path
        # leaves the bias correction of every later step unchanged
        self._steps = torch.zeros((), dtype=torch.int32, device=self.device)
        self.W, self.b = [], []
        for W, b in glorot_params(cfg.widths, seed):
            self.W.append(torch.tensor(W, dtype=self.dtype, device=self.device))
            self.b.append(torch.tensor(b, dtype=self.dtype, device=self.device))
        self.mW = [torch.zeros_like(w) for w in self.W]
        self.vW = [torch.zeros_like(w) for w in self.W]
        self.mb = [torch.zeros_like(b) for b in self.b]
        self.vb = [torch.zeros_like(b) for b in self.b]
        # Gram accumulation of the FP32 form (FP64 sums in FP64, split-BF16
        # in tensor memory)
        self.gram = gram or (cfg.gram if precision in ("fp32", "tf32", "bf16x9") else "plain")
        self.net = N.NebNet.make(cfg.dim, cfg.widths, precision, self.gram)
        # the reference-API forward/backward evaluate output-layer jets, which
        # the tensor-core path does not store: they run the FP32 kernels
        self.net_eval = self.net if precision != "bf16x3" else \
            N.NebNet.make(cfg.dim, cfg.widths, "fp32", self.gram)
        self._buf = _Buffers(self.device)
        N.load()

    # ------------------------------------------------------------ helpers
    @property
    def epoch(self) -> int:
        """Committed optimizer steps (reads the device counter)."""
        return int(self._steps.item())

    @epoch.setter
    def epoch(self, value: int) -> None:
        self._steps.fill_(int(value))

    @property
    def channels(self) -> int:
        return 4 if self.c.dim == 2 else 10

    @property
    def n_hidden(self) -> int:
        return len(self.c.widths) - 2

    def parameters(self):
        return [*self.W, *self.b]

    def set_parameters(self, params) -> None:
        """Load (W, b) pairs (float64 arrays or tensors) into the masters."""
        for j, (W, b) in enumerate(params):
            self.W[j].copy_(torch.as_tensor(np.asarray(W), dtype=self.dtype))
            self.b[j].copy_(torch.as_tensor(np.asarray(b), dtype=self.dtype))

    def _ws(self, n: int, net=None) -> torch.Tensor:
        net = self.net if net is None else net
        key = "ws" if net is self.net else "ws_eval"
        return self._buf.get(key, N.load().neb_workspace_bytes(ctypes.byref(net), n))

    def features(self, points) -> torch.Tensor:
        """Input feature jets [n, C, F] (device, master dtype) of points [n, dim]."""
        pts = _to_device(points, torch.float64, self.device).contiguous()
        if pts.ndim != 2 or pts.shape[1] != self.c.dim:
            raise ValueError(f"points must be [n, {self.c.dim}]")
        n = pts.shape[0]
        out = torch.empty((n, self.channels, self.c.widths[0]), dtype=self.dtype, device=self.device)
        prm = self.c.feature_params()
        arr = (ctypes.c_double * max(len(prm), 1))(*prm)
        N.call("neb_features", ctypes.byref(self.net), N.FEAT[self.c.features], self.c.n_freq, arr,
               len(prm), pts.data_ptr(), n, out.data_ptr(), _stream())
        return out

    def run_forward(self, feats: torch.Tensor, net=None) -> Tape:
        """Hidden layers over packed feature jets; returns the tape."""
        net = self.net if net is None else net
        feats = feats.to(self.dtype).contiguous()
        n = feats.shape[0]
        key = "tape" if net is self.net else "tape_eval"
        tape = self._buf.get(key, N.load().neb_tape_bytes(ctypes.byref(net), n))
        ws = self._ws(n, net)
        N.call("neb_forward", ctypes.byref(net), N.ptr_array(self.W), N.ptr_array(self.b),
               feats.data_ptr(), n, tape.data_ptr(), ws.data_ptr(), ws.numel(), _stream())
        return Tape(tape, n, feats)

    def check_device_status(self, n: int) -> None:
        """Raise if a bounded device-side wait gave up during this step."""
        ws = self._ws(n)
        N.call("neb_check_status", ctypes.byref(self.net), n, ws.data_ptr(), ws.numel(),
               _stream())

    def output(self, tape: Tape, start: int = 0, stop: int | None = None) -> torch.Tensor:
        stop = self.c.widths[-1] if stop is None else stop
        psi = torch.empty((tape.n_points, self.channels, stop - start), dtype=self.dtype,
                          device=self.device)
        N.call("neb_output", ctypes.byref(self.net_eval), self.W[-1].data_ptr(),
               self.b[-1].data_ptr(), start, stop, tape.n_points, tape.buffer.data_ptr(),
               psi.data_ptr(), _stream())
        return psi

    # ------------------------------------------------- reference backend API
    def forward(self, data, start: int = 0, stop: int | None = None, cache: bool = False):
        """Output jets of outputs [start, stop) at ``data.features``.

        ``data.features``: a :class:`Jet` or a packed [n, C, F] tensor;
        ``data.envelope`` (optional): a scalar :class:`Jet` per point or a
        packed [n, C] tensor; the output jets are multiplied by it
        (native_cupy_core.py:139 product1).  Returns ``(field_jet, tape)``;
        the tape is None unless ``cache``."""
        feats = data.features
        feats = pack(feats, self.c.dim).to(self.device, self.dtype) if isinstance(feats, Jet) else feats
        tape = self.run_forward(feats, self.net_eval)
        if cache:  # keep this tape: later calls must not overwrite it
            tape = Tape(tape.buffer.clone(), tape.n_points, tape.features)
        psi = self.output(tape, start, stop)
        env = self._envelope(data, tape.n_points)
        if env is not None:
            out = torch.empty_like(psi)
            N.call("neb_envelope_product", ctypes.byref(self.net_eval), env.data_ptr(),
                   tape.n_points, psi.shape[2], psi.data_ptr(), out.data_ptr(), 0, _stream())
            psi = out
        return unpack(psi, self.c.dim), (tape if cache else None)

    def _envelope(self, data, n: int):
        """The envelope of ``data`` as a packed [n, C] device tensor, or None."""
        env = getattr(data, "envelope", None)
        if env is None:
            return None
        if isinstance(env, Jet):
            env = pack(env, self.c.dim)
        env = torch.as_tensor(env).to(self.device, self.dtype).reshape(n, self.channels)
        return env.contiguous()

    def backward(self, data, start: int, stop: int | None, tape: Tape, adj):
        """Parameter gradients of <adj, forward(data, start, stop)> (lists of
        tensors shaped like ``W`` and ``b``; output rows outside [start, stop)
        are zero)."""
        stop = self.c.widths[-1] if stop is None else stop
        pb = pack(adj, self.c.dim).to(self.device, self.dtype).contiguous() \
            if isinstance(adj, Jet) else adj.to(self.dtype).contiguous()
        if pb.shape != (tape.n_points, self.channels, stop - start):
            raise ValueError(f"adjoint shape {tuple(pb.shape)} does not match the outputs")
        env = self._envelope(data, tape.n_points)
        if env is not None:  # adjoint of the raw outputs (envelope_product_backward_jet1)
            raw = torch.empty_like(pb)
            N.call("neb_envelope_product", ctypes.byref(self.net_eval), env.data_ptr(),
                   tape.n_points, pb.shape[2], pb.data_ptr(), raw.data_ptr(), 1, _stream())
            pb = raw
        gW = [torch.zeros_like(w) for w in self.W]
        gb = [torch.zeros_like(b) for b in self.b]
        ws = self._ws(tape.n_points, self.net_eval)
        N.call("neb_backward_output", ctypes.byref(self.net_eval), N.ptr_array(self.W), start, stop,
               pb.data_ptr(), tape.n_points, tape.buffer.data_ptr(), N.ptr_array(gW),
               N.ptr_array(gb), 0, ws.data_ptr(), ws.numel(), _stream())
        return gW, gb

    def adam(self, gW, gb, lr: float, clip: float = 8.0, beta1: float = 0.9,
             beta2: float = 0.999, eps: float = 1e-8) -> float:
        """One Adam transaction with global-norm clipping.  Raises
        FloatingPointError, with nothing changed, when a gradient is not
        finite or the norm is zero."""
        norm, committed = self.adam_async(gW, gb, lr, clip, beta1, beta2, eps)
        if not bool(committed.item()):
            raise FloatingPointError("Invalid parameter gradients; no optimizer update")
        return float(norm.item())

    def adam_async(self, gW, gb, lr, clip=8.0, beta1=0.9, beta2=0.999, eps=1e-8, gate=None):
        """Adam without a host synchronisation: returns device (norm,
        committed) tensors.  The step counter on the device advances only
        when the update commits (the caller checks ``committed``).  ``gate``:
        a device int status of the objective (e.g. ``SpectralResult.info``);
        the update commits only when it is 0."""
        params = [*self.W, *self.b]
        grads = [g.to(self.dtype).contiguous() for g in [*gW, *gb]]
        for p, g in zip(params, grads):
            if p.shape != g.shape:
                raise ValueError(f"gradient shape {tuple(g.shape)} != parameter {tuple(p.shape)}")
        sizes = (ctypes.c_int64 * len(params))(*[p.numel() for p in params])
        norm = torch.empty((), dtype=torch.float64, device=self.device)
        committed = torch.empty((), dtype=torch.int32, device=self.device)
        ws = self._buf.get("adam", N.load().neb_adam_workspace_bytes())
        N.call("neb_adam", 1 if self.dtype == torch.float64 else 0, len(params),
               N.ptr_array(params), N.ptr_array([*self.mW, *self.mb]),
               N.ptr_array([*self.vW, *self.vb]), N.ptr_array(grads), sizes, 0,
               self._steps.data_ptr(), 0 if gate is None else gate.data_ptr(), lr, clip,
               beta1, beta2, eps, norm.data_ptr(),
               committed.data_ptr(), ws.data_ptr(), ws.numel(), _stream())
        return norm, committed

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


# ----------------------------------------------------------------- spectral
@dataclass
class SpectralResult:
    loss: torch.Tensor            # device scalar (FP64)
    eigenvalues: torch.Tensor     # [m] FP64, ascending
    eigenvectors: torch.Tensor    # [m][m] FP64, row k = eigenvector k (pencil coordinates)
    rank: int                     # number of finite eigenpairs (dimension of range(M))
    info: torch.Tensor            # device int: solver status
    grads: tuple | None = None    # (gW list, gb list) when training
    M: torch.Tensor | None = None
    S: torch.Tensor | None = None
    A_M: torch.Tensor | None = None
    A_S: torch.Tensor | None = None
    chunks: int = 1               # point chunks (the reverse pass recomputes all but the last)


class SpectralState:
    """Per-model FP64 buffers of the spectral stage."""

    def __init__(self, model: Model):
        self.model = model
        self.buf = _Buffers(model.device)
        self._weights = {}

    def objective_weights(self, kind: str, m: int):
        """c_k on the device, copied from the host once per (objective, m): a
        per-step copy from pageable host memory would make the host wait for
        the stream to drain, leaving the GPU idle while the rest of the step
        is enqueued."""
        key = (kind, m)
        if key not in self._weights:
            self._weights[key] = torch.as_tensor(objective_weights(kind, m), dtype=torch.float64,
                                                 device=self.model.device)
        return self._weights[key]


def _to_device(x, dtype, device) -> torch.Tensor:
    """Host arrays and tensors to the device; a pinned host tensor is copied
    asynchronously on the current stream (the host does not wait for it)."""
    if isinstance(x, torch.Tensor) and x.device.type == "cpu" and x.is_pinned():
        return x.to(device=device, dtype=dtype, non_blocking=True)
    return torch.as_tensor(x, dtype=dtype, device=device)


def _f64(shape, device):
    return torch.empty(shape, dtype=torch.float64, device=device)


def _solve(model: Model, m: int, PM, PS, kind: str):
    """Spectral stage on the m x m pencil (PS, PM): eigenpairs, objective
    and its Gram adjoints, all on the device."""
    lib = N.load()
    dev = model.device
    st = getattr(model, "_spectral", None) or SpectralState(model)
    model._spectral = st
    c = st.objective_weights(kind, m)
    lam, V, GM, GS = _f64((m,), dev), _f64((m, m), dev), _f64((m, m), dev), _f64((m, m), dev)
    loss = _f64((), dev)
    info = torch.zeros((), dtype=torch.int32, device=dev)
    mixed_bytes = lib.neb_spectral_mixed_workspace_bytes(m) if model.spectral == "mixed" else 0
    name = "neb_spectral_mixed" if mixed_bytes else "neb_spectral"
    sws = st.buf.get(name, mixed_bytes or lib.neb_spectral_workspace_bytes(m))
    N.call(name, m, PM.data_ptr(), PS.data_ptr(), c.data_ptr(), lam.data_ptr(),
           V.data_ptr(), GM.data_ptr(), GS.data_ptr(), loss.data_ptr(), info.data_ptr(),
           sws.data_ptr(), sws.numel(), _stream())
    return loss, lam, V, GM, GS, info


# Rank tolerance of the range solve (the eigenvalue-ratio test of
# experiments/periodic/paper_rollout.py:180-186) per working precision.  The
# raw-coordinate bases are nearly dependent at init: the mass Gram's
# eigenvalues fall smoothly over ten decades, and a direction with e / e_max
# = tau carries its eigenvalue and its share of the gradient with a condition
# number growing like tau^-1/2 and faster.  Below a precision's tolerance the
# finite pencil is set by rounding rather than by the fields: FP64 resolves
# 1e-10; the FP32 form (compensated Grams, FP32 activations, FP32 Gram
# adjoints) 1e-5; split-BF16 (16-bit activations, FP32 accumulation in
# tensor memory) 1e-4.  The FP64 oracle solves the same pencil at the same
# tolerance, and the ranks agree.
# tf32: one pass of 10-bit TF32 inputs in the layer GEMMs; bf16x9: the
# BF16x9 emulation of FP32 products (FP32-class accuracy)
RANK_RTOL = {"fp64": 1e-10, "fp32": 1e-5, "bf16x3": 1e-4, "tf32": 1e-4, "bf16x9": 1e-5}


def _solve_range(model: Model, m: int, PM, PS, kind: str, rank_rtol: float = 1e-10):
    """FP64 finite pencil of a possibly singular M (rank from the eigenvalue
    ratio test); returns the r finite pairs.  Reads the rank back (one
    stream synchronisation)."""
    lib = N.load()
    dev = model.device
    st = getattr(model, "_spectral", None) or SpectralState(model)
    model._spectral = st
    c = st.objective_weights(kind, m)
    lam, V, GM, GS = _f64((m,), dev), _f64((m, m), dev), _f64((m, m), dev), _f64((m, m), dev)
    loss = _f64((), dev)
    info = torch.zeros((), dtype=torch.int32, device=dev)
    rank = ctypes.c_int(0)
    sws = st.buf.get("range", lib.neb_spectral_range_workspace_bytes(m))
    N.call("neb_spectral_range", m, PM.data_ptr(), PS.data_ptr(), c.data_ptr(), rank_rtol,
           lam.data_ptr(), V.data_ptr(), GM.data_ptr(), GS.data_ptr(), loss.data_ptr(),
           ctypes.byref(rank), info.data_ptr(), sws.data_ptr(), sws.numel(), _stream())
    r = rank.value
    return loss, lam[:r], V[:r], GM, GS, info, r


def _raise_on_info(info) -> None:
    code = int(info.item())
    if code != 0:
        raise FloatingPointError(
            f"spectral stage failed (info={code}): the mass matrix is not positive definite "
            "or the eigensolver did not converge; no update")


def spectral_step(model: Model, points=None, weights=None, training: bool = True,
                  objective: str | None = None, return_grams: bool = False,
                  features: torch.Tensor | None = None, check: bool = True,
                  route: str | None = None, chunk_points: int | None = None) -> SpectralResult:
    """One objective (+ gradient) evaluation of the eigenfluid basis.

    points [n, dim] and weights [n] (host arrays or device tensors), or
    ``features`` (packed jets) with ``weights``.

    route "factored" (the 2D default): the hidden-layer pencil A_M, A_S
    (H x H) from the last hidden layer, and M = W_out A_M W_out^T,
    S = W_out A_S W_out^T.  When K >= H the finite eigenvalues of (S, M) are
    those of (A_S, A_M) (the K fields span the H hidden fields); otherwise
    the K x K pencil is solved.

    route "direct" (the 3D default, FP32 / FP64 networks): the K x K Grams of
    the velocity and vorticity fields of every mode, accumulated over point
    chunks of ``chunk_points``; the reverse pass recomputes each chunk's
    activations instead of keeping them (velocity/core.py:88-99).  The
    pencil is solved in FP64 on range(M) (rank from the eigenvalue ratio
    test, ``model.rank_rtol``), so a mass matrix whose fields are nearly dependent
    gives the r finite eigenvalues rather than noise; ``rank`` reports r.

    ``check`` reads the solver status back (one 4-byte D2H) and raises
    FloatingPointError.
    """
    cfg = model.c
    route = route or ("factored" if cfg.dim == 2 else "direct")
    if route == "direct":
        return _spectral_step_direct(model, points, weights, training, objective, return_grams,
                                     features, check, chunk_points)
    if route != "factored":
        raise ValueError("route must be 'factored' or 'direct'")
    if cfg.dim != 2:
        raise ValueError("the factored route is the 2D scalar-potential route")
    kind = objective or cfg.objective
    dev = model.device
    feats = model.features(points) if features is None else features
    qw = _to_device(weights, model.dtype, dev).contiguous()
    n = feats.shape[0]
    if qw.shape != (n,):
        raise ValueError("weights must be [n]")
    lib = N.load()
    st = getattr(model, "_spectral", None) or SpectralState(model)
    model._spectral = st
    s = _stream()
    H, K = cfg.hidden, cfg.widths[-1]
    # point chunks: one chunk while the activation tape of all n points fits
    # the budget; otherwise the Grams accumulate chunk by chunk and the
    # reverse pass recomputes each chunk's activations (the last chunk's are
    # still resident and are used first)
    chunk = int(chunk_points) if chunk_points else _factored_chunk(model, n)
    if chunk <= 0:
        raise ValueError("chunk_points must be positive")
    bounds = [(a, min(n, a + chunk)) for a in range(0, n, chunk)]
    AM, AS = _f64((H, H), dev), _f64((H, H), dev)
    for i, (a, b) in enumerate(bounds):
        tape = model.run_forward(feats[a:b] if len(bounds) > 1 else feats)
        ws = model._ws(b - a)
        N.call("neb_hidden_gram", ctypes.byref(model.net), qw[a:b].data_ptr(), b - a,
               tape.buffer.data_ptr(), AM.data_ptr(), AS.data_ptr(), int(i > 0), ws.data_ptr(),
               ws.numel(), s)
    Wout = model.W[-1].to(torch.float64).contiguous()
    pws = st.buf.get("pencil", lib.neb_pencil_workspace_bytes(K, H))
    M = S = None
    if K < H or return_grams:
        M, S = _f64((K, K), dev), _f64((K, K), dev)
        N.call("neb_pencil_project", K, H, Wout.data_ptr(), AM.data_ptr(), AS.data_ptr(),
               M.data_ptr(), S.data_ptr(), pws.data_ptr(), pws.numel(), s)
    if K >= H:
        m, PM, PS = H, AM, AS
    else:
        m, PM, PS = K, M, S
    if model.spectral == "range":
        loss, lam, V, GM, GS, info, r = _solve_range(model, m, PM, PS, kind, model.rank_rtol)
    else:
        loss, lam, V, GM, GS, info = _solve(model, m, PM, PS, kind)
        r = m
    res = SpectralResult(loss, lam, V, r, info, M=M, S=S, A_M=AM, A_S=AS)
    if training:
        L = model.n_hidden
        gW = [torch.empty_like(w) for w in model.W]
        gb = [torch.empty_like(b) for b in model.b]
        if K >= H:
            GMh, GSh = GM, GS
            gW[L].zero_()
        else:
            GMh, GSh = _f64((H, H), dev), _f64((H, H), dev)
            gWo = _f64((K, H), dev)
            N.call("neb_pencil_pullback", K, H, Wout.data_ptr(), AM.data_ptr(), AS.data_ptr(),
                   GM.data_ptr(), GS.data_ptr(), GMh.data_ptr(), GSh.data_ptr(), gWo.data_ptr(),
                   pws.data_ptr(), pws.numel(), s)
            gW[L].copy_(gWo)
        gb[L].zero_()
        for i, (a, b) in enumerate(reversed(bounds)):
            if i > 0:  # recompute this chunk's activations
                tape = model.run_forward(feats[a:b])
            ws = model._ws(b - a)
            N.call("neb_backward_hidden", ctypes.byref(model.net), N.ptr_array(model.W),
                   GMh.data_ptr(), GSh.data_ptr(), qw[a:b].data_ptr(), b - a,
                   tape.buffer.data_ptr(), N.ptr_array(gW[:L]), N.ptr_array(gb[:L]), int(i > 0),
                   ws.data_ptr(), ws.numel(), s)
        res.chunks = len(bounds)
        res.grads = (gW, gb)
    if check:
        model.check_device_status(n)
        _raise_on_info(info)
    return res


DEFAULT_CHUNK_POINTS = 1 << 17
# activation tape one chunk of the factored route may hold (bytes)
FACTORED_TAPE_BUDGET = 32 << 30


def _factored_chunk(model: Model, n: int) -> int:
    """Points per chunk of the factored route: all n while their tape fits
    FACTORED_TAPE_BUDGET, else the largest multiple of 128 that does."""
    lib = N.load()
    per = lib.neb_tape_bytes(ctypes.byref(model.net), n)
    if per <= FACTORED_TAPE_BUDGET:
        return n
    return max(128, int(n * FACTORED_TAPE_BUDGET / per) // 128 * 128)


def _spectral_step_direct(model: Model, points, weights, training, objective, return_grams,
                          features, check, chunk_points) -> SpectralResult:
    cfg = model.c
    if model.precision == "bf16x3":
        raise NotImplementedError(
            "the direct (field-Gram) route runs the FP32 or FP64 kernels: build the Model with "
            "precision='fp32' or 'fp64'")
    kind = objective or cfg.objective
    dev = model.device
    n = int(features.shape[0]) if features is not None else len(points)
    qw = _to_device(weights, model.dtype, dev).contiguous()
    if qw.shape != (n,):
        raise ValueError("weights must be [n]")
    chunk = int(chunk_points or DEFAULT_CHUNK_POINTS)
    if chunk <= 0:
        raise ValueError("chunk_points must be positive")
    bounds = [(a, min(n, a + chunk)) for a in range(0, n, chunk)]
    K = model.K
    s = _stream()

    def forward_chunk(a, b):
        feats = features[a:b] if features is not None else model.features(points[a:b])
        return model.run_forward(feats)

    M, S = _f64((K, K), dev), _f64((K, K), dev)
    tape = None
    for i, (a, b) in enumerate(bounds):
        tape = forward_chunk(a, b)
        ws = model._ws(b - a)
        N.call("neb_fields_gram", ctypes.byref(model.net), model.W[-1].data_ptr(),
               qw[a:b].data_ptr(), b - a, tape.buffer.data_ptr(), M.data_ptr(), S.data_ptr(),
               int(i > 0), ws.data_ptr(), ws.numel(), s)
    loss, lam, V, GM, GS, info, r = _solve_range(model, K, M, S, kind, model.rank_rtol)
    res = SpectralResult(loss, lam, V, r, info, M=M, S=S)
    if training:
        gW = [torch.empty_like(w) for w in model.W]
        gb = [torch.empty_like(b) for b in model.b]
        for i, (a, b) in enumerate(bounds):
            if len(bounds) > 1:  # recompute this chunk's activations
                tape = forward_chunk(a, b)
            ws = model._ws(b - a)
            N.call("neb_backward_fields", ctypes.byref(model.net), N.ptr_array(model.W),
                   GM.data_ptr(), GS.data_ptr(), qw[a:b].data_ptr(), b - a,
                   tape.buffer.data_ptr(), N.ptr_array(gW), N.ptr_array(gb), int(i > 0),
                   ws.data_ptr(), ws.numel(), s)
        res.grads = (gW, gb)
    if check:
        _raise_on_info(info)
    return res


def train_step(model: Model, points, weights, lr: float | None = None,
               clip: float | None = None, check: bool = True) -> SpectralResult:
    """spectral_step + Adam (one optimizer update)."""
    res = spectral_step(model, points, weights, training=True, check=check)
    gW, gb = res.grads
    lr = model.c.lr if lr is None else lr
    clip = model.c.clip if clip is None else clip
    if check:
        model.adam(gW, gb, lr, clip)
    else:
        # the solver status gates the update on the device: a failed
        # eigensolve commits nothing
        model.adam_async(gW, gb, lr, clip, gate=res.info)
    return res


class SpectralObjective(torch.autograd.Function):
    """loss = sum_k c_k lam_k(S, M) as an autograd node over the parameters.

    ``SpectralObjective.apply(model, features, weights, *model.parameters())``
    returns the FP64 loss; its backward is the library's hand-written reverse
    pass (no autograd tape of the forward)."""

    @staticmethod
    def forward(ctx, model, features, weights, *params):
        res = spectral_step(model, features=features, weights=weights, training=True)
        gW, gb = res.grads
        ctx.save_for_backward(*gW, *gb)
        return res.loss.clone()

    @staticmethod
    def backward(ctx, grad_out):
        grads = ctx.saved_tensors
        return (None, None, None, *[g * grad_out.to(g.dtype) for g in grads])
