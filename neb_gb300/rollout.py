"""Periodic evaluation of a trained per-mode basis on the GPU.

The reference's frozen-basis evaluation (experiments/periodic/
paper_rollout.py; the Jet3 field sampling of experiments/2d/_backend/
periodic_core/vortex_merger/canonical_gauge/scripts/
evaluate_large_comparison.py:16-39) in three stages:

* ``sample_basis``: third-order jets of every mode of a ``HardcodedModel``
  on the n x n grid, reduced to the fields the rollout needs -- velocity
  (u, v) = (psi_y, -psi_x) and vorticity -lap psi -- and, on request, the
  diagnostic channels (psi, -lap u, -lap v);
* ``ritz``: the unit-velocity normalisation and the Ritz stage (FP64 Grams,
  the full-rank gate on the mass matrix, the generalized eigenproblem),
  kept as one K x K transform R instead of rotated fields;
* ``Rollout``: the matrix-free Galerkin ETDRK4 integration in the Ritz basis
  (one step captured as a CUDA graph and replayed), the initial projection,
  the frame schedule of the reference and the reconstruction of fields.

Every computation runs in the library's kernels (``neb_periodic_features``,
``neb_modes_forward``, ``neb_stream_fields``, ``neb_column_gram``,
``neb_normalize_pencil``, ``neb_spectral_range``, ``neb_ritz_transform``,
``neb_etdrk4_*``, ``neb_rollout_*``); PyTorch provides memory and streams.
"""
from __future__ import annotations

import ctypes
import math
from dataclasses import dataclass

import numpy as np
import torch

from . import _native as N
from .hardcoded import HardcodedModel, TAPE_BUDGET
from .modes import column_gram


def _stream() -> int:
    return torch.cuda.current_stream().cuda_stream


def grid_points(n: int, cfg) -> np.ndarray:
    """The n x n evaluation grid of the reference (x fastest, as
    ``np.meshgrid(axis, axis)`` with axis = xmin + i L / n)."""
    ax = cfg.xmin + np.arange(n) * (cfg.xmax - cfg.xmin) / n
    ay = cfg.ymin + np.arange(n) * (cfg.ymax - cfg.ymin) / n
    x, y = np.meshgrid(ax, ay, indexing="xy")
    return np.column_stack((x.ravel(), y.ravel()))


@dataclass
class GridBasis:
    """Fields of K modes at n points: UV [n][2][K] (u, v), Om [n][K]
    (omega), diag [n][3][K] (psi, -lap u, -lap v) or None; quadrature
    weight per point."""
    UV: torch.Tensor
    Om: torch.Tensor
    diag: torch.Tensor | None
    weight: float
    precision: str

    @property
    def n(self) -> int:
        return self.Om.shape[0]

    @property
    def K(self) -> int:
        return self.Om.shape[1]


def sample_basis(model: HardcodedModel, cfg, grid: int, diagnostics: bool = False,
                 points=None, weight: float | None = None) -> GridBasis:
    """Third-order jets of every mode on the grid x grid points (or on the
    given points with the given quadrature weight) and their fields."""
    core = model.core
    if points is None:
        points = grid_points(grid, cfg)
        weight = float((cfg.xmax - cfg.xmin) * (cfg.ymax - cfg.ymin)) / (grid * grid)
    elif weight is None:
        raise ValueError("weight is required with explicit points")
    n, K = len(points), core.K
    feats = model.features(cfg, points, 3)
    dt = core.dtype
    UV = torch.empty((n, 2, K), dtype=dt, device=core.device)
    Om = torch.empty((n, K), dtype=dt, device=core.device)
    diag = torch.empty((n, 3, K), dtype=dt, device=core.device) if diagnostics else None
    net3 = model._net(3)
    lib = N.load()
    per_mode = max(1, lib.neb_modes_tape_bytes(ctypes.byref(net3), 1, n))
    block = max(1, min(K, TAPE_BUDGET // per_mode))
    prec = core.storage_prec
    with model._order(3):
        for a in range(0, K, block):
            b = min(K, a + block)
            out, _ = core.forward_packed(feats, None, a, b)
            N.call("neb_stream_fields", prec, 3, out.data_ptr(), a, b, n, K, UV.data_ptr(),
                   Om.data_ptr(), 0 if diag is None else diag.data_ptr(), _stream())
    return GridBasis(UV, Om, diag, float(weight), "fp64" if dt == torch.float64 else "fp32")


@dataclass
class RitzBasis:
    """lam [K] ascending Ritz values (FP64), R [K][K] = D^-1 T mapping Ritz
    coefficients to raw-field coefficients, norm [K] velocity norms."""
    lam: torch.Tensor
    R: torch.Tensor
    norm: torch.Tensor
    rank: int
    pair: torch.Tensor  # [2][K][K]: R and R^T, what the rollout kernels take


def ritz(basis: GridBasis, rank_rtol: float = 1e-12) -> RitzBasis:
    """Normalisation and Ritz stage (paper_rollout.py:171-192): velocity
    norms of the modes, M = w (U^T U + V^T V) and S = w W^T W in FP64 on the
    normalised modes, the full-rank gate (ArithmeticError when any
    eigenvalue of M is at or below rank_rtol of the largest), eigh(S, M)."""
    K, n, dev = basis.K, basis.n, basis.Om.device
    M = column_gram(basis.UV.reshape(2 * n, K), basis.weight)
    S = column_gram(basis.Om, basis.weight)
    f64 = dict(dtype=torch.float64, device=dev)
    norm = torch.empty(K, **f64)
    N.call("neb_normalize_pencil", K, M.data_ptr(), S.data_ptr(), norm.data_ptr(), _stream())
    lam, V = torch.empty(K, **f64), torch.empty((K, K), **f64)
    GM, GS = torch.empty((K, K), **f64), torch.empty((K, K), **f64)
    c, loss = torch.zeros(K, **f64), torch.empty((), **f64)
    info = torch.zeros((), dtype=torch.int32, device=dev)
    rank = ctypes.c_int(0)
    lib = N.load()
    ws = torch.empty(max(lib.neb_spectral_range_workspace_bytes(K), 256), dtype=torch.uint8,
                     device=dev)
    N.call("neb_spectral_range", K, M.data_ptr(), S.data_ptr(), c.data_ptr(), rank_rtol,
           lam.data_ptr(), V.data_ptr(), GM.data_ptr(), GS.data_ptr(), loss.data_ptr(),
           ctypes.byref(rank), info.data_ptr(), ws.data_ptr(), ws.numel(), _stream())
    if rank.value != K:
        raise ArithmeticError(f"Full-K rank gate: the mass matrix resolves {rank.value}/{K}")
    if int(info.item()) != 0:
        raise ArithmeticError(f"Ritz stage failed (status {int(info.item())})")
    RR = torch.empty((2, K, K), **f64)  # R and its transpose
    N.call("neb_ritz_transform", K, V.data_ptr(), norm.data_ptr(), RR.data_ptr(), _stream())
    return RitzBasis(lam, RR[0], norm, rank.value, RR)


class Rollout:
    """Matrix-free Galerkin ETDRK4 in the Ritz basis (paper_rollout.py:31-79)
    with viscosity nu: d c / dt = -nu lam c + rhs(c)."""

    def __init__(self, basis: GridBasis, ritz_basis: RitzBasis, nu: float,
                 use_graph: bool = True):
        self.basis, self.ritz, self.nu = basis, ritz_basis, float(nu)
        self.K, self.n = basis.K, basis.n
        dev = basis.Om.device
        lib = N.load()
        self.ws = torch.empty(max(lib.neb_rollout_workspace_bytes(self.n, self.K), 256),
                              dtype=torch.uint8, device=dev)
        self.c = torch.zeros(self.K, dtype=torch.float64, device=dev)
        self.coef = torch.zeros((6, self.K), dtype=torch.float64, device=dev)
        self.prec = N.PREC["fp64" if basis.Om.dtype == torch.float64 else "fp32"]
        self.h = None
        self.use_graph = use_graph
        self._graph = None

    # ------------------------------------------------------------- primitives
    def _args(self):
        b = self.basis
        return (self.prec, self.n, self.K, b.UV.data_ptr(), b.Om.data_ptr(),
                self.ritz.pair.data_ptr(), b.weight)

    def rhs(self, x: torch.Tensor) -> torch.Tensor:
        """The Galerkin right-hand side of Ritz coefficients x (FP64)."""
        x = x.to(torch.float64).contiguous()
        out = torch.empty_like(x)
        N.call("neb_rollout_rhs", *self._args(), x.data_ptr(), out.data_ptr(),
               self.ws.data_ptr(), self.ws.numel(), _stream())
        return out

    def project(self, u0, v0) -> torch.Tensor:
        """Ritz coefficients of the velocity field (u0, v0) at the points:
        c = w (gu^T u0 + gv^T v0) (paper_rollout.py:197)."""
        dev = self.c.device
        u = torch.as_tensor(np.asarray(u0, dtype=np.float64).ravel(), device=dev)
        v = torch.as_tensor(np.asarray(v0, dtype=np.float64).ravel(), device=dev)
        out = torch.empty(self.K, dtype=torch.float64, device=dev)
        b = self.basis
        N.call("neb_rollout_project", self.prec, self.n, self.K, b.UV.data_ptr(),
               self.ritz.pair.data_ptr(), u.data_ptr(), v.data_ptr(), b.weight, out.data_ptr(),
               self.ws.data_ptr(), self.ws.numel(), _stream())
        return out

    def fields(self, c: torch.Tensor) -> torch.Tensor:
        """(u, v, omega) [3][n] of Ritz coefficients c."""
        c = c.to(torch.float64).contiguous()
        out = torch.empty((3, self.n), dtype=torch.float64, device=c.device)
        N.call("neb_rollout_fields", *self._args()[:6], c.data_ptr(), out.data_ptr(),
               self.ws.data_ptr(), self.ws.numel(), _stream())
        return out

    def energy_skew(self, seed: int = 42) -> float:
        """|r . rhs(r)| / |r|^3 for a seeded normal r: the rotational form
        conserves energy, so this is rounding (the reference asserts < 1e-9,
        paper_rollout.py:43-45)."""
        r = torch.as_tensor(np.random.default_rng(seed).normal(size=self.K),
                            device=self.c.device)
        return float(torch.abs(r @ self.rhs(r)) / torch.linalg.norm(r) ** 3)

    def _set_step(self, h: float) -> None:
        if self.h == h:
            return
        N.call("neb_etdrk4_coefficients", self.K, self.ritz.lam.data_ptr(), self.nu, h,
               self.coef.data_ptr(), _stream())
        self.h = h

    def _step(self) -> None:
        N.call("neb_etdrk4_step", *self._args(), self.coef.data_ptr(), self.c.data_ptr(),
               self.ws.data_ptr(), self.ws.numel(), _stream())

    def advance(self, steps: int) -> None:
        """steps ETDRK4 steps of the current size on self.c."""
        if steps <= 0:
            return
        if not self.use_graph:
            for _ in range(steps):
                self._step()
            return
        if self._graph is None:
            g = torch.cuda.CUDAGraph()
            torch.cuda.synchronize()
            with torch.cuda.graph(g):
                self._step()
            self._graph = g
        for _ in range(steps):
            self._graph.replay()

    # --------------------------------------------------------------- schedule
    def run(self, c0, times, dt: float) -> np.ndarray:
        """The reference's frame loop (paper_rollout.py:47-75): for every
        target time, ceil((t - t_prev) / dt - 1e-10) equal steps; returns the
        coefficient states [frames, K] (one device-to-host copy at the end)."""
        self.c.copy_(torch.as_tensor(c0, dtype=torch.float64, device=self.c.device))
        current = 0.0
        states = []
        for target in np.asarray(times, dtype=np.float64):
            steps = max(0, int(math.ceil((target - current) / dt - 1e-10)))
            if steps:
                self._set_step((target - current) / steps)
                self.advance(steps)
            current = float(target)
            states.append(self.c.clone())
        return torch.stack(states).cpu().numpy()
