"""Workload configurations and quadrature-point samplers.

The five workloads of the eigenfluid hot path:

* ``periodic_small``  2D periodic, 64 Fourier features, 3 x 128 tanh, K = 64,
                      64^2 grid, trace objective tr(M^-1 S), FP64.
* ``periodic_eval``   2D periodic, 4 x 512 tanh, K = 1024, 256^2 grid,
                      forward + Gram only.
* ``periodic_train``  as above, 128^2 uniform random points per step, ordering
                      objective sum_k lam_k / k, Adam lr 1e-3.
* ``multihole``       unit square minus 3 disks, 200,000 rejection samples,
                      features (x, y, 3 angles), 4 x 256 tanh, K = 1024.
* ``metaball3d``      1,599,754 rejection samples in a metaball region of
                      [0,1]^3, raw (x, y, z), 4 x 512 tanh, vector potential
                      with K = 512 modes (1,536 outputs), curl fields.

Samplers draw on the host with ``numpy.random.default_rng`` (PCG64), as the
reference's ``fluid_points`` does (hardcoded_backend.py:2424-2448 and
native_cupy_core.py:42-52), and are uploaded once.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field, replace

import numpy as np

TWO_PI = 2.0 * math.pi
MULTIHOLE_CENTRES = ((0.3, 0.3), (0.7, 0.4), (0.45, 0.75))
MULTIHOLE_RADII = (0.10, 0.08, 0.09)


@dataclass(frozen=True)
class NebConfig:
    name: str
    dim: int
    features: str                 # "periodic" | "multihole" | "raw3d"
    widths: tuple                 # (features, hidden..., outputs)
    objective: str                # "trace" | "ordering"
    n_freq: int = 0
    period: float = TWO_PI
    centres: tuple = ()
    sampler: str = "grid"         # "grid" | "uniform" | "multihole" | "metaball"
    n_points: int = 0
    grid_n: int = 0
    seed: int = 0
    lr: float = 1e-3
    steps: int = 0
    clip: float = 8.0
    # spectral stage: "mixed" for pencils that stay well conditioned (the
    # periodic Fourier-feature bases), "range" (FP64, rank-revealing) where
    # raw-coordinate inputs make the fields nearly dependent at init
    spectral: str = "mixed"
    # Gram accumulation of the FP32 / split-BF16 forms: "plain" FP32 sums, or
    # "compensated" (exact products, TwoSum chunk sums) for the bases whose
    # mass matrix is nearly singular at init
    gram: str = "plain"

    @property
    def K(self) -> int:
        return self.widths[-1] // (3 if self.dim == 3 else 1)

    @property
    def hidden(self) -> int:
        return self.widths[-2]

    def feature_params(self) -> list:
        if self.features == "periodic":
            return [self.period]
        if self.features == "multihole":
            return [v for c in self.centres for v in c]
        return []

    def scaled(self, **kw) -> "NebConfig":
        """Copy with overrides; ``hidden=`` and ``outputs=`` reshape widths."""
        hidden = kw.pop("hidden", None)
        outputs = kw.pop("outputs", None)
        widths = list(kw.pop("widths", self.widths))
        if hidden is not None:
            widths = [widths[0]] + [hidden] * (len(widths) - 2) + [widths[-1]]
        if outputs is not None:
            widths[-1] = outputs
        return replace(self, widths=tuple(widths), **kw)


CONFIGS = {
    "periodic_small": NebConfig("periodic_small", 2, "periodic", (64, 128, 128, 128, 64), "trace",
                                n_freq=16, sampler="grid", grid_n=64),
    "periodic_eval": NebConfig("periodic_eval", 2, "periodic", (64, 512, 512, 512, 512, 1024),
                               "ordering", n_freq=16, sampler="grid", grid_n=256),
    "periodic_train": NebConfig("periodic_train", 2, "periodic", (64, 512, 512, 512, 512, 1024),
                                "ordering", n_freq=16, sampler="uniform", n_points=128 * 128,
                                steps=25, lr=1e-3),
    "multihole": NebConfig("multihole", 2, "multihole", (5, 256, 256, 256, 256, 1024), "ordering",
                           centres=MULTIHOLE_CENTRES, sampler="multihole", n_points=200_000,
                           spectral="range", gram="compensated"),
    "metaball3d": NebConfig("metaball3d", 3, "raw3d", (3, 512, 512, 512, 512, 1536), "ordering",
                            sampler="metaball", n_points=1_599_754, spectral="range",
                            gram="compensated"),
}


def periodic_grid(n: int, period: float = TWO_PI):
    """n x n uniform grid of [0, period)^2, weight (period / n)^2 each."""
    g = np.arange(n, dtype=np.float64) * (period / n)
    xx, yy = np.meshgrid(g, g, indexing="ij")
    pts = np.stack([xx.ravel(), yy.ravel()], axis=1)
    return pts, np.full(len(pts), (period / n) ** 2)


def periodic_uniform(count: int, seed: int, step: int, period: float = TWO_PI):
    """count points ~ U[0, period)^2 from default_rng((seed, step)); equal
    weights period^2 / count."""
    rng = np.random.default_rng([seed, step])
    pts = rng.uniform(0.0, period, (count, 2))
    return pts, np.full(count, period * period / count)


def multihole_points(count: int, seed: int, centres=MULTIHOLE_CENTRES, radii=MULTIHOLE_RADII):
    """Rejection samples of the unit square minus the disks; weights area/N."""
    rng = np.random.default_rng(seed)
    out, remain = [], count
    c = np.asarray(centres, dtype=np.float64)
    r2 = np.asarray(radii, dtype=np.float64) ** 2
    while remain:
        cand = rng.random((max(2 * remain, 256), 2))
        d2 = ((cand[:, None, :] - c[None]) ** 2).sum(-1)
        acc = cand[np.all(d2 > r2[None], axis=1)][:remain]
        out.append(acc)
        remain -= len(acc)
    area = 1.0 - math.pi * float(r2.sum())
    pts = np.concatenate(out)
    return pts, np.full(count, area / count)


def metaball_points(count: int, seed: int, n_centres: int = 8, sigma: float = 0.08,
                    level: float = 0.5, batch: int = 1 << 20):
    """Rejection samples of {sum_i exp(-|x - c_i|^2 / (2 sigma^2)) < level} in
    [0,1]^3; the centres ~ U[0.2, 0.8]^3 come first from the same generator.
    Equal weights 1/N."""
    rng = np.random.default_rng(seed)
    centres = rng.uniform(0.2, 0.8, (n_centres, 3))
    out, remain = [], count
    while remain:
        cand = rng.random((min(max(2 * remain, 256), batch), 3))
        d2 = ((cand[:, None, :] - centres[None]) ** 2).sum(-1)
        acc = cand[np.exp(-d2 / (2 * sigma * sigma)).sum(1) < level][:remain]
        out.append(acc)
        remain -= len(acc)
    return np.concatenate(out), np.full(count, 1.0 / count)


def sample(cfg: NebConfig, step: int = 0, seed: int | None = None):
    """(points [n, dim] float64, weights [n] float64) for a configuration."""
    seed = cfg.seed if seed is None else seed
    if cfg.sampler == "grid":
        return periodic_grid(cfg.grid_n, cfg.period)
    if cfg.sampler == "uniform":
        return periodic_uniform(cfg.n_points, seed, step, cfg.period)
    if cfg.sampler == "multihole":
        return multihole_points(cfg.n_points, seed, cfg.centres or MULTIHOLE_CENTRES)
    if cfg.sampler == "metaball":
        return metaball_points(cfg.n_points, seed)
    raise ValueError(f"unknown sampler {cfg.sampler!r}")


def objective_weights(kind: str, m: int) -> np.ndarray:
    """c_k of L = sum_k c_k lam_k: 1 for the trace objective, 1/k for the
    ordering objective."""
    if kind == "trace":
        return np.ones(m)
    if kind == "ordering":
        return 1.0 / np.arange(1, m + 1, dtype=np.float64)
    raise ValueError(f"unknown objective {kind!r}")


def glorot_params(widths, seed: int):
    """Glorot-normal weights (std sqrt(2 / (fan_in + fan_out))) and zero
    biases, drawn layer by layer from default_rng(seed), as float64."""
    rng = np.random.default_rng(seed)
    out = []
    for fan_in, fan_out in zip(widths[:-1], widths[1:]):
        std = math.sqrt(2.0 / (fan_in + fan_out))
        out.append((rng.normal(0.0, std, (fan_out, fan_in)), np.zeros(fan_out)))
    return out
