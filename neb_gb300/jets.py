"""Jet containers of the host API and their packing to the device layout.

A 2D jet carries ``value [n, F]``, ``grad [n, F, 2]`` and ``lap [n, F]``
(the Laplacian channel, all the 2D fields need); a 3D jet carries
``value [n, F]``, ``grad [n, F, 3]`` and ``hess [n, F, 6]`` with the
Hessian order (xx, xy, xz, yy, yz, zz) of the reference's compact Jet2
(experiments/metaball/_backend/flow/cases/metaball/velocity_trace_jet2.py:9-25).
The device layout packs the channels of a point next to each other:
``[n, C, F]`` with C = 4 (value, x, y, lap) or 10 (value, x, y, z, 6 Hessian).
"""
from __future__ import annotations

from dataclasses import dataclass

import torch


@dataclass
class Jet:
    value: torch.Tensor
    grad: torch.Tensor
    lap: torch.Tensor | None = None
    hess: torch.Tensor | None = None
    third: torch.Tensor | None = None  # 2D third derivatives (xxx, xxy, xyy, yyy)

    @property
    def dim(self) -> int:
        return self.grad.shape[-1]


def pack(jet: Jet, dim: int) -> torch.Tensor:
    """[n, F] jets -> packed [n, C, F]."""
    v = torch.as_tensor(jet.value)
    g = torch.as_tensor(jet.grad)
    if dim == 2:
        lap = torch.as_tensor(jet.lap) if jet.lap is not None else \
            torch.as_tensor(jet.hess)[..., 0] + torch.as_tensor(jet.hess)[..., 2]
        chans = [v, g[..., 0], g[..., 1], lap]
    else:
        h = torch.as_tensor(jet.hess)
        chans = [v, g[..., 0], g[..., 1], g[..., 2], *[h[..., k] for k in range(6)]]
    return torch.stack(chans, dim=1).contiguous()


def unpack(packed: torch.Tensor, dim: int) -> Jet:
    """packed [n, C, F] -> Jet of [n, F] channels."""
    if dim == 2:
        return Jet(packed[:, 0], packed[:, 1:3].permute(0, 2, 1), lap=packed[:, 3])
    return Jet(packed[:, 0], packed[:, 1:4].permute(0, 2, 1), hess=packed[:, 4:10].permute(0, 2, 1))
