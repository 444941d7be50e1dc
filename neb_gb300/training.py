"""Training-loop glue around the hot path.

* ``cosine_learning_rate``: the cosine schedule of the reference's trainers
  (experiments/2d/_backend/flow/cases/vortex_merger/neural_training/
  train_gauge_canonical.py:827-835; experiments/metaball/train.py:304-305):
  lr(epoch) = lr_min + (lr_base - lr_min) (1 + cos(pi p)) / 2 with
  p = (epoch - 1) / max(epochs - 1, 1) clamped to [0, 1].
* ``velocity_train_step``: one update of the per-mode network on the 3D
  velocity objective, the ``step`` of experiments/metaball/train.py:208-214
  (objective and gradient, then Adam at the scheduled rate), with the
  peel's status word gating the update on the device.
* ``potential_train_step``: one epoch of the reference's periodic trainer
  (train_gauge_canonical.py:825-880): the epoch's points from
  ``fluid_points`` seeded cfg.seed + 1009 epoch, the learning rate of the
  schedule, one ``peel_step`` of the periodic backend.
* ``train``: the epoch loop (sample, step, optional validation, atomic
  checkpoint every ``checkpoint_every`` epochs) for every model family.
"""
from __future__ import annotations

import math
from pathlib import Path
from typing import Callable

import numpy as np
import torch


def cosine_learning_rate(base: float, minimum: float, epoch: int, epochs: int) -> float:
    """Learning rate of (1-based) ``epoch`` out of ``epochs``."""
    progress = min(max((epoch - 1) / max(int(epochs) - 1, 1), 0.0), 1.0)
    return float(minimum) + 0.5 * (float(base) - float(minimum)) * (1.0 + math.cos(math.pi * progress))


def velocity_train_step(model, data, lr: float, clip: float = 8.0, block: int = 256,
                        check: bool = False) -> dict:
    """Velocity objective + gradient + per-mode Adam.  With ``check`` the
    peel's gate raises FloatingPointError before any update; otherwise the
    gate is applied on the device (a failed peel commits nothing) and the
    status stays in ``result["info"]`` for the caller to read later."""
    from .modes import velocity_step
    res = velocity_step(model, data, training=True, block=block, check=check)
    gW, gb = res.pop("grads")
    norms, committed = model.adam_async(gW, gb, lr, clip, gate=res["info"])
    res.update(norms=norms, committed=committed)
    if check and not bool(committed.item()):
        raise FloatingPointError("Invalid parameter gradients; no optimizer update")
    return res


def potential_train_step(cfg, model, epoch: int, lr: float) -> dict:
    """One epoch of the periodic trainer on a HardcodedModel: cfg.learning_rate
    is set to lr (the schedule's value), points = fluid_points(cfg,
    cfg.points_per_step, 0, 0, cfg.seed + 1009 epoch), then peel_step with
    training.  Returns the peel step's diagnostics."""
    from .hardcoded import fluid_points, peel_step
    cfg.learning_rate = float(lr)
    points = fluid_points(cfg, int(cfg.points_per_step), 0.0, 0.0, int(cfg.seed) + epoch * 1009)
    return peel_step(cfg, model, points, 0.0, 0.0, True)


def train(model, step: Callable[[object, int, float], dict], epochs: int, base_lr: float,
          min_lr: float, start_epoch: int = 1, checkpoint: str | Path | None = None,
          checkpoint_every: int = 1, validate: Callable[[object, int], dict] | None = None,
          validate_every: int = 0) -> list:
    """The reference's epoch loop: for epoch = start_epoch .. epochs, call
    ``step(model, epoch, lr)`` at the cosine rate, validate every
    ``validate_every`` epochs, and save ``model`` atomically (temporary file
    then replace, the model's own ``save``) every ``checkpoint_every``
    epochs.  Returns one record per epoch with the loss read back (a
    device tensor's value is read once per epoch)."""
    history = []
    for epoch in range(int(start_epoch), int(epochs) + 1):
        lr = cosine_learning_rate(base_lr, min_lr, epoch, epochs)
        res = step(model, epoch, lr)
        losses = res.get("losses", res.get("loss"))
        if losses is None:
            loss = None
        elif isinstance(losses, torch.Tensor):
            loss = float(losses.double().mean())
        else:  # host values (a float or a list) keep their FP64 value
            loss = float(np.mean(np.asarray(losses, dtype=np.float64)))
        record = {"epoch": epoch, "learning_rate": lr, "loss": loss}
        if validate is not None and validate_every and epoch % validate_every == 0:
            record["validation"] = validate(model, epoch)
        if checkpoint is not None and checkpoint_every and epoch % checkpoint_every == 0:
            model.save(checkpoint)
        history.append(record)
    return history
