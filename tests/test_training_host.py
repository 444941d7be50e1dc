"""Training-loop glue on the host (no GPU): the cosine schedule equals the
reference trainers' formulas, and the epoch loop schedules, validates and
checkpoints as they do."""
import math

import numpy as np

from neb_gb300.training import cosine_learning_rate, train


def test_cosine_schedule_matches_reference_formulas():
    base, minimum, epochs = 2.8e-5, 1e-7, 2000
    for epoch in (1, 2, 500, 1000, 1999, 2000):
        # experiments/metaball/train.py:304-305 (2000 epochs)
        metaball = minimum + (base - minimum) * 0.5 * (1 + math.cos(math.pi * (epoch - 1) / 1999))
        assert abs(cosine_learning_rate(base, minimum, epoch, epochs) - metaball) <= 1e-20
    assert cosine_learning_rate(base, minimum, 1, epochs) == base
    assert abs(cosine_learning_rate(base, minimum, epochs, epochs) - minimum) < 1e-20
    # the periodic trainer clamps progress to [0, 1] and handles one epoch
    assert cosine_learning_rate(1.0, 0.0, 5000, 10) == 0.0
    assert cosine_learning_rate(1.0, 0.0, 1, 1) == 1.0


class _FakeModel:
    def __init__(self):
        self.saved = []

    def save(self, path):
        self.saved.append(str(path))


def test_epoch_loop_schedules_validates_and_checkpoints(tmp_path):
    model = _FakeModel()
    seen = []

    def step(m, epoch, lr):
        seen.append((epoch, lr))
        return {"losses": np.array([epoch, epoch + 1.0])}

    hist = train(model, step, epochs=6, base_lr=1.0, min_lr=0.0, start_epoch=2,
                 checkpoint=tmp_path / "state.npz", checkpoint_every=2,
                 validate=lambda m, e: {"epoch": e}, validate_every=3)
    assert [e for e, _ in seen] == [2, 3, 4, 5, 6]
    assert all(abs(lr - cosine_learning_rate(1.0, 0.0, e, 6)) == 0 for e, lr in seen)
    assert [h["loss"] for h in hist] == [2.5, 3.5, 4.5, 5.5, 6.5]
    assert [h.get("validation") for h in hist] == [None, {"epoch": 3}, None, None, {"epoch": 6}]
    assert len(model.saved) == 3  # epochs 2, 4, 6


def test_train_keeps_host_losses_in_fp64():
    """A step that returns its loss as a host float is recorded exactly (no
    round trip through a float32 tensor)."""
    from neb_gb300.training import train

    class M:
        def save(self, path):
            pass

    hist = train(M(), lambda m, e, lr: {"loss": 11.814643144231551}, 1, 1e-3, 1e-4)
    assert hist[0]["loss"] == 11.814643144231551
