"""Failure handling on the GPU, without faulting it (GB300 only).

* A bounded device-side wait whose phase never completes (no thread
  arrives) gives up after its spin limit, the call returns NEB_ERR_TIMEOUT,
  and the context stays usable for the next step.
* A rejected Adam transaction (non-finite gradient) changes nothing, not
  even the committed-step count that sets the next step's bias correction
  (the reference advances its epoch only after a committed update,
  experiments/metaball/_backend/flow/cases/metaball/native_cupy_core.py:
  157-170), on the synchronous and on the asynchronous path.
"""
import ctypes

import numpy as np
import pytest
import torch

from oracle import neb_oracle as O
from neb_gb300 import CONFIGS, Model, spectral_step
from neb_gb300 import _native as N
from neb_gb300 import configs as CF

pytestmark = pytest.mark.gpu


def _needs_gpu():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def _stream():
    return torch.cuda.current_stream().cuda_stream


def _params64(model):
    return [(W.detach().cpu().double().numpy(), b.detach().cpu().double().numpy())
            for W, b in zip(model.W, model.b)]


def test_bounded_wait_runs_out_and_context_survives():
    _needs_gpu()
    lib = N.load()
    status = torch.zeros((), dtype=torch.int32, device="cuda")
    # nothing arrives on the barrier: the wait gives up after 2^16 polls
    rc = lib.neb_wait_selftest(0, 1 << 16, ctypes.c_void_p(status.data_ptr()), _stream())
    assert rc == N.NEB_ERR_TIMEOUT, (rc, N.last_error())
    assert int(status.item()) & 1
    assert "gave up" in N.last_error()
    # with the arrival the same wait completes
    rc = lib.neb_wait_selftest(1, 1 << 16, ctypes.c_void_p(status.data_ptr()), _stream())
    assert rc == N.NEB_OK
    assert int(status.item()) == 0
    # out-of-range limits are argument errors, not launches
    rc = lib.neb_wait_selftest(0, 10, ctypes.c_void_p(status.data_ptr()), _stream())
    assert rc == N.NEB_ERR_ARG
    # the context is still usable: a full objective step afterwards
    cfg = CONFIGS["periodic_small"].scaled(hidden=16, outputs=8, grid_n=8)
    model = Model(cfg, precision="fp64")
    pts, w = CF.sample(cfg)
    res = spectral_step(model, pts, w, training=True)
    assert np.isfinite(float(res.loss))


def _grads(model, seed):
    rng = np.random.default_rng(seed)
    g = [(rng.normal(size=tuple(W.shape)), rng.normal(size=tuple(b.shape)))
         for W, b in zip(model.W, model.b)]
    gW = [torch.tensor(a, dtype=model.dtype, device="cuda") for a, _ in g]
    gb = [torch.tensor(b, dtype=model.dtype, device="cuda") for _, b in g]
    return g, gW, gb


@pytest.mark.parametrize("asynchronous", [False, True])
def test_rejected_adam_step_keeps_epoch(asynchronous):
    """A rejected step followed by a good one equals the oracle's first step
    (bias correction of step 1), and the epoch counts committed steps only."""
    _needs_gpu()
    cfg = CONFIGS["periodic_small"].scaled(hidden=16, outputs=8)
    model = Model(cfg, precision="fp32", seed=4)
    p0 = _params64(model)
    g, gW, gb = _grads(model, 1)
    bad = [t.clone() for t in gW]
    bad[1][0, 0] = float("inf")
    if asynchronous:
        _, committed = model.adam_async(bad, gb, 1e-3, clip=0.5)
        assert int(committed.item()) == 0
    else:
        with pytest.raises(FloatingPointError):
            model.adam(bad, gb, 1e-3, clip=0.5)
    assert model.epoch == 0
    for (W, b), (rW, rb) in zip(_params64(model), p0):
        assert np.array_equal(W, rW) and np.array_equal(b, rb)
    if asynchronous:
        _, committed = model.adam_async(gW, gb, 1e-3, clip=0.5)
        assert int(committed.item()) == 1
    else:
        model.adam(gW, gb, 1e-3, clip=0.5)
    assert model.epoch == 1
    ref, _ = O.adam_step(p0, O.zero_moments(p0), g, 0, 1e-3, 0.5)[:2]
    for (W, b), (rW, rb) in zip(_params64(model), ref):
        np.testing.assert_allclose(W, rW, rtol=2e-6, atol=2e-7)
        np.testing.assert_allclose(b, rb, rtol=2e-6, atol=2e-7)


def test_adam_gate_blocks_commit_on_device():
    """A non-zero objective status word handed to Adam as its gate commits
    nothing, for the shared network and the per-mode networks alike."""
    _needs_gpu()
    from types import SimpleNamespace
    from neb_gb300 import ModeModel
    cfg = CONFIGS["periodic_small"].scaled(hidden=16, outputs=8)
    model = Model(cfg, precision="fp32", seed=4)
    p0 = _params64(model)
    _, gW, gb = _grads(model, 1)
    bad = torch.ones((), dtype=torch.int32, device="cuda")
    good = torch.zeros((), dtype=torch.int32, device="cuda")
    _, committed = model.adam_async(gW, gb, 1e-3, gate=bad)
    assert int(committed.item()) == 0 and model.epoch == 0
    for (W, b), (rW, rb) in zip(_params64(model), p0):
        assert np.array_equal(W, rW) and np.array_equal(b, rb)
    _, committed = model.adam_async(gW, gb, 1e-3, gate=good)
    assert int(committed.item()) == 1 and model.epoch == 1
    c = SimpleNamespace(hidden=8, hidden_layers=2, siren_first_omega0=2.0, siren_hidden_omega0=1.5)
    mm = ModeModel(c, K=3, seed=1, inputs=5, outputs=3)
    W0 = [w.clone() for w in mm.W]
    gw = [torch.ones_like(w) for w in mm.W]
    gbb = [torch.ones_like(x) for x in mm.b]
    _, committed = mm.adam_async(gw, gbb, 1e-3, gate=bad)
    assert int(committed.item()) == 0 and mm.epoch == 0
    assert all(torch.equal(a, b) for a, b in zip(mm.W, W0))
    _, committed = mm.adam_async(gw, gbb, 1e-3, gate=good)
    assert int(committed.item()) == 1 and mm.epoch == 1
