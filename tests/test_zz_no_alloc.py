"""neb_hidden_gram_static (fixed device scratch, no workspace) against
neb_hidden_gram (caller-owned workspace), both through the C ABI.

Both run the same chunk kernels in the same order, so the Grams agree to
rounding; the test allows 1e-12 relative (FP64 network) and 1e-9 relative
to the largest entry (FP32 network).  Two calls in a row check that the
second call, which reuses the cached scratch address, gives the same result.
This file is collected last so it runs both alone and after the others.
"""
import ctypes

import pytest
import torch

from neb_gb300 import CONFIGS, Model
from neb_gb300 import _native as N
from neb_gb300 import configs as CF

pytestmark = pytest.mark.gpu


def _needs_gpu():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def _grams(model, n, static):
    cfg = model.c
    pts, w = CF.sample(cfg)
    pts, w = pts[:n], w[:n]
    feats = model.features(pts)
    qw = torch.as_tensor(w, device="cuda").to(model.dtype).contiguous()
    tape = model.run_forward(feats)
    H = cfg.hidden
    AM = torch.full((H, H), float("nan"), dtype=torch.float64, device="cuda")
    AS = torch.full((H, H), float("nan"), dtype=torch.float64, device="cuda")
    s = torch.cuda.current_stream().cuda_stream
    if static:
        N.call("neb_hidden_gram_static", ctypes.byref(model.net), qw.data_ptr(), n,
               tape.buffer.data_ptr(), AM.data_ptr(), AS.data_ptr(), s)
    else:
        ws = model._ws(n)
        N.call("neb_hidden_gram", ctypes.byref(model.net), qw.data_ptr(), n,
               tape.buffer.data_ptr(), AM.data_ptr(), AS.data_ptr(), 0, ws.data_ptr(), ws.numel(),
               s)
    torch.cuda.synchronize()
    return AM.cpu(), AS.cpu()


@pytest.mark.parametrize("precision,rtol", [("fp64", 1e-12), ("fp32", 1e-9)])
@pytest.mark.parametrize("hidden,n", [(128, 4096), (64, 1000), (256, 4096)])
def test_static_scratch_gram_matches_workspace_gram(precision, rtol, hidden, n):
    _needs_gpu()
    cfg = CONFIGS["periodic_small"].scaled(hidden=hidden, outputs=32, grid_n=64)
    model = Model(cfg, precision=precision, seed=3)
    ref_M, ref_S = _grams(model, n, static=False)
    for _ in range(2):
        AM, AS = _grams(model, n, static=True)
        for got, ref in ((AM, ref_M), (AS, ref_S)):
            assert torch.isfinite(got).all()
            err = float((got - ref).abs().max() / ref.abs().max())
            assert err <= rtol, err


def test_static_scratch_rejects_oversized_request():
    """width 256 at 8192 points needs 32 chunks x 256^2 doubles = 16 MiB > 8 MiB:
    rejected on the host before any launch."""
    _needs_gpu()
    cfg = CONFIGS["periodic_small"].scaled(hidden=256, outputs=32, grid_n=91)
    model = Model(cfg, precision="fp32", seed=3)
    n = 8192
    H = cfg.hidden
    AM = torch.zeros((H, H), dtype=torch.float64, device="cuda")
    AS = torch.zeros((H, H), dtype=torch.float64, device="cuda")
    qw = torch.ones(n, dtype=torch.float32, device="cuda")
    tape = torch.zeros(1, dtype=torch.uint8, device="cuda")
    with pytest.raises(ValueError, match="scratch"):
        N.call("neb_hidden_gram_static", ctypes.byref(model.net), qw.data_ptr(), n,
               tape.data_ptr(), AM.data_ptr(), AS.data_ptr(),
               torch.cuda.current_stream().cuda_stream)
    assert float(AM.abs().sum()) == 0.0
