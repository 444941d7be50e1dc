"""CPU checks of the C ABI and the host logic (no GPU needed)."""
import ctypes
import re
from pathlib import Path

import numpy as np
import pytest
import torch

from oracle import neb_oracle as O
from neb_gb300 import _native as N
from neb_gb300 import configs as CF
from neb_gb300.jets import Jet, pack, unpack

ROOT = Path(__file__).resolve().parents[1]


@pytest.fixture(scope="module")
def lib():
    if not N.LIB_PATH.exists():
        from neb_gb300 import build
        build.build()
    return N.load()


def declared_symbols():
    text = (ROOT / "include" / "neb_gb300.h").read_text()
    return sorted(set(re.findall(r"^\s*(?:const\s+)?\w+\*?\s+\*?(neb_\w+)\(", text, re.M)))


def test_every_declared_symbol_is_exported_and_bound(lib):
    names = declared_symbols()
    assert len(names) >= 15
    for name in names:
        assert hasattr(lib, name), name
        assert name in N.EXPORTED, f"{name} has no ctypes signature"


def test_tape_and_workspace_sizes_are_host_computed(lib):
    net = N.NebNet.make(2, [64, 512, 512, 512, 512, 1024], "fp32")
    n = 16384
    tape = lib.neb_tape_bytes(ctypes.byref(net), n)
    # X_0 + 4 x (Z_l + X_l) in FP32
    expect = n * 4 * 64 * 4 + 4 * 2 * n * 4 * 512 * 4
    assert expect <= tape <= expect + 4096
    assert lib.neb_workspace_bytes(ctypes.byref(net), n) > 0
    bad = N.NebNet.make(2, [64, 8, 8], "fp32")
    bad.dim = 5
    assert lib.neb_tape_bytes(ctypes.byref(bad), n) == 0
    assert "dim" in N.last_error()


def test_status_codes_map_to_reference_exceptions():
    with pytest.raises(ValueError):
        N.check(N.NEB_ERR_ARG, "x")
    for code in (N.NEB_ERR_NONFINITE, N.NEB_ERR_NOT_PD, N.NEB_ERR_SOLVER):
        with pytest.raises(FloatingPointError):
            N.check(code, "x")
    with pytest.raises(RuntimeError):
        N.check(N.NEB_ERR_CUDA, "x")
    N.check(N.NEB_OK, "x")


def test_netstruct_layout_and_limits():
    net = N.NebNet.make(3, [3, 512, 512, 512, 512, 1536], "bf16x3")
    assert (net.dim, net.n_hidden, net.precision) == (3, 4, 2)
    assert list(net.widths)[:6] == [3, 512, 512, 512, 512, 1536]
    with pytest.raises(ValueError):
        N.NebNet.make(2, [4, 8], "fp32")


def test_samplers_agree_with_the_oracle():
    p, w = CF.multihole_points(3000, 5)
    q, wq = O.multihole_points(3000, 5)
    np.testing.assert_array_equal(p, q)
    assert np.allclose(w, wq)
    p, w = CF.metaball_points(2000, 1)
    q, wq, _ = O.metaball_points(2000, 1)
    np.testing.assert_array_equal(p, q)
    p, w = CF.periodic_uniform(500, 0, 3)
    q, wq = O.periodic_minibatch(500, 0, 3)
    np.testing.assert_array_equal(p, q)
    g, wg = CF.periodic_grid(16)
    h, wh = O.periodic_grid(16)
    np.testing.assert_array_equal(g, h)
    for widths in ([64, 128, 128, 128, 64], [5, 7, 9]):
        for (a, b), (c, d) in zip(CF.glorot_params(widths, 3), O.glorot_init(widths, 3)):
            np.testing.assert_array_equal(a, c)
            np.testing.assert_array_equal(b, d)


def test_objective_weights_and_configs():
    np.testing.assert_array_equal(CF.objective_weights("trace", 4), O.objective_weights("trace", 4))
    np.testing.assert_array_equal(CF.objective_weights("ordering", 5), O.objective_weights("ordering", 5))
    c = CF.CONFIGS["periodic_train"]
    assert c.K == 1024 and c.hidden == 512 and c.n_points == 16384
    assert CF.CONFIGS["metaball3d"].K == 512
    s = c.scaled(hidden=32, outputs=24)
    assert s.widths == (64, 32, 32, 32, 32, 24)


@pytest.mark.parametrize("dim", [2, 3])
def test_jet_pack_roundtrip(dim):
    n, F = 5, 7
    g = torch.randn(n, F, dim)
    if dim == 2:
        j = Jet(torch.randn(n, F), g, lap=torch.randn(n, F))
    else:
        j = Jet(torch.randn(n, F), g, hess=torch.randn(n, F, 6))
    p = pack(j, dim)
    assert p.shape == (n, 4 if dim == 2 else 10, F)
    u = unpack(p, dim)
    assert torch.equal(u.value, j.value) and torch.equal(u.grad, j.grad)
    if dim == 2:
        assert torch.equal(u.lap, j.lap)
    else:
        assert torch.equal(u.hess, j.hess)
