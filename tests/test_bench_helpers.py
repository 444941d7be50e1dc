"""bench.py helpers that need no GPU: the Gram throughput convention
(symmetric count R * K * (K + 1) per Gram) and the kernel-table pick."""
import pytest

import bench


def test_gram_rate_symmetric_count():
    n, H = 16384, 512
    g = bench.gram_rate(0.1, (2 * n, n), H)  # 0.1 ms per step
    flops = 3 * n * H * (H + 1)
    assert g["flops_per_step"] == flops
    assert g["tflops"] == pytest.approx(flops / 1e-4 / 1e12)


def test_gram_rate_without_gram_time():
    assert bench.gram_rate(0.0, (10,), 4)["tflops"] is None


def test_gram_ms_sums_the_gram_scopes_only():
    kern = {"tc_gram": 0.06, "simt_gram": 0.04, "tc_weight_grad": 0.5}
    assert bench._gram_ms(kern) == pytest.approx(0.10)
