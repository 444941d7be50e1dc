"""Replica mode of bench.py (--gpus N runs N independent replicas) on CPU
with the gloo backend, world size 2: each rank draws its own point batches,
the slowest rank's time sets the whole-job value, and the reduction is a
real torch.distributed all-reduce."""
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

import bench
from neb_gb300 import CONFIGS
from neb_gb300 import configs as CF


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    import os

    import torch
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    cfg = CONFIGS["periodic_train"]
    pts, _ = CF.sample(cfg, step=0, seed=bench.replica_seed(cfg.seed, rank))
    ms = 10.0 + 5.0 * rank  # this rank's timed region
    ms_max = bench.max_over_ranks(ms, world, "cpu")
    head = torch.tensor(pts[:4].ravel())
    gathered = [torch.zeros_like(head) for _ in range(world)]
    dist.all_gather(gathered, head)
    out[rank] = (ms_max, bench.whole_job_steps_per_s(world, 20, ms_max),
                 [g.tolist() for g in gathered])
    dist.destroy_process_group()


def test_replicas_world2_gloo():
    ctx = mp.get_context("spawn")
    with ctx.Manager() as manager:
        out = manager.dict()
        port = _free_port()
        procs = [ctx.Process(target=_worker, args=(r, 2, port, out)) for r in range(2)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(timeout=180)
        codes = [p.exitcode for p in procs]
        results = dict(out)
    assert codes == [0, 0], codes
    for rank in (0, 1):
        ms_max, value, gathered = results[rank]
        assert ms_max == 15.0
        assert value == pytest.approx(2 * 20 / 0.015)
        assert not np.allclose(gathered[0], gathered[1])  # distinct batches per replica


def test_single_rank_needs_no_process_group():
    assert bench.max_over_ranks(3.5, 1) == 3.5
    assert bench.whole_job_steps_per_s(1, 10, 100.0) == pytest.approx(100.0)
