"""Multi-rank path sharding on CPU (gloo, world size 2).

A weak-scaling run gives rank r the paths [r M, (r+1) M) of the counter-based
stream; the only exchange is the sum of the integer counts.  Two gloo ranks
each count their shard with the oracle's FP64 restatement of the engine's
layout, all-reduce the counts, and must equal one rank counting all 2M
paths.  No GPU is used."""
import os
import socket

import numpy as np
import pytest


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, M, out):
    import sys
    here = os.path.dirname(os.path.abspath(__file__))
    root = os.path.dirname(here)
    for p in (os.path.join(root, "gpu-montecarlo-risk_gb300"), os.path.join(root, "oracle")):
        sys.path.insert(0, p)
    import torch
    import torch.distributed as dist
    import mc_oracle
    from riskgpu import synth
    from riskgpu import shard_range  # noqa: F401  (pure Python helper; no library load)
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    p = synth.one_factor_20()
    L, _ = mc_oracle.cholesky_lower(p.sigma)
    off, cnt = shard_range(rank, world, M)
    r = mc_oracle.mc_philox(p.mu, L, p.weights, 1, cnt, p.seed, p.x, p.k, p.port_threshold,
                            path_offset=off, nthreads=1)
    t = torch.tensor([r["crash"], r["breach"]], dtype=torch.int64)
    dist.all_reduce(t)
    if rank == 0:
        out.put(t.tolist())
    dist.destroy_process_group()


def test_two_rank_shards_sum_to_single_rank(oracle):
    import multiprocessing as mp
    from riskgpu import synth
    M = 20000
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, M, q)) for r in range(2)]
    for pr in procs:
        pr.start()
    got = q.get(timeout=120)
    for pr in procs:
        pr.join(timeout=60)
        assert pr.exitcode == 0
    p = synth.one_factor_20()
    L, _ = oracle.cholesky_lower(p.sigma)
    full = oracle.mc_philox(p.mu, L, p.weights, 1, 2 * M, p.seed, p.x, p.k, p.port_threshold)
    assert got == [full["crash"], full["breach"]]


def test_shard_range_validation():
    import sys
    from riskgpu import shard_range
    assert shard_range(0, 2, 10) == (0, 10)
    assert shard_range(1, 2, 10) == (10, 10)
    with pytest.raises(ValueError):
        shard_range(2, 2, 10)
