"""Replica sharding across ranks on CPU (gloo, world size 2): every rank
evaluates its contiguous share of the query rows and the shares concatenate
to the single-process result; timings reduce to the maximum.  The per-rank
evaluator is the CPU oracle (the product has no CPU path)."""
import os
import socket

import numpy as np
import pytest

from arbinterp_gb300.replicas import shard_range


def test_shard_range_partitions():
    for n in (0, 1, 7, 100, 101):
        for world in (1, 2, 3, 8):
            spans = [shard_range(n, world, r) for r in range(world)]
            assert spans[0][0] == 0 and spans[-1][1] == n
            for (a, b), (c, d) in zip(spans, spans[1:]):
                assert b == c and a <= b
            sizes = [b - a for a, b in spans]
            assert max(sizes) - min(sizes) <= 1
    with pytest.raises(ValueError):
        shard_range(10, 2, 2)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, field, q, result_path):
    import torch.distributed as dist
    from arbinterp_gb300.replicas import max_over_ranks, query_sharded
    from oracle.arb_oracle import OracleTricubic
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        o = OracleTricubic(field)

        def evaluate(rows):
            r = o.query(rows.copy())
            return r["norms"], r["grads"]

        norms, grads = query_sharded(evaluate, q)
        t = max_over_ranks(1.0 + rank)
        np.savez(f"{result_path}.{rank}.npz", norms=norms, grads=grads, t=t)
    finally:
        dist.destroy_process_group()


def test_query_sharded_gloo_world2(tmp_path):
    import torch.multiprocessing as mp
    from arbinterp_gb300 import synth
    from oracle.arb_oracle import OracleTricubic
    field = synth.gaussian_field3(n=(12, 11, 10), h=(0.1, 0.12, 0.08), seed=3).numpy()
    o = OracleTricubic(field)
    q = synth.uniform_queries(o.lo, o.hi, 997, 13, o.h, seed=4).numpy()
    ref = o.query(q.copy())
    world = 2
    path = str(tmp_path / "res")
    mp.start_processes(_worker, args=(world, _free_port(), field, q, path), nprocs=world, join=True,
                       start_method="spawn")
    for rank in range(world):
        r = np.load(f"{path}.{rank}.npz")
        assert float(r["t"]) == 2.0
        assert np.array_equal(r["norms"], ref["norms"], equal_nan=True)
        assert np.array_equal(r["grads"], ref["grads"], equal_nan=True)
