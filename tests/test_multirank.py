"""Sharding reads across ranks (one process per GPU) with a gloo world of 2 on
CPU: each rank takes its contiguous shard, results come back in read order.
The data path has no exchange; only the 32-byte result records are gathered."""
import os
import socket

import numpy as np
import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

from dtwax_gb300.shard import gather_results, shard_range

RESULT_DTYPE = np.dtype([("score", "<f4"), ("score_fwd", "<f4"), ("score_rev", "<f4"), ("strand", "<i4"),
                         ("end_pos", "<i8"), ("call", "<i4"), ("n_samples", "<i4")])


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, n, q):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    b, e = shard_range(n, rank, world)
    local = np.zeros(e - b, RESULT_DTYPE)
    local["end_pos"] = np.arange(b, e)          # stand-in for this rank's classification
    local["score"] = np.arange(b, e) * 0.5
    allres = gather_results(local, n, rank, world)
    q.put((rank, allres["end_pos"].tolist(), allres["score"].tolist()))
    dist.barrier()
    dist.destroy_process_group()


@pytest.mark.parametrize("n", [7, 2048])
def test_gloo_world2_shards_and_gathers_in_order(n):
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, n, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, ends, scores in out:
        assert ends == list(range(n))
        assert scores == [i * 0.5 for i in range(n)]
