"""Read sharding across GPUs (one process per GPU).

Reads are independent, so a batch is split into contiguous, nearly equal
shards, each rank classifies its own shard, and the per-read results are
gathered back in read order.  There is no exchange on the data path.
"""
from __future__ import annotations

import numpy as np


def shard_range(n: int, rank: int, world: int):
    """[begin, end) of rank's share of n reads."""
    base, extra = divmod(n, world)
    begin = rank * base + min(rank, extra)
    return begin, begin + base + (1 if rank < extra else 0)


def gather_results(local: np.ndarray, n: int, rank: int, world: int, group=None) -> np.ndarray:
    """All-gather every rank's result records (structured array) into read
    order.  Control-plane only (results, not the DP data): uses
    torch.distributed with whatever backend the group has."""
    import torch
    import torch.distributed as dist

    if world == 1:
        return local
    raw = np.frombuffer(local.tobytes(), np.uint8)
    sizes = [shard_range(n, r, world)[1] - shard_range(n, r, world)[0] for r in range(world)]
    itemsize = local.dtype.itemsize
    # NCCL gathers device tensors; gloo host tensors
    device = "cuda" if dist.get_backend(group) == "nccl" else "cpu"
    buf = torch.zeros(max(sizes) * itemsize, dtype=torch.uint8)
    buf[: raw.size] = torch.from_numpy(raw.copy())
    buf = buf.to(device)
    outs = [torch.zeros_like(buf) for _ in range(world)]
    dist.all_gather(outs, buf, group=group)
    parts = [np.frombuffer(o.cpu().numpy().tobytes()[: sizes[r] * itemsize], local.dtype)
             for r, o in enumerate(outs)]
    return np.concatenate(parts)
