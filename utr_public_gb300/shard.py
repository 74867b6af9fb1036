"""Orientations across ranks: one process per GPU, no exchange on the data path.

A tilt series's orientations (and thermal configurations) are independent
(the reference runs one host thread per orientation, MultisliceT.cpp:403-448),
so N GPUs either each run their own series (weak scaling, as bench.py does) or
split one series and gather the images at the end (strong scaling, below).
"""
import numpy as np


def shard(n, rank, world):
    """Contiguous block of range(n) owned by `rank` of `world` (sizes differ by <= 1)."""
    base, extra = divmod(n, world)
    lo = rank * base + min(rank, extra)
    return np.arange(lo, lo + base + (1 if rank < extra else 0))


def gather_images(local, n, rank, world, group=None):
    """All-gather per-rank image blocks [k_r, ...] into [n, ...] on every rank
    (torch.distributed; works with gloo on CPU and nccl on GPUs)."""
    import torch
    import torch.distributed as dist
    t = torch.as_tensor(np.ascontiguousarray(local))
    shape = tuple(t.shape[1:])
    counts = [len(shard(n, r, world)) for r in range(world)]
    mx = max(counts)
    pad = torch.zeros((mx,) + shape, dtype=t.dtype)
    pad[:t.shape[0]] = t
    out = [torch.zeros_like(pad) for _ in range(world)]
    dist.all_gather(out, pad, group=group)
    return torch.cat([o[:c] for o, c in zip(out, counts)]).numpy()
