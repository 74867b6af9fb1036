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


def gather_device(group=None):
    """The device the gather's tensors must live on: the current CUDA device
    under a NCCL process group (NCCL moves device memory only), the CPU
    otherwise (gloo)."""
    import torch
    import torch.distributed as dist
    if dist.get_backend(group) == "nccl":
        return torch.device("cuda", torch.cuda.current_device())
    return torch.device("cpu")


def gather_images(local, n, rank, world, group=None):
    """All-gather per-rank image blocks [k_r, ...] into [n, ...] on every rank
    (torch.distributed): `local` is a numpy array or a tensor (host or device);
    the exchange runs on gather_device(group) -- gloo on the CPU, nccl on the
    current GPU -- and the result comes back as a numpy array."""
    import torch
    import torch.distributed as dist
    dev = gather_device(group)
    t = local if torch.is_tensor(local) else torch.as_tensor(np.ascontiguousarray(local))
    t = t.to(dev)
    shape = tuple(t.shape[1:])
    counts = [len(shard(n, r, world)) for r in range(world)]
    if t.shape[0] != counts[rank]:
        raise ValueError("rank %d holds %d blocks, its shard has %d" % (rank, t.shape[0],
                                                                       counts[rank]))
    mx = max(counts)
    pad = torch.zeros((mx,) + shape, dtype=t.dtype, device=dev)
    pad[:t.shape[0]] = t
    out = [torch.zeros_like(pad) for _ in range(world)]
    dist.all_gather(out, pad, group=group)
    return torch.cat([o[:c] for o, c in zip(out, counts)]).cpu().numpy()
