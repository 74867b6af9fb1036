"""The N > 1 path on CPU: two gloo ranks split a tilt series's orientations,
compute their share (oracle, small grid) and gather the images; the result is
the single-process result bit for bit."""
import os
import socket

import numpy as np
import pytest

from conftest import ROOT

torch = pytest.importorskip("torch")


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _series():
    import sys
    sys.path.insert(0, ROOT)
    from oracle.oracle import SeriesParams
    p = SeriesParams()
    p.ax, p.ctblengthz, p.nx, p.ny, p.v0, p.deltaz = 32.0, 32.0, 32, 32, 200.0, 2.0
    p.max_slices, p.min_slice = -1, 0
    return p


def _worker(rank, world, port, q):
    import sys
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    from oracle.oracle import Oracle
    from utr_public_gb300 import specimen, shard
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    spec = specimen.random_specimen(150, 32.0, 5.0, 27.0, 31)
    angY = np.deg2rad(np.arange(7) * 25.0)
    mine = shard.shard(len(angY), rank, world)
    O = Oracle()
    local = np.stack([O.orientation(_series(), spec.Znum, spec.x, spec.y, spec.z, spec.occ, 0.0,
                                    angY[a], np.array([0.0, 80.0]))[0] for a in mine])
    full = shard.gather_images(local, len(angY), rank, world)
    dist.barrier()
    dist.destroy_process_group()
    q.put((rank, full))


def test_shard_covers_everything_once():
    from utr_public_gb300 import shard
    for n in (1, 7, 180):
        for w in (1, 2, 3, 8):
            idx = np.concatenate([shard.shard(n, r, w) for r in range(w)])
            assert np.array_equal(idx, np.arange(n))


def test_two_ranks_gather_equals_single_process():
    import multiprocessing as mp
    from oracle.oracle import Oracle
    from utr_public_gb300 import specimen
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = dict(q.get(timeout=180) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    spec = specimen.random_specimen(150, 32.0, 5.0, 27.0, 31)
    angY = np.deg2rad(np.arange(7) * 25.0)
    O = Oracle()
    ref = np.stack([O.orientation(_series(), spec.Znum, spec.x, spec.y, spec.z, spec.occ, 0.0, a,
                                  np.array([0.0, 80.0]))[0] for a in angY])
    for r in (0, 1):
        assert np.array_equal(res[r], ref)
