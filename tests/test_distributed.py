"""Row sharding and the global-clim exchange on world size 2 (gloo, CPU)."""
from __future__ import annotations

import math
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

from oct_recon_af_v1_gb300.distributed import global_clim, shard_rows


def test_shard_rows_partitions_every_row():
    for n in (0, 1, 2, 5, 17):
        for w in (1, 2, 3, 8):
            got = [r for k in range(w) for r in shard_rows(n, k, w)]
            assert got == list(range(n))
    with pytest.raises(ValueError):
        shard_rows(4, 2, 2)


def _port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        rng = np.random.default_rng(rank)
        planes = rng.uniform(-60, 30, (3, 4, 5)).astype(np.float32)
        planes[0] = np.nan
        fin = planes[np.isfinite(planes)]
        lo, hi = global_clim(float(fin.min()), float(fin.max()))
        empty = global_clim(math.nan, math.nan) if rank == 0 else global_clim(float(fin.min()), float(fin.max()))
        none = global_clim(math.nan, math.nan)
        q.put((rank, float(fin.min()), float(fin.max()), lo, hi, empty, none))
    finally:
        dist.destroy_process_group()


def test_global_clim_two_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    lo = min(r[1] for r in res)
    hi = max(r[2] for r in res)
    for r in res:
        assert (r[3], r[4]) == (lo, hi)
        assert r[5] == (res[1][1], res[1][2])          # rank 0 had no finite value
        assert math.isnan(r[6][0]) and math.isnan(r[6][1])
