"""Replicas over GPUs, host side: balanced disjoint column shards, and the
timing/work reduction over world_size 2 gloo ranks on the CPU."""
import os
import socket

import numpy as np
import pytest

from vulcan_gb300 import configs
from vulcan_gb300.replicas import column_shards


def test_shards_disjoint_cover_balanced():
    nz = np.array([s.pco.size for s in configs.config2_columns(ncols=512, seed=2)])
    for n in (1, 2, 4, 8):
        parts = column_shards(nz, n)
        allc = np.sort(np.concatenate(parts))
        np.testing.assert_array_equal(allc, np.arange(nz.size))
        loads = np.array([nz[p].sum() for p in parts])
        assert loads.max() - loads.min() <= nz.max()


def _worker(rank, port, q):
    os.environ.update(MASTER_ADDR='127.0.0.1', MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE='2', LOCAL_RANK=str(rank))
    from vulcan_gb300 import replicas
    dist = replicas.init(backend='gloo')
    replicas.barrier(dist)
    work, sec = replicas.reduce_run(dist, work=10 * (rank + 1), seconds=1.5 + rank)
    q.put((rank, work, sec))
    dist.destroy_process_group()


def test_reduce_over_two_gloo_ranks():
    pytest.importorskip('torch')
    import multiprocessing as mp
    with socket.socket() as s:
        s.bind(('127.0.0.1', 0))
        port = s.getsockname()[1]
    ctx = mp.get_context('spawn')
    q = ctx.Queue()
    ps = [ctx.Process(target=_worker, args=(r, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    for p in ps:
        p.join(120)
        assert p.exitcode == 0
    res = sorted(q.get(timeout=10) for _ in range(2))
    for rank, work, sec in res:
        assert work == 30.0 and sec == 2.5
