"""Replicas over GPUs: columns are independent (no coupling anywhere in the
reference's op.py), so N GPUs run N independent batches over disjoint column
sets.  The only collectives are a barrier and the reduction of the timing
(max) and of the work done (sum) -- nothing on the data path.
"""
from __future__ import annotations

import os

import numpy as np


def world():
    """(rank, world_size, local_rank) from the torchrun environment."""
    return (int(os.environ.get('RANK', '0')), int(os.environ.get('WORLD_SIZE', '1')),
            int(os.environ.get('LOCAL_RANK', '0')))


def column_shards(nz, nshards):
    """Split columns over shards with balanced work (sum of nz, the block
    solve's cost per column being proportional to nz): longest column first
    onto the least-loaded shard.  Returns a list of index arrays (ascending)."""
    nz = np.asarray(nz)
    load = np.zeros(nshards)
    parts = [[] for _ in range(nshards)]
    for c in np.argsort(-nz, kind='stable'):
        s = int(np.argmin(load))
        parts[s].append(int(c))
        load[s] += nz[c]
    return [np.array(sorted(p), dtype=np.int64) for p in parts]


def init(backend=None):
    """Initialise torch.distributed when WORLD_SIZE > 1 (nccl on GPUs, gloo
    otherwise); returns the torch.distributed module or None."""
    rank, ws, local = world()
    if ws <= 1:
        return None
    import torch
    import torch.distributed as dist
    if not dist.is_initialized():
        if backend is None:
            backend = 'nccl' if torch.cuda.is_available() else 'gloo'
        if backend == 'nccl':
            torch.cuda.set_device(local)
        dist.init_process_group(backend=backend)
    return dist


def barrier(dist):
    if dist is not None:
        dist.barrier()


def reduce_run(dist, work, seconds):
    """(total work over ranks, max seconds over ranks)."""
    if dist is None:
        return float(work), float(seconds)
    import torch
    dev = 'cuda' if dist.get_backend() == 'nccl' else 'cpu'
    t = torch.tensor([float(work), float(seconds)], dtype=torch.float64, device=dev)
    w = t[:1].clone()
    s = t[1:].clone()
    dist.all_reduce(w, op=dist.ReduceOp.SUM)
    dist.all_reduce(s, op=dist.ReduceOp.MAX)
    return float(w.item()), float(s.item())
