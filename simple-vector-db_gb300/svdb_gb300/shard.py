"""Row-range sharding of one store over several processes (one GPU each).

Each rank holds rows [offset, offset + n_local) of the global positional order
in its own VectorDatabase and answers a query batch with its local exact top-k;
`gather_topk` turns the local indices into global ones, gathers every rank's
lists (one all_gather of Q x k pairs -- the only exchange) and merges them into
the exact global top-k with ties to the lowest global index (svdb_merge_topk).
With torch.distributed on NCCL the tensors move between GPUs; on gloo (tests)
they stay on the host.
"""
from __future__ import annotations

import numpy as np


def shard_bounds(n_rows: int, world: int, rank: int) -> tuple[int, int]:
    """Contiguous row range [lo, hi) of `rank` among `world` near-equal shards."""
    lo = n_rows * rank // world
    hi = n_rows * (rank + 1) // world
    return lo, hi


def gather_topk(metric: int, local_ids: np.ndarray, local_vals: np.ndarray, offset: int, group=None):
    """Exact global top-k on every rank from each rank's local top-k.

    local_ids are indices within the rank's shard (-1 for missing); the
    result's ids are global positions."""
    import torch
    import torch.distributed as dist

    from . import merge_topk

    gids = np.where(local_ids >= 0, local_ids + offset, -1).astype(np.int64)
    world = dist.get_world_size(group)
    t_ids = torch.from_numpy(gids)
    t_vals = torch.from_numpy(np.ascontiguousarray(local_vals, np.float64))
    if dist.get_backend(group) == "nccl":
        t_ids, t_vals = t_ids.cuda(), t_vals.cuda()
    all_ids = [torch.empty_like(t_ids) for _ in range(world)]
    all_vals = [torch.empty_like(t_vals) for _ in range(world)]
    dist.all_gather(all_ids, t_ids, group=group)
    dist.all_gather(all_vals, t_vals, group=group)
    ids = np.stack([a.cpu().numpy() for a in all_ids])
    vals = np.stack([a.cpu().numpy() for a in all_vals])
    return merge_topk(metric, ids, vals)
