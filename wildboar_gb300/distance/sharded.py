"""Row-sharded distance calls across the ranks of a process group.

The distance path has no exchange step inside it: every (x_i, y_j) pair, every
query's k-nearest search and every (series, shapelet) scan is independent.
A world of N ranks (one GPU each) therefore splits the *rows of x* into N
contiguous blocks, replicates y (or the shapelets), runs the single-GPU call
on its block and concatenates the blocks with one all_gather at the end.
Sharding the query rows keeps argmin bit-exact with the reference, including
its heap order: each query's whole candidate loop (distance/_cdistance.pyx:
1270-1378) runs on one rank.

``compute`` is the per-rank call; it defaults to the GPU drop-in and exists
so that the exchange logic can be exercised on CPU ranks (gloo) with another
implementation of the same contract.
"""

import numpy as np


def shard_bounds(n, rank, world):
    """Contiguous block [start, stop) of n rows owned by `rank` of `world`.

    The first n % world ranks own one extra row, so block sizes differ by at
    most one and the blocks tile [0, n) in rank order.
    """
    if world < 1 or not 0 <= rank < world:
        raise ValueError("rank must be in [0, world)")
    if n < 0:
        raise ValueError("n must be >= 0")
    base, extra = divmod(n, world)
    start = rank * base + min(rank, extra)
    stop = start + base + (1 if rank < extra else 0)
    return start, stop


def _gather_rows(block, n_total, group=None):
    """all_gather of per-rank row blocks (numpy, float64 or int64) into the
    full (n_total, ...) array on every rank."""
    import torch
    import torch.distributed as dist

    world = dist.get_world_size(group)
    block = np.ascontiguousarray(block)
    tail = block.shape[1:]
    rows = max(shard_bounds(n_total, r, world)[1] - shard_bounds(n_total, r, world)[0]
               for r in range(world))
    buf = np.zeros((rows,) + tail, dtype=block.dtype)
    buf[: block.shape[0]] = block
    t = torch.from_numpy(buf)
    backend = dist.get_backend(group)
    if backend == "nccl":
        t = t.cuda()
    parts = [torch.empty_like(t) for _ in range(world)]
    dist.all_gather(parts, t, group=group)
    out = []
    for r in range(world):
        s0, s1 = shard_bounds(n_total, r, world)
        out.append(parts[r][: s1 - s0].cpu().numpy())
    return np.concatenate(out, axis=0)


def max_over_ranks(value, group=None):
    """Largest of one float per rank (the step time of a weak-scaling run)."""
    import torch
    import torch.distributed as dist

    t = torch.tensor([float(value)], dtype=torch.float64)
    if dist.get_backend(group) == "nccl":
        t = t.cuda()
    dist.all_reduce(t, op=dist.ReduceOp.MAX, group=group)
    return float(t.item())


def pairwise_distance(x, y, *, group=None, compute=None, **kwargs):
    """``pairwise_distance(x, y, **kwargs)`` with the rows of x sharded over
    the ranks of `group`; every rank returns the full (n_x, n_y) matrix.

    x: (n_x, n_timestep) or (n_x, n_dims, n_timestep) numpy array; y likewise
    (not sharded).  Only integer ``dim`` values keep the row axis first and
    are accepted.
    """
    import torch.distributed as dist

    if compute is None:
        from ._distance import pairwise_distance as compute
    dim = kwargs.get("dim", 0)
    if not isinstance(dim, (int, np.integer)):
        raise ValueError("sharded pairwise_distance takes an integer dim")
    x = np.asarray(x)
    if x.ndim < 2:
        raise ValueError("x must hold several series (2-D or 3-D)")
    s0, s1 = shard_bounds(x.shape[0], dist.get_rank(group), dist.get_world_size(group))
    part = np.asarray(compute(x[s0:s1], y, **kwargs), dtype=np.float64)
    part = part.reshape(s1 - s0, -1)
    return _gather_rows(part, x.shape[0], group)


def argmin_distance(x, y, *, k=1, group=None, compute=None, **kwargs):
    """``argmin_distance(x, y, k=k, return_distance=True, **kwargs)`` with the
    queries (rows of x) sharded over the ranks of `group`.

    Returns (indices, distances), each (n_x, k), on every rank; indices are
    positions in y, in the order the single-GPU call returns them.
    """
    import torch.distributed as dist

    if compute is None:
        from ._distance import argmin_distance as compute
    x = np.asarray(x)
    s0, s1 = shard_bounds(x.shape[0], dist.get_rank(group), dist.get_world_size(group))
    idx, dist_ = compute(x[s0:s1], y, k=k, return_distance=True, **kwargs)
    idx = np.asarray(idx, dtype=np.int64).reshape(s1 - s0, k)
    dist_ = np.asarray(dist_, dtype=np.float64).reshape(s1 - s0, k)
    return (_gather_rows(idx, x.shape[0], group).astype(np.intp),
            _gather_rows(dist_, x.shape[0], group))


def pairwise_subsequence_distance(y, x, *, group=None, compute=None, **kwargs):
    """``pairwise_subsequence_distance(y, x, **kwargs)`` with the series (rows
    of x) sharded over the ranks of `group`; y (the subsequences) is
    replicated.  Returns the full (n_x, n_y) distances, and the (n_x, n_y)
    indices when ``return_index=True``.
    """
    import torch.distributed as dist

    if compute is None:
        from ._distance import pairwise_subsequence_distance as compute
    x = np.asarray(x)
    s0, s1 = shard_bounds(x.shape[0], dist.get_rank(group), dist.get_world_size(group))
    res = compute(y, x[s0:s1], **kwargs)
    n_y = len(y) if isinstance(y, (list, tuple)) else np.asarray(y).shape[0]
    if kwargs.get("return_index", False):
        d, i = res
        d = np.asarray(d, dtype=np.float64).reshape(s1 - s0, n_y)
        i = np.asarray(i, dtype=np.int64).reshape(s1 - s0, n_y)
        return (_gather_rows(d, x.shape[0], group),
                _gather_rows(i, x.shape[0], group).astype(np.intp))
    d = np.asarray(res, dtype=np.float64).reshape(s1 - s0, n_y)
    return _gather_rows(d, x.shape[0], group)
