"""Host-side sharding of the scorers over ranks, one process per GPU.

Pairs are independent, so a choice list splits into contiguous shards with no
exchange on the data path: cdist writes each shard's columns in place, and
extract / extractOne need one host-side merge of the per-shard best lists.  The
merge keeps the reference's order (README.md:153-214): best score first, ties by
the lower choice index, or by the later index for extractOne's `score >= best`
loop (tie_last).  torch.distributed carries the small per-shard lists (any
backend: gloo on CPU, nccl on GPUs); nothing here touches a device.
"""
import numpy as np


def shard_bounds(n, world):
    """[(start, stop)] of `world` contiguous shards of n items, sizes differing by at most 1"""
    base, extra = divmod(int(n), int(world))
    out, start = [], 0
    for r in range(world):
        stop = start + base + (1 if r < extra else 0)
        out.append((start, stop))
        start = stop
    return out


def shard_of(n, rank, world):
    return shard_bounds(n, world)[rank]


def merge_extract(parts, limit, higher_is_better, tie_last=False):
    """Merge per-shard extract results.

    parts: [(index int64 [nq, L], score float64 [nq, L], count int32 [nq])] with GLOBAL
    choice indices (entries past count[q] ignored).  Returns the same triple for the
    whole list with `limit` columns, -1 / 0.0 past count."""
    nq = parts[0][0].shape[0]
    idx = np.full((nq, limit), -1, dtype=np.int64)
    sc = np.zeros((nq, limit), dtype=np.float64)
    cnt = np.zeros(nq, dtype=np.int32)
    for q in range(nq):
        ii = np.concatenate([p[0][q, :p[2][q]] for p in parts]).astype(np.int64)
        ss = np.concatenate([p[1][q, :p[2][q]] for p in parts]).astype(np.float64)
        key = -ss if higher_is_better else ss
        tie = -ii if tie_last else ii
        order = np.lexsort((tie, key))[:limit]
        k = len(order)
        idx[q, :k] = ii[order]
        sc[q, :k] = ss[order]
        cnt[q] = k
    return idx, sc, cnt


def gather_extract(local, start, limit, higher_is_better, tie_last=False, group=None):
    """All ranks: offset the local shard's indices by `start`, gather every shard's
    result and merge.  local = (index, score, count) of this rank's shard."""
    import torch.distributed as dist
    i, s, c = local
    i = np.where(i >= 0, i + int(start), -1)
    mine = (i, np.asarray(s, dtype=np.float64), np.asarray(c, dtype=np.int32))
    world = dist.get_world_size(group)
    parts = [None] * world
    dist.all_gather_object(parts, mine, group=group)
    return merge_extract(parts, limit, higher_is_better, tie_last)


def max_over_ranks(value, device=None, group=None):
    """The maximum of a per-rank float (timings: a job is as slow as its slowest rank)"""
    import torch
    import torch.distributed as dist
    if not dist.is_initialized() or dist.get_world_size(group) == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX, group=group)
    return float(t.item())
