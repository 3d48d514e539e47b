"""Several GPUs, one process each: the screen shards by star and the pair Monte Carlo by pair.

Every rank screens (or traces) its own contiguous block of the input with the whole cluster table resident on its own
GPU; no device data crosses ranks.  The only exchange is host-side: rank 0 collects the per-rank results in rank
order, which is the single-GPU order (rows in (star, cluster) order, pairs in input order), over any
torch.distributed process group (NCCL between GPU ranks, gloo on CPU).

    lo, hi = block_range(len(stars), world, rank)
    rows = ctx.screen(*draw_targets(stars[lo:hi]), tmax)          # star indices local to the block
    all_rows = gather_rows(rows, lo)                              # on rank 0, stars renumbered globally
"""
import numpy as np


def block_range(n, world, rank):
    """[lo, hi) of `rank` when n items are split into `world` contiguous blocks whose sizes differ by at most 1."""
    if world <= 0 or not 0 <= rank < world or n < 0:
        raise ValueError("block_range(%r, %r, %r)" % (n, world, rank))
    q, r = divmod(n, world)
    lo = rank * q + min(rank, r)
    return lo, lo + q + (1 if rank < r else 0)


def gather_records(arr, group=None, dst=0):
    """Concatenate a numpy array from every rank of `group`, in rank order, on rank `dst` (None on the others)."""
    import torch.distributed as dist
    me = dist.get_rank(group)
    objs = [None] * dist.get_world_size(group) if me == dst else None
    dist.gather_object(np.ascontiguousarray(arr), objs, dst=dst, group=group)
    if me != dst:
        return None
    return np.concatenate(objs) if objs else np.ascontiguousarray(arr)[:0]


def gather_rows(rows, first_star, group=None, dst=0):
    """Screen rows of this rank's star block (star indices local to it, as pgx_screen returns them) -> all ranks'
    rows on `dst`, star indices global: the rows one GPU gives for the whole star list."""
    rows = np.array(rows, copy=True)
    rows["star"] += first_star
    return gather_records(rows, group, dst)


def gather_pairs(results, group=None, dst=0):
    """pgx_pair results of this rank's pair block -> all ranks' results on `dst`, in input order."""
    return gather_records(results, group, dst)
