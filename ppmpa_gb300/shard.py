"""Progressive rendering sharded by passes over ranks (one GPU per rank).

PA passes are independent given their index: pass k's radius is the
schedule's k-th value and its random streams are keyed by k.  Rank r
renders a contiguous block of pass indices (RenderConfig.first_pass), and
one FP64 sum of the ranks' image sums, divided by the total pass count, is
the image a single GPU rendering all passes produces (up to the order of the
final sum).  The reduction is the only collective; no pass exchanges data.
"""
from dataclasses import replace

import numpy as np


def shard_passes(total: int, rank: int, world: int):
    """(first, count): contiguous blocks, the first total % world ranks one longer."""
    if world < 1 or not 0 <= rank < world or total < 0:
        raise ValueError(f"bad shard {rank}/{world} of {total} passes")
    base, extra = divmod(total, world)
    count = base + (1 if rank < extra else 0)
    first = rank * base + min(rank, extra)
    return first, count


def render_sharded(render_passes, total_passes: int, rank: int, world: int, reduce_sum=None):
    """render_passes(first, count) -> FP64 sum image of passes first..first+count-1;
    reduce_sum(array) -> the sum over ranks on rank 0 (None with one rank).
    Returns the averaged image on rank 0, None elsewhere."""
    first, count = shard_passes(total_passes, rank, world)
    part = render_passes(first, count) if count else None
    if world > 1:
        if part is None:
            raise ValueError("every rank needs at least one pass")
        part = reduce_sum(part)
    if rank != 0:
        return None
    return part / float(total_passes)


def context_renderer(ctx, cfg):
    """render_passes for a Context and RenderConfig (its passes field is ignored)."""
    def run(first, count):
        ctx.render_begin(replace(cfg, passes=count, first_pass=cfg.first_pass + first))
        ctx.render_step(count)
        return ctx.render_image() * float(count)
    return run


def torch_reduce_sum(group=None):
    """reduce_sum over torch.distributed (gloo or nccl), FP64, to rank 0."""
    import torch
    import torch.distributed as dist

    def red(a):
        dev = "cuda" if dist.get_backend(group) == "nccl" else "cpu"
        t = torch.from_numpy(np.ascontiguousarray(a, np.float64)).to(dev)
        dist.reduce(t, dst=0, op=dist.ReduceOp.SUM, group=group)
        return t.cpu().numpy()
    return red
