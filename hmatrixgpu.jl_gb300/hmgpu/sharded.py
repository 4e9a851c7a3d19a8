"""Products of one H-matrix split over the ranks of a torch.distributed group.

The reference's product writes every row of the permuted output once
(src/mult.jl:144), so rows shard across GPUs with no reduction of y. Rank r
holds shard r (hmgpu_hmatrix_shard): a contiguous range of permuted rows.
Before each product the ranks all-gather x in the permuted source order, each
contributing the slice it owns; a rank then computes its rows of y, again in
the permuted order. In an iterative solver the next x slice is made from the
local y rows, so the one collective per product is the gather of x.

Ownership of x: for a square H-matrix whose two trees are the same, rank r
owns the same permuted range of x as of y; otherwise x is split evenly. The
gather runs over whatever backend the group has (gloo: host tensors, nccl:
device tensors); remote slices land in this rank's own buffer before the
product reads them.
"""
import numpy as np


def even_splits(n, world):
    """[0, n) cut into `world` near-equal contiguous ranges, as (begin, end) pairs."""
    return [(n * r // world, n * (r + 1) // world) for r in range(world)]


def allgather_ranges(local, group=None):
    """The (begin, end) pair of every rank, in rank order."""
    import torch
    import torch.distributed as dist
    world = dist.get_world_size(group)
    dev = _comm_device(group)
    mine = torch.tensor([int(local[0]), int(local[1])], dtype=torch.int64, device=dev)
    out = [torch.empty(2, dtype=torch.int64, device=dev) for _ in range(world)]
    dist.all_gather(out, mine, group=group)
    return [(int(t[0]), int(t[1])) for t in out]


def _comm_device(group=None):
    import torch
    import torch.distributed as dist
    if dist.get_backend(group) == "nccl":
        return torch.device("cuda", torch.cuda.current_device())
    return torch.device("cpu")


def gather_slices(local, splits, group=None):
    """All-gather of a vector cut into `splits`: every rank passes its own
    slice (length end - begin of its split) and gets the whole vector, slices
    in rank order. Slices may differ in length; they travel padded to the
    longest one. Returns a tensor on the communication device."""
    import torch
    import torch.distributed as dist
    rank = dist.get_rank(group)
    b, e = splits[rank]
    if local.numel() != e - b:
        raise ValueError(f"rank {rank} holds {local.numel()} entries, its split has {e - b}")
    dev = _comm_device(group)
    width = max(hi - lo for lo, hi in splits)
    buf = torch.zeros(width, dtype=local.dtype, device=dev)
    buf[: e - b] = local.to(dev)
    parts = [torch.empty(width, dtype=local.dtype, device=dev) for _ in splits]
    dist.all_gather(parts, buf, group=group)
    return torch.cat([p[: hi - lo] for p, (lo, hi) in zip(parts, splits)])


class ShardedProduct:
    """y = H x with H's rows split over the group's ranks, one GPU per rank.

    `H` is the whole H-matrix on this rank's GPU (each rank builds or loads the
    same one; its shard copies only what the rank needs, after which H may be
    dropped). mul(x_rows) takes this rank's slice of x in the permuted source
    order (`x_splits[rank]`) and returns this rank's rows of y in the permuted
    target order (`row_splits[rank]`)."""

    def __init__(self, H, group=None):
        import torch.distributed as dist
        self.group = group
        self.rank = dist.get_rank(group)
        self.world = dist.get_world_size(group)
        self.shard = H.shard(self.rank, self.world)
        self.shape = H.shape
        self.row_splits = allgather_ranges(self.shard.rows, group)
        m, n = H.shape
        self.x_splits = self.row_splits if m == n else even_splits(n, self.world)

    def mul(self, x_rows):
        import torch
        x_full = gather_slices(x_rows, self.x_splits, self.group).to(x_rows.device)
        b, e = self.row_splits[self.rank]
        y = torch.empty(e - b, dtype=x_rows.dtype, device=x_rows.device)
        return self.shard.mul_permuted(y, x_full.contiguous())
