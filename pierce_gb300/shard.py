"""Joins split across processes, one process per GPU.

Every rank holds both datasets and runs the same join with
``shard_index = rank, shard_count = world`` (``pierce_join_opts``): each edge
ray belongs to one rank by a hash of its segment's endpoints (rays from the
kept triangles) or by its range of edge indices (the dataset's edges), never
by its position in a ray list, whose order differs from run to run; the
parity rays are split into ranges of source objects.  The union of the
ranks' pair sets is the join's pair set; containment is split by B object,
which makes the ranks' pair sets disjoint.  The one exchange is at the end:
an all-gather of each rank's pairs (variable counts, padded to the largest)
and a sort + unique of the union.

The reference runs one process on one GPU (its launches cover every edge,
pierce/query/src/raytracing/MeshOverlapEdgesLauncher.cpp:140-154); the
units it launches over -- one ray per edge, one parity ray per object --
are independent, which is what makes these ranges a valid split.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import capi
from .join import JoinResult, run_join


def shard_opts(opts: capi.JoinOpts, rank: int, world: int) -> capi.JoinOpts:
    o = capi.JoinOpts.from_buffer_copy(opts)
    o.shard_index, o.shard_count = (int(rank), int(world)) if world > 1 else (0, 1)
    return o


def gather_pairs(local: np.ndarray, group=None) -> np.ndarray:
    """All ranks' (a, b) pairs (int32, shape (n, 2)), concatenated in rank
    order, on every rank.  Counts differ per rank: they are exchanged first
    and every rank's block is padded to the largest."""
    import torch
    import torch.distributed as dist
    world = dist.get_world_size(group)
    nccl = dist.get_backend(group) == "nccl"
    dev = torch.device("cuda", torch.cuda.current_device()) if nccl else torch.device("cpu")
    flat = torch.from_numpy(np.ascontiguousarray(local, dtype=np.int32).reshape(-1).view(np.int64).copy()).to(dev)
    n = torch.tensor([flat.numel()], dtype=torch.int64, device=dev)
    sizes = [torch.zeros_like(n) for _ in range(world)]
    dist.all_gather(sizes, n, group=group)
    counts = [int(x.item()) for x in sizes]
    padded = torch.zeros(max(max(counts), 1), dtype=torch.int64, device=dev)
    padded[: flat.numel()] = flat
    blocks = [torch.empty_like(padded) for _ in range(world)]
    dist.all_gather(blocks, padded, group=group)
    parts = [blocks[r][: counts[r]].cpu().numpy() for r in range(world)]
    allp = np.concatenate(parts) if parts else np.zeros(0, np.int64)
    return allp.view(np.int32).reshape(-1, 2)


def unique_pairs(pairs: np.ndarray) -> np.ndarray:
    """Sorted by the key (a << 32 | b) -- by a, then b as unsigned, the
    library's order -- with duplicates removed."""
    if len(pairs) == 0:
        return np.zeros((0, 2), np.int32)
    keys = (pairs[:, 0].astype(np.int64) << 32) | (pairs[:, 1].astype(np.int64) & 0xFFFFFFFF)
    u = np.unique(keys)
    return np.stack([(u >> 32).astype(np.int32), (u & 0xFFFFFFFF).astype(np.uint32).view(np.int32)], 1)


def merge_on_device(ctx, pairs: np.ndarray) -> np.ndarray:
    """Sort + unique of gathered pairs with the library's de-duplication
    (pierce_merge_and_deduplicate_pairs) on the context's device."""
    import torch
    if len(pairs) == 0:
        return np.zeros((0, 2), np.int32)
    d_in = torch.from_numpy(np.ascontiguousarray(pairs, dtype=np.int32)).to(torch.device("cuda", ctx.device))
    d_out = torch.empty_like(d_in)
    nu = C.c_int64()
    torch.cuda.synchronize(ctx.device)
    capi.check(capi.lib().pierce_merge_and_deduplicate_pairs(ctx.handle, d_in.data_ptr(), len(pairs), None, 0,
                                                              d_out.data_ptr(), C.byref(nu)), "merge shards")
    return d_out[: nu.value].cpu().numpy()


def sharded_join(ctx, a, b, opts: capi.JoinOpts, group=None) -> JoinResult:
    """The join of a and b split over the ranks of `group` (each rank
    passes its own context and its replicas of the datasets); every rank
    returns the whole sorted pair set.  Stats are this rank's."""
    import torch.distributed as dist
    rank, world = dist.get_rank(group), dist.get_world_size(group)
    local = run_join(ctx, a, b, shard_opts(opts, rank, world))
    gathered = gather_pairs(local.pairs, group)
    merged = merge_on_device(ctx, gathered) if dist.get_backend(group) == "nccl" else unique_pairs(gathered)
    return JoinResult(merged, local.stats, local.containment_count)
