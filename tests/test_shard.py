"""Joins split across processes (pierce_gb300/shard.py), on the CPU over
gloo with world size 2.

Each rank traces a contiguous range of both datasets' edge lists -- the
split the library applies to a join's ray list -- here through the CPU
oracle, which stands in for the GPU join of the rank; the ranks' pairs are
all-gathered (unequal counts) and de-duplicated.  The union must equal the
unsplit join."""
import os
import socket
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _edge_shard(G, rank, world):
    import pierce_gb300 as pg
    n = G.num_edges
    lo, hi = n * rank // world, n * (rank + 1) // world
    sub = pg.Geometry.from_arrays(G.vertices, G.indices, G.tri_to_object)
    sub.set_edges(G.edge_starts[lo:hi], G.edge_ends[lo:hi], G.edge_src[lo:hi])
    return sub


def _cases():
    import pierce_gb300 as pg
    return (pg.icospheres(101, 120, 2, hi=30.0), pg.icospheres(202, 120, 2, hi=30.0))


def _worker(rank, world, port, out):
    sys.path.insert(0, str(ROOT))
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    import torch.distributed as dist
    from oracle import pyoracle as O
    from pierce_gb300 import join as J
    from pierce_gb300 import shard as SH
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        A, B = _cases()
        keys, _ = O.overlap_keys(_edge_shard(A, rank, world), _edge_shard(B, rank, world))
        local = np.stack([(keys >> np.uint64(32)).astype(np.int32),
                          (keys & np.uint64(0xFFFFFFFF)).astype(np.int32)], 1) if len(keys) else \
            np.zeros((0, 2), np.int32)
        merged = SH.unique_pairs(SH.gather_pairs(local))
        out.put((rank, len(local), J.pairs_to_keys(merged).tolist()))
    finally:
        dist.destroy_process_group()


def test_sharded_overlap_union_equals_join_gloo_world2():
    torch = pytest.importorskip("torch")
    sys.path.insert(0, str(ROOT))
    from oracle import pyoracle as O
    O.build()
    A, B = _cases()
    want, _ = O.overlap_keys(A, B)
    assert len(want) > 20
    mp = torch.multiprocessing.get_context("spawn")
    q = mp.Queue()
    port = _free_port()
    procs = [mp.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = {}
    for _ in procs:
        r, n_local, merged = q.get(timeout=300)
        got[r] = (n_local, merged)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for r in range(2):
        assert got[r][1] == want.tolist()
    # each shard alone misses pairs: the split is real
    assert all(got[r][0] < len(want) for r in range(2))


def test_unique_pairs_and_shard_opts():
    sys.path.insert(0, str(ROOT))
    from pierce_gb300 import join as J
    from pierce_gb300 import shard as SH
    p = np.array([[3, 1], [0, 2], [3, 1], [0, -1], [2**31 - 1, 0]], np.int32)
    u = SH.unique_pairs(p)
    # b compares unsigned, as in the library's (a << 32 | b) keys
    assert u.tolist() == [[0, 2], [0, -1], [3, 1], [2**31 - 1, 0]]
    o = SH.shard_opts(J.make_opts(), 2, 4)
    assert (o.shard_index, o.shard_count) == (2, 4)
    o1 = SH.shard_opts(J.make_opts(), 0, 1)
    assert (o1.shard_index, o1.shard_count) == (0, 1)
