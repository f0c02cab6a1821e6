"""Sharded joins on one GPU: the shards of a join run one after another
(each a complete join call with shard_index = k of shard_count), and their
union must equal the unsplit join and the oracle.  Containment shards are
split by B object, so they are disjoint."""
import ctypes as C

import numpy as np
import pytest

import pierce_gb300 as pg
from pierce_gb300 import capi
from pierce_gb300 import join as J
from pierce_gb300 import shard as SH
from oracle import pyoracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def pair():
    return pg.ellipsoid_pair(8, 9, 250, 250, 2, lo=0, hi=60, frac_contact=0.1)


def datasets(ctx, A, B, edges=True):
    t = J.default_tuning(defer_build=1, skip_edges=0 if edges else 1)
    return J.Dataset.from_geometry(ctx, A, t), J.Dataset.from_geometry(ctx, B, t)


@pytest.mark.parametrize("predicate", ["overlap", "intersection", "containment"])
@pytest.mark.parametrize("world", [2, 3])
@pytest.mark.parametrize("sizing", ["hash", "two_pass"])
def test_shard_union_equals_join(ctx, pair, predicate, world, sizing):
    A, B = pair
    want = {"overlap": lambda: O.overlap_keys(A, B)[0], "intersection": lambda: O.intersection_keys(A, B),
            "containment": lambda: O.containment_keys(A, B)}[predicate]()
    da, db = datasets(ctx, A, B)
    base = J.make_opts(predicate=predicate, sizing=sizing)
    whole_run = J.run_join(ctx, da, db, base)
    whole = J.pairs_to_keys(whole_run.pairs)
    assert np.array_equal(whole, want)
    runs = [J.run_join(ctx, da, db, SH.shard_opts(base, k, world)) for k in range(world)]
    parts = [J.pairs_to_keys(r.pairs) for r in runs]
    union = np.unique(np.concatenate(parts))
    assert np.array_equal(union, want), (predicate, world)
    if predicate == "containment":
        assert sum(len(p) for p in parts) == len(want)  # disjoint by B object
    else:
        # every ray and every parity ray is traced by exactly one shard
        for key in ("rays", "parity_rays"):
            assert sum(r.stats[key] for r in runs) == whole_run.stats[key], key
        assert all(0 < r.stats["rays"] < whole_run.stats["rays"] for r in runs)


def test_shard_merge_on_device(ctx, pair):
    A, B = pair
    da, db = datasets(ctx, A, B, edges=False)
    base = J.make_opts(predicate="intersection")
    parts = [J.run_join(ctx, da, db, SH.shard_opts(base, k, 4)).pairs for k in range(4)]
    merged = SH.merge_on_device(ctx, np.concatenate(parts))
    assert np.array_equal(J.pairs_to_keys(merged), O.intersection_keys(A, B))


def test_plain_form_shards(ctx, pair):
    """Unlisted rays (the plain form over the dataset's own hierarchies)
    split by edge index."""
    A, B = pair
    da, db = datasets(ctx, A, B)
    da.build(J.default_tuning(leaf_size=4))
    db.build(J.default_tuning(leaf_size=4))
    plain = J.make_opts(predicate="overlap", sizing="two_pass", precision="fp32", cull_objects=False,
                        defer_exact=False, active_bvh=False)
    whole = J.pairs_to_keys(J.run_join(ctx, da, db, plain).pairs)
    parts = [J.pairs_to_keys(J.run_join(ctx, da, db, SH.shard_opts(plain, k, 3)).pairs) for k in range(3)]
    assert np.array_equal(np.unique(np.concatenate(parts)), whole)


def test_shard_arguments_checked(ctx, pair):
    A, B = pair
    da, db = datasets(ctx, A, B)
    L = capi.lib()
    r = C.c_void_p()
    for kw in ({"shard_index": 3, "shard_count": 3}, {"shard_index": -1, "shard_count": 2},
               {"shard_index": 1, "shard_count": 1},
               {"predicate": "containment", "include_overlap_pairs": True, "shard_index": 0, "shard_count": 2}):
        o = J.make_opts(**kw)
        assert L.pierce_join(ctx.handle, da.handle, db.handle, C.byref(o), C.byref(r), None) == \
            capi.ERR_INVALID_ARGUMENT, kw
