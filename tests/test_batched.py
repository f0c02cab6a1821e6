"""Batches of independent joins: partitioned datasets joined in one pass
must return, per partition, exactly the pairs of the stand-alone join of
that partition -- never a pair across partitions, although all partitions
share one coordinate cube here so cross pairs would exist otherwise."""
import numpy as np
import pytest

import pierce_gb300 as pg

pytestmark = pytest.mark.gpu


def batch(seed, q, lo_n=0, hi_n=40, extent=40.0):
    rng = np.random.default_rng(seed)
    side = []
    for s in range(2):
        parts = []
        for g in range(q):
            n = int(rng.integers(lo_n, hi_n + 1))
            inst = pg.instances(int(rng.integers(1, 2**62)), n, int(rng.integers(0, 2)), 0, 3, hi=extent)
            inst["group"] = g
            parts.append(inst)
        side.append(parts)
    return side


def concat(parts):
    return np.concatenate(parts) if parts else np.zeros(0, dtype=pg.capi.INSTANCE_DTYPE)


def split(pairs, offs_a, offs_b):
    """Global pairs -> {query: local pairs}, checking no pair crosses queries."""
    qa = np.searchsorted(offs_a, pairs[:, 0], side="right") - 1
    qb = np.searchsorted(offs_b, pairs[:, 1], side="right") - 1
    assert np.array_equal(qa, qb), "pair across partitions"
    out = {}
    for q in np.unique(qa):
        sel = pairs[qa == q]
        out[int(q)] = np.stack([sel[:, 0] - offs_a[q], sel[:, 1] - offs_b[q]], 1)
    return out


@pytest.fixture(scope="module")
def case(ctx):
    from pierce_gb300 import join as J
    A_parts, B_parts = batch(5, 12)
    # query 3: empty A side; query 7: a single mesh on each side
    A_parts[3] = A_parts[3][:0]
    A_parts[7], B_parts[7] = A_parts[7][:1], B_parts[7][:1]
    offs_a = np.concatenate([[0], np.cumsum([len(p) for p in A_parts])])
    offs_b = np.concatenate([[0], np.cumsum([len(p) for p in B_parts])])
    singles = []
    for a, b in zip(A_parts, B_parts):
        a0, b0 = a.copy(), b.copy()
        a0["group"], b0["group"] = 0, 0
        singles.append((a0, b0))
    return A_parts, B_parts, offs_a, offs_b, singles


@pytest.mark.parametrize("leaf", [1, 8])
@pytest.mark.parametrize("active_bvh", [True, False])
@pytest.mark.parametrize("predicate,sizing", [("overlap", "hash"), ("overlap", "two_pass"),
                                              ("intersection", "hash")])
def test_batched_join_equals_per_query_joins(ctx, case, leaf, active_bvh, predicate, sizing):
    from pierce_gb300 import join as J
    A_parts, B_parts, offs_a, offs_b, singles = case
    t = J.default_tuning(leaf_size=leaf)
    A = J.Dataset.from_instances(ctx, concat(A_parts), t)
    B = J.Dataset.from_instances(ctx, concat(B_parts), t)
    assert A.info().num_parts == 12 and B.info().num_parts == 12
    got = J.join(ctx, A, B, predicate=predicate, sizing=sizing, active_bvh=active_bvh)
    per_q = split(got.pairs, offs_a, offs_b)
    total = 0
    for q, (ia, ib) in enumerate(singles):
        if len(ia) == 0 or len(ib) == 0:
            assert q not in per_q
            continue
        a1 = J.Dataset.from_instances(ctx, ia, t)
        b1 = J.Dataset.from_instances(ctx, ib, t)
        want = J.join(ctx, a1, b1, predicate=predicate, sizing="two_pass").pairs
        have = per_q.get(q, np.zeros((0, 2), np.int32))
        assert np.array_equal(have, want), f"query {q}"
        total += len(want)
    assert total == len(got.pairs) and total > 20


def test_batched_join_matches_oracle(ctx, case):
    from pierce_gb300 import join as J
    from oracle import pyoracle as O
    A_parts, B_parts, offs_a, offs_b, singles = case
    A = J.Dataset.from_instances(ctx, concat(A_parts))
    B = J.Dataset.from_instances(ctx, concat(B_parts))
    per_q = split(J.intersection_join(ctx, A, B).pairs, offs_a, offs_b)
    for q in (0, 5, 11):
        ia, ib = singles[q]
        want = O.intersection_keys(pg.expand_instances(ia), pg.expand_instances(ib))
        have = J.pairs_to_keys(per_q.get(q, np.zeros((0, 2), np.int32)))
        assert np.array_equal(np.sort(have), np.sort(want)), f"query {q}"


def test_partition_count_mismatch_is_rejected(ctx, case):
    from pierce_gb300 import join as J
    A_parts, B_parts, *_ = case
    A = J.Dataset.from_instances(ctx, concat(A_parts))
    b = concat(B_parts).copy()
    b["group"] = 0
    B = J.Dataset.from_instances(ctx, b)
    with pytest.raises(Exception):
        J.overlap_join(ctx, A, B)
    # explicit re-partitioning through the C ABI makes them compatible
    B.set_partitions(concat(B_parts)["group"], 12)
    r = J.overlap_join(ctx, A, B)
    assert len(r.pairs) > 0


@pytest.mark.parametrize("level,leaf", [(1, 4), (0, 8), (0, 4)])
def test_partitions_by_object_equal_filtered_join(ctx, level, leaf):
    """Objects dealt round-robin into 3 partitions of one dataset: the
    partitioned join equals the unpartitioned join restricted to pairs
    within one partition.  Level-0 meshes (20 triangles) with leaves of 8 put
    groups across objects of different partitions, which takes the fallback
    over the surviving triangles; the other cases take the group path."""
    from pierce_gb300 import join as J
    A = pg.icospheres(31, 300, level, hi=30.0)
    B = pg.icospheres(32, 300, level, hi=30.0)
    t = J.default_tuning(leaf_size=leaf)
    for predicate in ("overlap", "intersection"):
        da, db = J.Dataset.from_geometry(ctx, A, t), J.Dataset.from_geometry(ctx, B, t)
        full = J.join(ctx, da, db, predicate=predicate).pairs
        pa, pb = np.arange(A.num_objects) % 3, np.arange(B.num_objects) % 3
        da.set_partitions(pa, 3)
        db.set_partitions(pb, 3)
        got = J.join(ctx, da, db, predicate=predicate).pairs
        want = full[pa[full[:, 0]] == pb[full[:, 1]]]
        assert np.array_equal(got, want), predicate
        assert len(want) > 20
        da.close()
        db.close()
