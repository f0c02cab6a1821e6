"""64 queries of the 4,096-query batched workload at their full mesh sizes
(levels 1-5, 10-10,000 meshes per side), run as batched waves (partitioned
datasets, one captured graph per wave), against the oracle's stored pair
sets (tests/golden/pairs_batched_64.npz, from make_golden.py --batched)."""
from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLD = Path(__file__).resolve().parent / "golden" / "pairs_batched_64.npz"


def test_batched_subset_matches_oracle(ctx):
    from pierce_gb300 import batched as BT
    from pierce_gb300 import join as J
    gold = np.load(GOLD)
    qs_all = BT.workload(seed=3, queries=4096)
    picked = [int(i) for i in gold["queries"]]
    qs = [qs_all[i] for i in picked]
    waves = BT.make_waves(qs, budget_tris=0.6e9)

    def opts_fn(w):
        return J.make_opts(predicate="overlap", expected_pairs=BT.expected_pairs(w))

    res = BT.run_batched(ctx, waves, opts_fn, warmup=0, replays=1, keep_pairs=True)
    empty = np.zeros((0, 2), np.int32)
    bad = []
    for local, q in enumerate(picked):
        got = np.sort(J.pairs_to_keys(res["results"].get(local, empty)))
        want = gold[f"q{q}"]
        if not np.array_equal(got, want):
            bad.append((q, len(got), len(want)))
    assert not bad, bad
    assert sum(len(gold[f"q{q}"]) for q in picked) > 1000
    ctx.release_scratch()
