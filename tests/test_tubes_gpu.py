"""The large tube-mesh overlap join at its full size (2,000 tubes of about
200k triangles against 100,000 ellipsoids, the benchmark's default
workload), checked against the oracle.

The oracle cannot join 400 M triangles in test time, so its pair set is
stored for the first 50 tubes against every ellipsoid that can meet them
(tests/golden/pairs_tubes_head50.npz, from make_golden.py --tubes): the
full join's pairs of tubes 0..49 must equal it bit for bit.  The whole pair
set must be the same for the tuned form (learned sizing, culling, per-join
hierarchies), the exact hash form and the plain FP32 two-pass form."""
from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLD = Path(__file__).resolve().parent / "golden" / "pairs_tubes_head50.npz"


@pytest.fixture(scope="module")
def tube_datasets(ctx):
    import bench
    from pierce_gb300 import join as J
    t = J.default_tuning(defer_build=1)
    A = bench.tube_geometry()
    da = J.Dataset.from_geometry(ctx, A, t)
    del A
    db = J.Dataset.from_instances(ctx, bench.ellipsoid_instances(), t)
    yield da, db
    da.close()
    db.close()
    ctx.release_scratch()


@pytest.fixture(scope="module")
def tuned_keys(ctx, tube_datasets):
    from pierce_gb300 import join as J
    from pierce_gb300 import sizing as S
    da, db = tube_datasets
    model = S.SizingModel.load(ctx, S.TRAINED_MODEL)
    r = J.run_join(ctx, da, db, J.make_opts(predicate="overlap", sizing="learned", sizing_model=model))
    return J.pairs_to_keys(r.pairs), r.stats


def test_tube_join_head_matches_oracle(tuned_keys):
    gold = np.load(GOLD)
    keys, stats = tuned_keys
    first = int(gold["first"])
    head = np.sort(keys[(keys >> np.uint64(32)) < np.uint64(first)])
    want = gold["overlap"]
    assert len(want) > 100
    assert np.array_equal(head, want), (len(head), len(want), len(np.setxor1d(head, want)))
    # the network over-predicts tube joins (their boxes meet nearly
    # everything: 67 M pairs predicted, 2^27 slots); the sampled incidence
    # cap brings the table down to 2^25 slots (268 MB) without falling back
    # to two-pass
    assert stats["sizing_overflow"] == 0
    assert stats["hash_slots"] <= 1 << 25, stats["hash_slots"]


def test_tube_join_forms_agree(ctx, tube_datasets, tuned_keys):
    from pierce_gb300 import join as J
    da, db = tube_datasets
    keys, _ = tuned_keys
    exact_hash = J.pairs_to_keys(J.run_join(ctx, da, db, J.make_opts(predicate="overlap", sizing="hash",
                                                                     expected_pairs=1 << 18)).pairs)
    assert np.array_equal(exact_hash, keys)
    ctx.release_scratch()
    plain = J.make_opts(predicate="overlap", sizing="two_pass", precision="fp32", cull_objects=False,
                        defer_exact=False, active_bvh=False)
    da.build(J.default_tuning(leaf_size=8))
    db.build(J.default_tuning(leaf_size=8))
    plain_keys = J.pairs_to_keys(J.run_join(ctx, da, db, plain).pairs)
    assert np.array_equal(plain_keys, keys)
