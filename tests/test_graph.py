"""Joins captured as CUDA graphs: every replay returns the eager join's
pairs and device counters, for single and partitioned (batched) joins."""
import numpy as np
import pytest

import pierce_gb300 as pg

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def datasets(ctx):
    from pierce_gb300 import join as J
    A = J.Dataset.from_instances(ctx, pg.instances(71, 800, pg.SPHERES, 1, 3, hi=80.0),
                                 J.default_tuning(leaf_size=4))
    B = J.Dataset.from_instances(ctx, pg.instances(72, 900, pg.ELLIPSOIDS, 1, 3, p0=1.0, p1=3.0, hi=80.0),
                                 J.default_tuning(leaf_size=4))
    return A, B


@pytest.mark.parametrize("kw", [dict(predicate="overlap", sizing="hash"),
                                dict(predicate="overlap", sizing="two_pass"),
                                dict(predicate="overlap", sizing="two_pass", traversal="per_ray_binary"),
                                dict(predicate="overlap", sizing="hash", active_bvh=False),
                                dict(predicate="intersection", sizing="hash"),
                                dict(predicate="containment", sizing="hash", include_overlap_pairs=True)])
def test_graph_replays_equal_the_eager_join(ctx, datasets, kw):
    from pierce_gb300 import join as J
    A, B = datasets
    eager = J.join(ctx, A, B, **kw)
    g = J.JoinGraph(ctx, A, B, J.make_opts(**kw))
    assert np.array_equal(g.pairs(), eager.pairs)
    for _ in range(3):
        st = g.launch()
        assert np.array_equal(g.pairs(), eager.pairs)
        for k in ("rays", "tri_tests", "raw_hits", "fp32_ambiguous"):
            assert st[k] == eager.stats[k], k
        assert st["launches"] > 5 and st["ms_total"] > 0
    g.close()


def test_graph_of_a_learned_sizing_join(ctx, datasets):
    from pierce_gb300 import join as J, sizing as S
    A, B = datasets
    ref = J.overlap_join_two_pass(ctx, A, B)
    model = S.SizingModel.load(ctx, S.TRAINED_MODEL)
    g = J.JoinGraph(ctx, A, B, J.make_opts(predicate="overlap", sizing="learned", sizing_model=model))
    for _ in range(2):
        g.launch()
        assert np.array_equal(g.pairs(), ref.pairs)


def test_graph_of_a_batched_join(ctx):
    from pierce_gb300 import join as J
    rng = np.random.default_rng(3)
    sides = []
    for s in range(2):
        parts = []
        for q in range(20):
            inst = pg.instances(int(rng.integers(1, 2**62)), int(rng.integers(1, 50)), pg.SPHERES, 1, 2, hi=30.0)
            inst["group"] = q
            parts.append(inst)
        sides.append(np.concatenate(parts))
    A = J.Dataset.from_instances(ctx, sides[0])
    B = J.Dataset.from_instances(ctx, sides[1])
    eager = J.overlap_join(ctx, A, B)
    g = J.JoinGraph(ctx, A, B, J.make_opts(predicate="overlap"))
    g.launch()
    assert np.array_equal(g.pairs(), eager.pairs) and len(eager.pairs) > 20


def test_batched_waves_equal_per_query_joins(ctx):
    """The batched runner (waves of partitioned joins, each captured as a
    graph) against one join call per query, plain and tuned."""
    from pierce_gb300 import batched as BT, join as J
    qs = BT.workload(seed=9, queries=40, n_lo=2, n_hi=60)
    for q in qs:
        q.extent *= 0.7  # denser than the workload: more pairs to compare
    waves = BT.make_waves(qs, budget_tris=2e5)
    assert len(waves) > 2 and sum(len(w.queries) for w in waves) == 40
    opts = lambda w: J.make_opts(predicate="overlap", expected_pairs=BT.expected_pairs(w), leaf_size=4)
    bat = BT.run_batched(ctx, waves, opts, warmup=0, replays=1, keep_pairs=True)
    plain = BT.run_per_query(ctx, qs, J.make_opts(predicate="overlap", sizing="two_pass", precision="fp32",
                                                  cull_objects=False, defer_exact=False, active_bvh=False),
                             build_leaf=4, keep_pairs=True)
    assert bat["pairs"] == plain["pairs"] > 20
    for i in range(40):
        have = bat["results"].get(i, np.zeros((0, 2), np.int32))
        assert np.array_equal(have, plain["results"][i]), i


def test_autotuner_returns_a_tried_setting_with_identical_pairs(ctx, datasets):
    from pierce_gb300 import join as J
    A, B = datasets
    base = J.make_opts(predicate="overlap", expected_pairs=2000)
    best, trials = J.autotune(ctx, A, B, base, repeats=1)
    assert len(trials) == 4 + 3 + 3 + 3 + 3 + 2  # the last two: the rays' source
    assert best["ms"] == min(t["ms"] for t in trials)
    assert best["leaf_size"] in (1, 2, 4, 8) and best["rays_per_warp"] in (32, 64, 128)
    assert best["stack_depth"] in (8, 16, 32) and best["hash_load_factor"] in (0.25, 0.5, 0.75)
    assert best["traversal"] in (0, 1, 2) and best["edge_source"] in (0, 1)
    ref = J.run_join(ctx, A, B, base)
    for t in trials[::3]:
        r = J.run_join(ctx, A, B, J.tuned_opts(base, t))
        assert np.array_equal(r.pairs, ref.pairs)
