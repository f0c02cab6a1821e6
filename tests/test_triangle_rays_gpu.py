"""Edge rays taken from the kept triangles instead of the dataset's edge
list (pierce_join_opts.edge_source), and datasets uploaded without their
edges (pierce_tuning.skip_edges).

Exact predicates do not depend on a segment's orientation, so tracing the
edges of the triangles each join keeps gives the pair set of the `.pre`
edges whenever those are the triangles' edges, as pierce_preprocess
extracts them.  Every case is checked against the CPU oracle (which traces
the dataset's edge list)."""
import ctypes as C

import numpy as np
import pytest

import pierce_gb300 as pg
from pierce_gb300 import capi
from pierce_gb300 import join as J
from oracle import pyoracle as O

pytestmark = pytest.mark.gpu

CASES = {
    "icospheres": lambda: (pg.icospheres(101, 300, 3, hi=60.0), pg.icospheres(202, 300, 3, hi=60.0)),
    "ellipsoids_contacts": lambda: pg.ellipsoid_pair(1, 2, 300, 300, 2, lo=0, hi=70, frac_contact=0.1),
    "tubes_vs_ellipsoids": lambda: (pg.tubes(5, 4, 6000, hi=40.0),
                                    pg.ellipsoid_pair(3, 4, 10, 400, 2, lo=0, hi=40)[1]),
}


@pytest.fixture(scope="module", params=sorted(CASES))
def case(request):
    A, B = CASES[request.param]()
    return request.param, A, B


def edgeless(ctx, geom, leaf=0):
    t = J.default_tuning(defer_build=1, skip_edges=1)
    if leaf:
        t.leaf_size = leaf
    return J.Dataset.from_geometry(ctx, geom, t)


@pytest.mark.parametrize("predicate", ["overlap", "intersection", "containment"])
@pytest.mark.parametrize("sizing", ["hash", "two_pass"])
def test_edgeless_datasets_match_oracle(ctx, case, predicate, sizing):
    name, A, B = case
    want = {"overlap": lambda: O.overlap_keys(A, B)[0], "intersection": lambda: O.intersection_keys(A, B),
            "containment": lambda: O.containment_keys(A, B)}[predicate]()
    da, db = edgeless(ctx, A), edgeless(ctx, B)
    assert da.info().num_edges == 0 and db.info().num_edges == 0
    got = J.join(ctx, da, db, predicate=predicate, sizing=sizing)
    assert np.array_equal(J.pairs_to_keys(got.pairs), want), name


@pytest.mark.parametrize("leaf", [1, 2, 8])
def test_edgeless_leaf_sizes_and_directions(ctx, case, leaf):
    name, A, B = case
    for direction, code in (("both", 0), ("mesh1_to_mesh2", 1), ("mesh2_to_mesh1", 2)):
        want, _ = O.overlap_keys(A, B, direction=code)
        got = J.overlap_join(ctx, edgeless(ctx, A, leaf), edgeless(ctx, B, leaf), direction=direction,
                             leaf_size=leaf)
        assert np.array_equal(J.pairs_to_keys(got.pairs), want), (name, direction)


def test_triangle_rays_without_chunk_culling(ctx, case):
    """The hierarchies over active objects' triangles (no chunk culling):
    rays from groups of four soup triangles."""
    name, A, B = case
    want, _ = O.overlap_keys(A, B)
    t = J.default_tuning(defer_build=1)
    got = J.overlap_join(ctx, J.Dataset.from_geometry(ctx, A, t), J.Dataset.from_geometry(ctx, B, t),
                         cull_objects=False, edge_source="triangles")
    assert np.array_equal(J.pairs_to_keys(got.pairs), want), name
    got2 = J.intersection_join(ctx, edgeless(ctx, A), edgeless(ctx, B), cull_objects=False)
    assert np.array_equal(J.pairs_to_keys(got2.pairs), O.intersection_keys(A, B)), name


def test_triangle_rays_traversal_forms(ctx, case):
    name, A, B = case
    want, _ = O.overlap_keys(A, B)
    for form in ("per_ray", "packets", "per_ray_binary"):
        got = J.overlap_join(ctx, edgeless(ctx, A), edgeless(ctx, B), traversal=form)
        assert np.array_equal(J.pairs_to_keys(got.pairs), want), (name, form)


def test_learned_sizing_on_edgeless_datasets(ctx, case):
    from pierce_gb300 import sizing as S
    name, A, B = case
    want, _ = O.overlap_keys(A, B)
    model = S.SizingModel.load(ctx, S.TRAINED_MODEL)
    got = J.overlap_join(ctx, edgeless(ctx, A), edgeless(ctx, B), sizing="learned", sizing_model=model)
    assert np.array_equal(J.pairs_to_keys(got.pairs), want), name
    # an under-predicting capacity sends the join to the two-pass method
    tiny = J.overlap_join(ctx, edgeless(ctx, A), edgeless(ctx, B), sizing="learned", sizing_model=model,
                          output_safety=1e-9)
    assert np.array_equal(J.pairs_to_keys(tiny.pairs), want), name


def test_edgeless_instanced_batch(ctx):
    """Partitioned (batched) datasets expanded on the device without edges."""
    rng = np.random.default_rng(17)
    parts_a, parts_b = [], []
    for g in range(6):
        for parts in (parts_a, parts_b):
            inst = pg.instances(int(rng.integers(1, 2**62)), int(rng.integers(1, 30)), int(rng.integers(0, 2)), 0,
                                3, hi=30.0)
            inst["group"] = g
            parts.append(inst)
    ia, ib = np.concatenate(parts_a), np.concatenate(parts_b)
    t = J.default_tuning(defer_build=1, skip_edges=1)
    da, db = J.Dataset.from_instances(ctx, ia, t), J.Dataset.from_instances(ctx, ib, t)
    got = J.pairs_to_keys(J.overlap_join(ctx, da, db).pairs)
    want = []
    oa = np.concatenate([[0], np.cumsum([len(p) for p in parts_a])])
    ob = np.concatenate([[0], np.cumsum([len(p) for p in parts_b])])
    for g in range(6):
        a0, b0 = parts_a[g].copy(), parts_b[g].copy()
        a0["group"], b0["group"] = 0, 0
        k, _ = O.overlap_keys(pg.expand_instances(a0), pg.expand_instances(b0))
        want.append(((k >> np.uint64(32)) + np.uint64(oa[g])) << np.uint64(32) | ((k & np.uint64(0xFFFFFFFF))
                                                                                 + np.uint64(ob[g])))
    assert np.array_equal(got, np.sort(np.concatenate(want)))


def test_edgeless_dataset_needs_per_join_hierarchies(ctx):
    A = pg.icospheres(3, 20, 2, hi=20.0)
    da = edgeless(ctx, A)
    db = J.Dataset.from_geometry(ctx, A)  # with edges and its own hierarchy
    L = capi.lib()
    r = C.c_void_p()
    plain = J.make_opts(active_bvh=False, cull_objects=False)
    da.build(J.default_tuning())
    assert L.pierce_join(ctx.handle, da.handle, db.handle, C.byref(plain), C.byref(r), None) == \
        capi.ERR_INVALID_ARGUMENT
    assert b"edges" in L.pierce_last_error()
    dataset_rays = J.make_opts(edge_source="dataset")
    assert L.pierce_join(ctx.handle, da.handle, db.handle, C.byref(dataset_rays), C.byref(r), None) == \
        capi.ERR_INVALID_ARGUMENT
