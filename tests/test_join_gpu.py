"""GPU parity tests: the CUDA join path against the CPU oracle.

Every case compares the sorted (a, b) pair set bit-for-bit.  Inputs are the
seeded generators at sizes the oracle finishes in seconds.
"""
import numpy as np
import pytest

import pierce_gb300 as pg
from pierce_gb300 import join as J
from oracle import pyoracle as O

pytestmark = pytest.mark.gpu


def keys(res):
    return J.pairs_to_keys(res.pairs)


def ds(ctx, geom, leaf=1):
    return J.Dataset.from_geometry(ctx, geom, J.default_tuning(leaf_size=leaf))


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


@pytest.mark.parametrize("edge_source", ["dataset", "triangles"])
@pytest.mark.parametrize("sizing", ["hash", "two_pass"])
@pytest.mark.parametrize("leaf", [1, 4])
def test_overlap_exact_matches_oracle(ctx, case, sizing, leaf, edge_source):
    name, A, B = case
    want, _ = O.overlap_keys(A, B)
    got = J.overlap_join(ctx, ds(ctx, A, leaf), ds(ctx, B, leaf), sizing=sizing, edge_source=edge_source)
    assert np.array_equal(keys(got), want), name
    passes = 2 if sizing == "two_pass" else 1
    # culling traces only edges near the other side: dataset edges at most
    # once, the kept triangles' edges at most once per triangle
    bound = (A.num_edges + B.num_edges) if edge_source == "dataset" else 3 * (A.num_triangles + B.num_triangles)
    assert 0 < got.stats["rays"] <= passes * bound
    plain = J.overlap_join(ctx, ds(ctx, A, leaf), ds(ctx, B, leaf), sizing=sizing, cull_objects=False,
                           active_bvh=False)
    assert plain.stats["rays"] == passes * (A.num_edges + B.num_edges)


def test_overlap_fp32_plain_matches_oracle_fp32(ctx, case):
    name, A, B = case
    want, _ = O.overlap_keys(A, B, mode=1)
    got = J.overlap_join(ctx, ds(ctx, A), ds(ctx, B), precision="fp32", sizing="two_pass")
    assert np.array_equal(keys(got), want), name


@pytest.mark.parametrize("direction", ["mesh1_to_mesh2", "mesh2_to_mesh1"])
def test_overlap_direction(ctx, case, direction):
    name, A, B = case
    want, _ = O.overlap_keys(A, B, direction=1 if direction == "mesh1_to_mesh2" else 2)
    got = J.overlap_join(ctx, ds(ctx, A), ds(ctx, B), direction=direction)
    assert np.array_equal(keys(got), want), name


@pytest.mark.parametrize("edge_source", ["dataset", "triangles"])
@pytest.mark.parametrize("sizing", ["hash", "two_pass"])
def test_intersection_matches_oracle(ctx, case, sizing, edge_source):
    name, A, B = case
    want = O.intersection_keys(A, B)
    got = J.intersection_join(ctx, ds(ctx, A), ds(ctx, B), sizing=sizing, edge_source=edge_source)
    assert np.array_equal(keys(got), want), name


@pytest.mark.parametrize("edge_source", ["dataset", "triangles"])
@pytest.mark.parametrize("sizing", ["hash", "two_pass"])
def test_containment_matches_oracle(ctx, case, sizing, edge_source):
    name, A, B = case
    want = O.containment_keys(A, B)
    got = J.containment_join(ctx, ds(ctx, A), ds(ctx, B), sizing=sizing, edge_source=edge_source)
    assert np.array_equal(keys(got), want), name
    assert got.containment_count == len(want)


def test_containment_include_overlap(ctx, case):
    name, A, B = case
    cont = O.containment_keys(A, B)
    over, _ = O.overlap_keys(A, B)
    got = J.containment_join(ctx, ds(ctx, A), ds(ctx, B), include_overlap_pairs=True)
    k = keys(got)
    assert got.containment_count == len(cont)
    assert np.array_equal(k[: len(cont)], cont)
    assert np.array_equal(k[len(cont):], over)


def test_tiny_hash_table_recovers(ctx, case):
    """A deliberately undersized table is enlarged and the join rerun."""
    name, A, B = case
    want, _ = O.overlap_keys(A, B)
    got = J.overlap_join(ctx, ds(ctx, A), ds(ctx, B), sizing="fixed", hash_table_slots=16, max_retries=12)
    assert np.array_equal(keys(got), want)
    if len(want) > 8:
        assert got.stats["retries"] > 0


def test_empty_and_single(ctx):
    A = pg.icospheres(1, 1, 0, hi=0.0)          # one icosahedron at the origin
    z = np.zeros((0, 3), np.float32)
    empty = J.Dataset.from_arrays(ctx, z, np.zeros((0, 3), np.uint32), np.zeros(0, np.int32), z, z,
                                  np.zeros(0, np.int32))
    got = J.intersection_join(ctx, ds(ctx, A), empty)
    assert got.pairs.shape == (0, 2)
    # single triangle target
    v = np.array([[-5, -5, 0], [5, -5, 0], [0, 5, 0]], np.float32)
    T = pg.Geometry.from_arrays(v, np.array([[0, 1, 2]], np.uint32), np.array([0], np.int32)).extract_edges()
    want, _ = O.overlap_keys(A, T)
    got = J.overlap_join(ctx, ds(ctx, A), ds(ctx, T))
    assert np.array_equal(keys(got), want)
    assert len(want) == 1


def test_identical_datasets_coplanar(ctx):
    """B == A: every face coplanar with a face of the other side."""
    A = pg.icospheres(7, 50, 2, hi=30.0)
    B = pg.Geometry.from_arrays(A.vertices, A.indices, A.tri_to_object).extract_edges()
    want, _ = O.overlap_keys(A, B)
    got = J.overlap_join(ctx, ds(ctx, A), ds(ctx, B))
    assert np.array_equal(keys(got), want)
    assert all((want >> np.uint64(32)) >= 0)
    diag = (want >> np.uint64(32)) == (want & np.uint64(0xFFFFFFFF))
    assert diag.sum() == 50


@pytest.mark.parametrize("defer", [False, True])
def test_one_ulp_shifted_copy_needs_exact_arithmetic(ctx, defer):
    """B is A moved by one ulp: every B edge lies within rounding of an A
    face, so the float32 filter is undecided and the exact stages decide."""
    A = pg.icospheres(9, 40, 2, hi=25.0)
    v = np.nextafter(A.vertices, np.float32(np.inf)).astype(np.float32)
    B = pg.Geometry.from_arrays(v, A.indices, A.tri_to_object).extract_edges()
    want, _ = O.overlap_keys(A, B)
    got = J.overlap_join(ctx, ds(ctx, A), ds(ctx, B), defer_exact=defer)
    assert np.array_equal(keys(got), want)
    assert got.stats["fp32_ambiguous"] > 0
    inter = J.intersection_join(ctx, ds(ctx, A), ds(ctx, B), defer_exact=defer)
    assert np.array_equal(keys(inter), O.intersection_keys(A, B))


@pytest.mark.parametrize("active_bvh", [False, True])
@pytest.mark.parametrize("cull", [False, True])
@pytest.mark.parametrize("defer", [False, True])
@pytest.mark.parametrize("sizing", ["hash", "two_pass"])
def test_culling_and_deferral_do_not_change_pairs(ctx, case, cull, defer, sizing, active_bvh):
    name, A, B = case
    want, _ = O.overlap_keys(A, B)
    kw = dict(sizing=sizing, cull_objects=cull, defer_exact=defer, active_bvh=active_bvh)
    got = J.overlap_join(ctx, ds(ctx, A), ds(ctx, B), **kw)
    assert np.array_equal(keys(got), want), (name, kw)
    inter = J.intersection_join(ctx, ds(ctx, A), ds(ctx, B), **kw)
    assert np.array_equal(keys(inter), O.intersection_keys(A, B)), (name, kw)
    cont = J.containment_join(ctx, ds(ctx, A), ds(ctx, B), **kw)
    assert np.array_equal(keys(cont), O.containment_keys(A, B)), (name, kw)
    if active_bvh:
        assert got.stats["active_triangles"][0] <= A.num_triangles


def test_active_bvh_needs_no_dataset_bvh(ctx):
    A, B = pg.icospheres(61, 200, 2, hi=40.0), pg.icospheres(62, 200, 2, hi=40.0)
    lazy = J.default_tuning(defer_build=1)
    da, db = ds_t(ctx, A, lazy), ds_t(ctx, B, lazy)
    assert da.info().built == 0
    want = O.intersection_keys(A, B)
    assert np.array_equal(keys(J.intersection_join(ctx, da, db)), want)
    with pytest.raises(Exception):
        J.intersection_join(ctx, da, db, active_bvh=False)   # needs built datasets


def ds_t(ctx, geom, tuning):
    return J.Dataset.from_geometry(ctx, geom, tuning)


@pytest.mark.parametrize("name", ["icospheres", "ellipsoid_contacts"])
def test_golden_pair_sets(ctx, name):
    """GPU joins against the committed oracle answers (tests/golden)."""
    import importlib.util
    from pathlib import Path
    golden = Path(__file__).resolve().parent / "golden"
    spec = importlib.util.spec_from_file_location("make_golden", golden / "make_golden.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    A, B = mod.JOIN_CASES[name]()
    g = np.load(golden / f"pairs_{name}.npz")
    da, db = ds(ctx, A), ds(ctx, B)
    assert np.array_equal(keys(J.overlap_join(ctx, da, db)), g["overlap"])
    assert np.array_equal(keys(J.overlap_join(ctx, da, db, precision="fp32", sizing="two_pass",
                                              cull_objects=False)), g["overlap_fp32"])
    assert np.array_equal(keys(J.intersection_join(ctx, da, db)), g["intersection"])
    assert np.array_equal(keys(J.containment_join(ctx, da, db)), g["containment"])


@pytest.mark.parametrize("predicate", ["intersection", "containment"])
def test_noncontiguous_objects_match_oracle(ctx, predicate):
    """Objects whose triangles are interleaved take the parity path over the
    per-join triangle hierarchies (whole objects kept); contiguous ones take
    the object-pair parity path.  Both must equal the oracle."""
    A, B = pg.ellipsoid_pair(11, 12, 120, 120, 2, lo=0, hi=45, frac_inside=0.3)
    rng = np.random.default_rng(4)
    perm = rng.permutation(B.num_triangles)
    Bs = pg.Geometry.from_arrays(B.vertices, B.indices[perm], B.tri_to_object[perm])
    Bs.set_edges(B.edge_starts, B.edge_ends, B.edge_src)
    want = O.intersection_keys(A, B) if predicate == "intersection" else O.containment_keys(A, B)
    for geom in (B, Bs):
        da, db = ds(ctx, A, 4), ds(ctx, geom, 4)
        got = keys(J.join(ctx, da, db, predicate=predicate))
        assert np.array_equal(np.sort(got), np.sort(want))
    assert len(want) > 10


@pytest.mark.parametrize("sizing", ["hash", "two_pass"])
@pytest.mark.parametrize("predicate", ["overlap", "intersection"])
def test_warp_packets_equal_per_ray_traversal(ctx, case, sizing, predicate):
    """Warp-cooperative traversal of the culled rays against one ray per
    thread: same pairs, same raw hit counts, same triangle tests."""
    name, A, B = case
    da, db = ds(ctx, A, 8), ds(ctx, B, 8)
    r1 = J.join(ctx, da, db, predicate=predicate, sizing=sizing, traversal="packets")
    r2 = J.join(ctx, da, db, predicate=predicate, sizing=sizing, traversal="per_ray_binary")
    assert np.array_equal(r1.pairs, r2.pairs)
    assert r1.stats["raw_hits"] == r2.stats["raw_hits"] and r1.stats["tri_tests"] == r2.stats["tri_tests"]
    assert r1.stats["node_visits"] < r2.stats["node_visits"]


@pytest.mark.parametrize("sizing", ["hash", "two_pass"])
@pytest.mark.parametrize("predicate", ["overlap", "intersection", "containment"])
def test_four_wide_nodes_equal_binary_walk(ctx, case, sizing, predicate):
    """One ray per thread over the four-wide copies of the per-join
    hierarchies against the same walk over the binary nodes: same pairs, and
    fewer (wider) node visits."""
    name, A, B = case
    da, db = ds(ctx, A, 4), ds(ctx, B, 4)
    r4 = J.join(ctx, da, db, predicate=predicate, sizing=sizing, traversal="per_ray")
    r2 = J.join(ctx, da, db, predicate=predicate, sizing=sizing, traversal="per_ray_binary")
    assert np.array_equal(r4.pairs, r2.pairs)
    assert r4.stats["rays"] == r2.stats["rays"]
    if r2.stats["node_visits"] > 100:
        assert r4.stats["node_visits"] < 0.75 * r2.stats["node_visits"]


def test_config1_full_size_matches_oracle(ctx):
    """The small CPU-runnable configuration at its full size: 2 x 2,000
    level-3 icospheres, radii lognormal(ln 1.5, 0.3), centres in [0, 200]^3;
    a pair overlaps when the surfaces meet or one mesh contains the other
    (the intersection predicate)."""
    A = pg.icospheres(1, 2000, 3, hi=200.0)
    B = pg.icospheres(2, 2000, 3, hi=200.0)
    want = O.intersection_keys(A, B)
    da, db = ds(ctx, A, 8), ds(ctx, B, 8)
    for kw in (dict(), dict(sizing="two_pass"), dict(precision="fp32", cull_objects=False, active_bvh=False,
                                                      sizing="two_pass")):
        got = keys(J.intersection_join(ctx, da, db, **kw))
        assert np.array_equal(np.sort(got), np.sort(want)), kw
    assert len(want) > 50


def test_parity_with_open_meshes_far_above(ctx):
    """An open surface (two separate triangles of one object, interleaved with
    another object's triangles) high above a closed mesh: the +Z ray from the
    mesh's first vertex crosses it once, so the pair is in the intersection
    set although the boxes do not meet.  Both parity paths must see it."""
    A = pg.icospheres(3, 3, 1, hi=6.0)
    fv = A.first_vertices()[0].astype(np.float64)
    # object 0: two triangles far above object-0 first vertex; object 1: a triangle elsewhere
    z = fv[2] + 50.0
    tri = lambda cx, cy, cz, s: [[cx - s, cy - s, cz], [cx + s, cy - s, cz + 0.1], [cx, cy + s, cz + 0.2]]
    verts = np.array(tri(fv[0] + 0.01, fv[1] + 0.013, z, 3.0) + tri(300, 300, 300, 1.0)
                     + tri(fv[0] + 40.0, fv[1], z, 1.0), np.float32)
    idx = np.arange(9, dtype=np.uint32).reshape(3, 3)
    t2o = np.array([0, 1, 0], np.int32)            # object 0 not contiguous
    B = pg.Geometry.from_arrays(verts, idx, t2o)
    B.extract_edges(1)
    want = O.intersection_keys(A, B)
    assert len(want) >= 1
    Bc = pg.Geometry.from_arrays(verts[[0, 1, 2, 6, 7, 8, 3, 4, 5]], idx, np.array([0, 0, 1], np.int32))
    Bc.extract_edges(1)
    for geom in (B, Bc):
        da, db = ds(ctx, A, 4), ds(ctx, geom, 4)
        got = keys(J.intersection_join(ctx, da, db))
        assert np.array_equal(np.sort(got), np.sort(O.intersection_keys(A, geom)))


def test_nested_containers_enlarge_and_rerun(ctx):
    """Thirty concentric spheres around small spheres: every B object lies
    in about thirty A objects, far beyond the containment buffer's first
    size (8 per B object) and a pair table sized for a handful of pairs.
    Both are enlarged and the pairs stay exact."""
    A = pg.icospheres(41, 30, 2, ln_mu=float(np.log(5.0)), sigma=0.5, lo=0.0, hi=0.0)
    B = pg.icospheres(42, 40, 1, ln_mu=float(np.log(0.5)), sigma=0.2, lo=-0.5, hi=0.5)
    cont = O.containment_keys(A, B)
    inter = O.intersection_keys(A, B)
    assert len(cont) >= 10 * B.num_objects
    for sizing in ("hash", "two_pass"):
        got = J.containment_join(ctx, ds(ctx, A), ds(ctx, B), sizing=sizing)
        assert np.array_equal(keys(got), cont), sizing
    got = J.containment_join(ctx, ds(ctx, A), ds(ctx, B), include_overlap_pairs=True)
    assert np.array_equal(keys(got)[: got.containment_count], cont)
    got = J.intersection_join(ctx, ds(ctx, A), ds(ctx, B), sizing="fixed", hash_table_slots=64, max_retries=8)
    assert np.array_equal(keys(got), inter)
    assert got.stats["retries"] > 0


@pytest.mark.parametrize("sizing", ["hash", "two_pass"])
def test_containment_pairs_and_their_fallback(ctx, sizing):
    """Containment tests its odd-parity candidate pairs directly, a block
    per pair: a 320-triangle sphere inside a 5,120-triangle one has a
    container patch larger than the shared-memory list, read in place.  A
    pair too large for that -- a 327,680-triangle container (past 65,536
    triangles together), or nested spheres of 5,120 or 20,480 triangles each
    (an unlisted patch past 4 M triangle pairs) -- sends the join through
    the culling pipeline.  All must give the oracle's pairs."""
    small = pg.ellipsoid_pair(1, 2, 300, 300, 2, lo=0, hi=70, frac_contact=0.1)
    big = (pg.icospheres(51, 1, 7, ln_mu=float(np.log(20.0)), sigma=0.0, lo=0.0, hi=0.0),
           pg.icospheres(52, 30, 2, ln_mu=0.0, sigma=0.2, lo=-10.0, hi=10.0))
    tight = (pg.icospheres(53, 1, 4, ln_mu=float(np.log(10.0)), sigma=0.0, lo=0.0, hi=0.0),
             pg.icospheres(54, 1, 4, ln_mu=float(np.log(9.9)), sigma=0.0, lo=0.0, hi=0.0))
    patch = (pg.icospheres(55, 1, 4, ln_mu=float(np.log(10.0)), sigma=0.0, lo=0.0, hi=0.0),
             pg.icospheres(56, 1, 2, ln_mu=float(np.log(9.9)), sigma=0.0, lo=0.0, hi=0.0))
    many = (pg.icospheres(57, 1, 5, ln_mu=float(np.log(10.0)), sigma=0.0, lo=0.0, hi=0.0),
            pg.icospheres(58, 1, 5, ln_mu=float(np.log(9.9)), sigma=0.0, lo=0.0, hi=0.0))
    by_pairs = {"pairs": 1, "large patch": 1, "dense container": 0, "large container": 0, "nested 20,480": 0}
    for name, (A, B) in (("pairs", small), ("large patch", patch), ("dense container", tight),
                         ("large container", big), ("nested 20,480", many)):
        want = O.containment_keys(A, B)
        got = J.containment_join(ctx, ds(ctx, A), ds(ctx, B), sizing=sizing)
        assert np.array_equal(keys(got), want), name
        assert got.stats["containment_by_pairs"] == by_pairs[name], name
    assert len(O.containment_keys(*big)) > 5 and len(O.containment_keys(*tight)) == 1


def test_object_hierarchy_and_grid_kept_per_dataset(ctx):
    """A dataset's object hierarchy and column grid are built by its first
    join and kept: the next join on the same datasets launches fewer
    kernels and returns the same pairs; fresh datasets build them again."""
    A, B = pg.icospheres(71, 200, 2, hi=40.0), pg.icospheres(72, 200, 2, hi=40.0)
    want = O.intersection_keys(A, B)
    da, db = ds(ctx, A), ds(ctx, B)
    r1 = J.intersection_join(ctx, da, db)
    r2 = J.intersection_join(ctx, da, db)
    assert np.array_equal(keys(r1), want) and np.array_equal(keys(r2), want)
    assert r2.stats["launches"] < r1.stats["launches"]
    r3 = J.intersection_join(ctx, ds(ctx, A), ds(ctx, B))
    assert np.array_equal(keys(r3), want)
    assert r3.stats["launches"] == r1.stats["launches"]


def test_objects_as_triangle_ranges(ctx):
    """A mesh stored object by object may give its objects as triangle
    offsets instead of per-triangle ids: the library writes the ids on the
    device, and the joins are those of the per-triangle form.  Offsets that
    do not rise from 0 to the triangle count are rejected."""
    A, B = pg.icospheres(81, 150, 2, hi=35.0), pg.icospheres(82, 150, 2, hi=35.0)
    def ranged(G):
        off = J.object_offsets(G.tri_to_object, G.num_objects)
        assert off is not None
        return J.Dataset.from_arrays(ctx, G.vertices, G.indices, None, G.edge_starts, G.edge_ends, G.edge_src,
                                     G.num_objects, object_offsets=off)
    da, db = ranged(A), ranged(B)
    assert np.array_equal(da.download()["tri_to_object"], A.tri_to_object)
    assert np.array_equal(keys(J.intersection_join(ctx, da, db)), O.intersection_keys(A, B))
    bad = J.object_offsets(A.tri_to_object, A.num_objects).copy()
    bad[1], bad[2] = bad[2], bad[1]
    if bad[1] != bad[2]:
        with pytest.raises(Exception):
            J.Dataset.from_arrays(ctx, A.vertices, A.indices, None, A.edge_starts, A.edge_ends, A.edge_src,
                                  A.num_objects, object_offsets=bad)
