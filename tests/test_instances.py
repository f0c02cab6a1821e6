"""Instanced datasets: parameters, host expansion and device expansion.

The host expansion must reproduce the existing generators bit for bit (same
random stream, same arithmetic), and the device expansion must reproduce the
host expansion bit for bit, edges included, in the same order.
"""
import numpy as np
import pytest

import pierce_gb300 as pg


def edge_set(starts, ends, src):
    s = np.asarray(starts, np.float32).reshape(-1, 3)
    e = np.asarray(ends, np.float32).reshape(-1, 3)
    a = np.concatenate([s, e], 1).view(np.uint32)
    b = np.concatenate([e, s], 1).view(np.uint32)
    swap = [tuple(x) > tuple(y) for x, y in zip(a[:, :3], a[:, 3:])]
    canon = np.where(np.asarray(swap)[:, None], b, a)
    rows = np.concatenate([np.asarray(src, np.uint32)[:, None], canon], 1)
    return set(map(tuple, rows.tolist()))


def test_sphere_instances_reproduce_icosphere_generator():
    g = pg.icospheres(77, 40, 2, hi=50.0)
    inst = pg.instances(77, 40, pg.SPHERES, 2, hi=50.0)
    h = pg.expand_instances(inst)
    assert np.array_equal(h.vertices.view(np.uint32), g.vertices.view(np.uint32))
    assert np.array_equal(h.indices, g.indices)
    assert np.array_equal(h.tri_to_object, g.tri_to_object)
    assert h.num_edges == g.num_edges == 40 * 480
    assert edge_set(h.edge_starts, h.edge_ends, h.edge_src) == edge_set(g.edge_starts, g.edge_ends, g.edge_src)


def test_ellipsoid_instances_reproduce_pair_generator_side_a():
    A, _ = pg.ellipsoid_pair(5, 6, 25, 0, 2, frac_inside=0.0, frac_contact=0.0)
    inst = pg.instances(5, 25, pg.ELLIPSOIDS, 2, lo=0.0, hi=1000.0, noise_amp=0.05)
    h = pg.expand_instances(inst)
    assert np.array_equal(h.vertices.view(np.uint32), A.vertices.view(np.uint32))
    assert edge_set(h.edge_starts, h.edge_ends, h.edge_src) == edge_set(A.edge_starts, A.edge_ends, A.edge_src)


def test_instance_levels_and_sizes():
    inst = pg.instances(9, 200, pg.SPHERES, 1, 4)
    assert set(inst["level"].tolist()) == {1, 2, 3, 4}
    h = pg.expand_instances(inst)
    lv = inst["level"].astype(np.int64)
    assert h.num_triangles == int((20 * 4 ** lv).sum())
    assert h.num_edges == int((30 * 4 ** lv).sum())
    assert len(h.vertices) == int((10 * 4 ** lv + 2).sum())
    # closed 2-manifold per mesh: every template edge borders two triangles
    assert np.array_equal(np.bincount(h.tri_to_object), 20 * 4 ** lv)


def test_instance_argument_errors():
    with pytest.raises(Exception):
        pg.instances(1, 3, pg.SPHERES, 2, 9)
    bad = pg.instances(1, 3, pg.SPHERES, 2)
    bad["level"][1] = 12
    with pytest.raises(Exception):
        pg.expand_instances(bad)


@pytest.mark.gpu
@pytest.mark.parametrize("family", [pg.SPHERES, pg.ELLIPSOIDS])
def test_device_expansion_matches_host(ctx, family):
    from pierce_gb300 import join as J
    inst = pg.instances(31 + family, 120, family, 1, 4, hi=300.0)
    h = pg.expand_instances(inst)
    d = J.Dataset.from_instances(ctx, inst, J.default_tuning(defer_build=1))
    a = d.download()
    assert a["num_objects"] == 120
    assert np.array_equal(a["vertices"].reshape(-1).view(np.uint32), h.vertices.reshape(-1).view(np.uint32))
    assert np.array_equal(a["indices"].reshape(-1), h.indices.reshape(-1))
    assert np.array_equal(a["tri_to_object"], h.tri_to_object)
    assert np.array_equal(a["edge_src"], h.edge_src)
    assert np.array_equal(a["edge_starts"].reshape(-1).view(np.uint32), h.edge_starts.reshape(-1).view(np.uint32))
    assert np.array_equal(a["edge_ends"].reshape(-1).view(np.uint32), h.edge_ends.reshape(-1).view(np.uint32))


@pytest.mark.gpu
def test_instanced_join_matches_oracle(ctx):
    from pierce_gb300 import join as J
    from oracle import pyoracle as O
    ia = pg.instances(41, 150, pg.SPHERES, 1, 3, hi=40.0)
    ib = pg.instances(42, 150, pg.ELLIPSOIDS, 1, 3, p0=1.0, p1=3.0, hi=40.0)
    A = J.Dataset.from_instances(ctx, ia)
    B = J.Dataset.from_instances(ctx, ib)
    ha, hb = pg.expand_instances(ia), pg.expand_instances(ib)
    want = O.intersection_keys(ha, hb)
    got = J.pairs_to_keys(J.intersection_join(ctx, A, B).pairs)
    assert np.array_equal(np.sort(got), np.sort(want))
    assert len(want) > 20


def test_tube_structural_edges_equal_extracted_edges():
    g = pg.tubes(5, 6, 30000, hi=40.0)
    es, ee, src = g.edge_starts.copy(), g.edge_ends.copy(), g.edge_src.copy()
    h = pg.Geometry.from_arrays(g.vertices, g.indices, g.tri_to_object)
    h.extract_edges(order=1)
    assert h.num_edges == len(src)
    assert edge_set(es, ee, src) == edge_set(h.edge_starts, h.edge_ends, h.edge_src)


@pytest.mark.gpu
def test_object_contiguity_flag(ctx):
    from pierce_gb300 import join as J
    g = pg.ellipsoid_pair(3, 4, 300, 0, 2, frac_inside=0.0, frac_contact=0.0)[0]
    d = J.Dataset.from_geometry(ctx, g)
    assert d.info().objects_contiguous == 1
    perm = np.random.default_rng(1).permutation(g.num_triangles)
    s = pg.Geometry.from_arrays(g.vertices, g.indices[perm], g.tri_to_object[perm])
    s.set_edges(g.edge_starts, g.edge_ends, g.edge_src)
    assert J.Dataset.from_geometry(ctx, s).info().objects_contiguous == 0
    assert J.Dataset.from_instances(ctx, pg.instances(1, 500, pg.SPHERES, 0, 4)).info().objects_contiguous == 1
