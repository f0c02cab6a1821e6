"""The oracle's emulation of the reference's edge-ray semantics
(pierce/query/src/cuda/mesh_overlap_edges.cu:105-176: the ray starts at
tmin = nextafterf(0), one closest hit per iteration with tmin moved past
it, at most overlap_max_iterations iterations; a ray parallel to a
triangle misses it), against the exact set on crafted cases where each
quirk loses a pair."""
import numpy as np
import pytest

import pierce_gb300 as pg
from oracle import pyoracle as O


def mesh(tris, objs, edges):
    """Triangles (list of 3 points) with object ids and an explicit edge
    list [(start, end, object)]."""
    v = np.array([p for t in tris for p in t], np.float32)
    idx = np.arange(len(v), dtype=np.uint32).reshape(-1, 3)
    g = pg.Geometry.from_arrays(v, idx, np.array(objs, np.int32))
    if edges:
        s = np.array([e[0] for e in edges], np.float32)
        t = np.array([e[1] for e in edges], np.float32)
        src = np.array([e[2] for e in edges], np.int32)
    else:
        s = t = np.zeros((0, 3), np.float32)
        src = np.zeros(0, np.int32)
    g.set_edges(s, t, src)
    return g


BIG = [(-10, -10, 0), (10, -10, 0), (0, 10, 0)]


def big_at(z):
    return [(x, y, z) for x, y, _ in BIG]


def test_hit_at_start_point_is_not_seen():
    # A's edges both start on B's triangle (at the origin) and lead away
    A = mesh([[(0, 0, 0), (1, 0, 2), (0, 1, 2)]], [0],
             [((0, 0, 0), (1, 0, 2), 0), ((0, 0, 0), (0, 1, 2), 0), ((1, 0, 2), (0, 1, 2), 0)])
    B = mesh([BIG], [0], [(BIG[0], BIG[1], 0), (BIG[1], BIG[2], 0), (BIG[2], BIG[0], 0)])
    exact, _ = O.overlap_keys(A, B)
    assert exact.tolist() == [0]
    assert O.overlap_keys_reference(A, B).tolist() == []
    # reversed, the same edge ends on the triangle: t = 1 is seen
    A2 = mesh([[(0, 0, 0), (1, 0, 2), (0, 1, 2)]], [0], [((1, 0, 2), (0, 0, 0), 0)])
    assert O.overlap_keys_reference(A2, B).tolist() == [0]


def test_hits_at_one_t_count_once():
    # B objects 1 and 2 are coincident triangles; A's vertical edge crosses both at one point
    A = mesh([[(0, 0, -1), (0.01, 0, 1), (0, 0.01, 1)]], [0], [((0, 0, -1), (0.01, 0, 1), 0)])
    B = mesh([BIG, BIG], [1, 2], [])
    exact, _ = O.overlap_keys(A, B)
    assert exact.tolist() == [1, 2]
    assert O.overlap_keys_reference(A, B).tolist() == [1]
    d = O.reference_semantics_diff(A, B)
    assert d["only_exact"] == 1 and d["only_reference"] == 0


def test_iteration_cap():
    # one edge crosses three parallel triangles of objects 1, 2, 3 in t order 3, 2, 1
    A = mesh([[(0, 0, 5), (0.01, 0, -5), (0, 0.01, 5)]], [0], [((0, 0, 5), (0.01, 0, -5), 0)])
    B = mesh([big_at(-2), big_at(0), big_at(2)], [1, 2, 3], [])
    assert O.overlap_keys(A, B)[0].tolist() == [1, 2, 3]
    assert O.overlap_keys_reference(A, B, max_iterations=2).tolist() == [2, 3]
    assert O.overlap_keys_reference(A, B, max_iterations=1).tolist() == [3]
    assert O.overlap_keys_reference(A, B, max_iterations=100).tolist() == [1, 2, 3]


def test_ray_in_the_triangles_plane_misses():
    A = mesh([[(-1, 0, 0), (1, 0, 0), (0, 0, 3)]], [0], [((-1, 0, 0), (1, 0, 0), 0)])
    B = mesh([BIG], [0], [])
    assert O.overlap_keys(A, B)[0].tolist() == [0]
    assert O.overlap_keys_reference(A, B).tolist() == []


def test_generated_workload_agrees():
    A, B = pg.ellipsoid_pair(21, 22, 200, 200, 2, lo=0, hi=50, frac_contact=0.2)
    d = O.reference_semantics_diff(A, B, 100)
    assert d["exact_pairs"] > 100
    assert d["only_reference"] == 0  # the emulation only ever drops hits
