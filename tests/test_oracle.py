"""Pins of the CPU oracle's exact predicates against rational arithmetic,
and self-consistency checks of its join definitions (CPU only)."""
from fractions import Fraction as Fr
from pathlib import Path

import numpy as np
import pytest

import pierce_gb300 as pg
from oracle import pyoracle as O

GOLDEN = Path(__file__).resolve().parent / "golden"
rng = np.random.default_rng(1234)


def f32(*v):
    return np.array(v, dtype=np.float32)


def frac(p):
    return [Fr(float(x)) for x in p]


def det3(u, v, w):
    return (u[0] * (v[1] * w[2] - v[2] * w[1]) + u[1] * (v[2] * w[0] - v[0] * w[2])
            + u[2] * (v[0] * w[1] - v[1] * w[0]))


def sub(a, b):
    return [x - y for x, y in zip(a, b)]


def sgn(x):
    return (x > 0) - (x < 0)


def exact_orient3d(a, b, c, d):
    A, B, Cc, D = map(frac, (a, b, c, d))
    return sgn(det3(sub(B, A), sub(Cc, A), sub(D, A)))


def random_points(n, degenerate):
    pts = rng.uniform(-50, 50, size=(n, 4, 3)).astype(np.float32)
    if degenerate:
        # d in the plane of a, b, c up to float rounding, plus exact coplanar lattice cases
        for k in range(n):
            a, b, c = pts[k, 0], pts[k, 1], pts[k, 2]
            s, t = rng.uniform(-1, 2, 2)
            pts[k, 3] = (a + s * (b - a) + t * (c - a)).astype(np.float32)
            if k % 3 == 0:
                pts[k] = rng.integers(-4, 5, size=(4, 3)).astype(np.float32)
                pts[k, 3] = pts[k, 0] + (pts[k, 1] - pts[k, 0]) + 2 * (pts[k, 2] - pts[k, 0])
    return pts


@pytest.mark.parametrize("degenerate", [False, True])
def test_orient3d_matches_rationals(degenerate):
    L = O.lib()
    pts = random_points(400, degenerate)
    zero = 0
    for a, b, c, d in pts:
        want = exact_orient3d(a, b, c, d)
        got = L.oracle_orient3d(a.ctypes.data, b.ctypes.data, c.ctypes.data, d.ctypes.data)
        got_exact = L.oracle_orient3d_exact(a.ctypes.data, b.ctypes.data, c.ctypes.data, d.ctypes.data)
        assert got == want and got_exact == want
        zero += want == 0
    if degenerate:
        assert zero > 50  # the lattice cases are exactly coplanar


def test_orient3d_extreme_exponents():
    L = O.lib()
    tiny = np.float32(1e-40)   # subnormal
    cases = [(f32(0, 0, 0), f32(tiny, 0, 0), f32(0, tiny, 0), f32(0, 0, tiny)),
             (f32(1e30, 0, 0), f32(0, 1e30, 0), f32(0, 0, 1e30), f32(1e-30, 1e-30, 1e-30)),
             (f32(1, 1, 1), f32(1, 1, 1), f32(2, 3, 4), f32(5, 6, 7))]
    for a, b, c, d in cases:
        assert L.oracle_orient3d(a.ctypes.data, b.ctypes.data, c.ctypes.data, d.ctypes.data) == \
            exact_orient3d(a, b, c, d)


def exact_seg_tri(p, q, a, b, c):
    """Closed segment vs closed triangle with rational arithmetic, by a
    formulation independent of the oracle: solve p + t (q - p) = a + u e1 + v e2
    when not parallel, else test in the plane by barycentric/segment logic."""
    P, Q, A, B, Cc = map(frac, (p, q, a, b, c))
    e1, e2, d = sub(B, A), sub(Cc, A), sub(Q, P)
    n = [e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2], e1[0] * e2[1] - e1[1] * e2[0]]
    if n == [0, 0, 0]:
        return False
    den = sum(x * y for x, y in zip(n, d))
    s = sub(P, A)
    if den != 0:
        t = -sum(x * y for x, y in zip(n, s)) / den
        if t < 0 or t > 1:
            return False
        X = [P[i] + t * d[i] for i in range(3)]
        return point_in_tri(X, A, B, Cc, n)
    if sum(x * y for x, y in zip(n, s)) != 0:
        return False
    # coplanar: endpoints inside, or crossing an edge (sampled exactly on the segment)
    if point_in_tri(P, A, B, Cc, n) or point_in_tri(Q, A, B, Cc, n):
        return True
    for U, W in ((A, B), (B, Cc), (Cc, A)):
        if seg_seg_coplanar(P, Q, U, W, n):
            return True
    return False


def point_in_tri(X, A, B, Cc, n):
    def side(U, W):
        e = sub(W, U)
        r = sub(X, U)
        cr = [e[1] * r[2] - e[2] * r[1], e[2] * r[0] - e[0] * r[2], e[0] * r[1] - e[1] * r[0]]
        return sgn(sum(x * y for x, y in zip(cr, n)))
    s = [side(A, B), side(B, Cc), side(Cc, A)]
    return not (1 in s and -1 in s)


def seg_seg_coplanar(P, Q, U, W, n):
    def o(a, b, c):
        e, r = sub(b, a), sub(c, a)
        cr = [e[1] * r[2] - e[2] * r[1], e[2] * r[0] - e[0] * r[2], e[0] * r[1] - e[1] * r[0]]
        return sgn(sum(x * y for x, y in zip(cr, n)))

    def on(a, b, c):
        return all(min(a[i], b[i]) <= c[i] <= max(a[i], b[i]) for i in range(3))
    d1, d2, d3, d4 = o(P, Q, U), o(P, Q, W), o(U, W, P), o(U, W, Q)
    if d1 * d2 < 0 and d3 * d4 < 0:
        return True
    return ((d1 == 0 and on(P, Q, U)) or (d2 == 0 and on(P, Q, W)) or (d3 == 0 and on(U, W, P))
            or (d4 == 0 and on(U, W, Q)))


def seg_tri_cases(n):
    out = []
    for k in range(n):
        tri = rng.integers(-3, 4, size=(3, 3)).astype(np.float32)
        kind = k % 4
        if kind == 0:      # generic
            p, q = rng.uniform(-3, 3, size=(2, 3)).astype(np.float32)
        elif kind == 1:    # endpoint on a vertex / edge point of the triangle
            p = tri[rng.integers(3)] if k % 8 == 1 else ((tri[0] + tri[1]) / 2).astype(np.float32)
            q = rng.integers(-3, 4, size=3).astype(np.float32)
        elif kind == 2:    # coplanar segment
            s, t, u, w = rng.integers(-2, 3, 4)
            p = (tri[0] + s * (tri[1] - tri[0]) + t * (tri[2] - tri[0])).astype(np.float32)
            q = (tri[0] + u * (tri[1] - tri[0]) + w * (tri[2] - tri[0])).astype(np.float32)
        else:              # lattice segment
            p, q = rng.integers(-3, 4, size=(2, 3)).astype(np.float32)
        out.append((p, q, tri[0], tri[1], tri[2]))
    return out


def test_segment_triangle_matches_rationals():
    L = O.lib()
    hits = 0
    for p, q, a, b, c in seg_tri_cases(1500):
        want = exact_seg_tri(p, q, a, b, c)
        got = L.oracle_seg_tri(p.ctypes.data, q.ctypes.data, a.ctypes.data, b.ctypes.data, c.ctypes.data, 0)
        assert bool(got) == want, (p, q, a, b, c)
        hits += want
    assert 200 < hits < 1400


def test_zray_crossing_counts_each_crossing_once():
    """A +Z ray through shared edges and vertices of a closed lattice cube
    crosses it exactly twice (once in, once out) from below and once from
    inside; the symbolic perturbation resolves every tie."""
    L = O.lib()
    cube_v = np.array([[x, y, z] for x in (0, 2) for y in (0, 2) for z in (0, 2)], np.float32)
    # 12 triangles of the cube surface (two per face)
    faces = [(0, 1, 3, 2), (4, 6, 7, 5), (0, 4, 5, 1), (2, 3, 7, 6), (0, 2, 6, 4), (1, 5, 7, 3)]
    tris = []
    for a, b, c, d in faces:
        tris += [(a, b, c), (a, c, d)]
    for px, py in [(1, 1), (0, 0), (1, 0), (2, 2), (0.5, 1.5), (2, 1), (0, 2)]:
        for pz, want in [(-1, 2), (1, 1), (3, 0)]:
            p = np.array([px, py, pz], np.float32)
            n = 0
            for t in tris:
                a, b, c = (cube_v[i] for i in t)
                n += L.oracle_zray_crosses(p.ctypes.data, a.ctypes.data, b.ctypes.data, c.ctypes.data)
            if px in (0, 2) or py in (0, 2):
                # on the boundary in x or y: perturbation moves the point to +x/+y
                inside_xy = (px < 2) and (py < 2)
                assert n == (want if inside_xy else 0), (px, py, pz, n)
            else:
                assert n == want, (px, py, pz, n)


def test_face_restatement_equals_edge_definition():
    A, B = pg.ellipsoid_pair(21, 22, 120, 120, 2, lo=0, hi=40, frac_contact=0.1)
    edge, _ = O.overlap_keys(A, B)
    face = O.face_keys(A, B)
    assert np.array_equal(edge, face)
    assert len(edge) > 50


@pytest.mark.parametrize("case", ["ellipsoid_contacts", "tubes_vs_spheres", "one_object_each", "disjoint",
                                  "nested"])
def test_touch_restatement_equals_face_and_edge_definition(case):
    """TOUCH's candidates are every pair of overlapping object boxes whatever
    the tree's shape, so after exact refinement its pairs are Face's."""
    A, B = {
        "ellipsoid_contacts": lambda: pg.ellipsoid_pair(21, 22, 120, 120, 2, lo=0, hi=40, frac_contact=0.1),
        "tubes_vs_spheres": lambda: (pg.tubes(4, 3, 4000, hi=30.0), pg.icospheres(5, 150, 2, hi=30.0)),
        "one_object_each": lambda: (pg.icospheres(6, 1, 2, hi=0.0), pg.icospheres(7, 1, 2, lo=0.5, hi=0.5)),
        "disjoint": lambda: (pg.icospheres(8, 40, 1, hi=10.0), pg.icospheres(9, 40, 1, lo=100.0, hi=110.0)),
        "nested": lambda: (pg.icospheres(41, 30, 2, ln_mu=float(np.log(5.0)), sigma=0.5, lo=0.0, hi=0.0),
                           pg.icospheres(42, 40, 1, ln_mu=float(np.log(0.5)), sigma=0.2, lo=-0.5, hi=0.5)),
    }[case]()
    touch, candidates = O.touch_keys(A, B)
    face = O.face_keys(A, B)
    edge, _ = O.overlap_keys(A, B)
    assert np.array_equal(touch, face) and np.array_equal(touch, edge), case
    assert candidates >= len(touch)
    if case == "disjoint":
        assert candidates == 0 and len(touch) == 0


@pytest.mark.parametrize("name", ["icospheres", "ellipsoid_contacts"])
def test_golden_pair_sets_reproduce(name):
    import importlib.util
    spec = importlib.util.spec_from_file_location("make_golden", GOLDEN / "make_golden.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    A, B = mod.JOIN_CASES[name]()
    g = np.load(GOLDEN / f"pairs_{name}.npz")
    assert np.array_equal(O.overlap_keys(A, B)[0], g["overlap"])
    assert np.array_equal(O.overlap_keys(A, B, mode=1)[0], g["overlap_fp32"])
    assert np.array_equal(O.intersection_keys(A, B), g["intersection"])
    assert np.array_equal(O.containment_keys(A, B), g["containment"])


def test_direction_split_and_swap():
    A, B = pg.icospheres(31, 100, 2, hi=30.0), pg.icospheres(32, 100, 2, hi=30.0)
    both, _ = O.overlap_keys(A, B)
    ab, _ = O.overlap_keys(A, B, direction=1)
    ba, _ = O.overlap_keys(A, B, direction=2)
    assert np.array_equal(both, np.union1d(ab, ba))
    # swapping the datasets swaps every pair
    rev, _ = O.overlap_keys(B, A)
    swapped = np.sort((rev << np.uint64(32)) | (rev >> np.uint64(32)))
    assert np.array_equal(both, swapped)


def _lattice_cube(lo, hi, obj):
    """Closed lattice cube [lo, hi]^3 as 12 triangles of object `obj`."""
    v = np.array([[x, y, z] for x in (lo, hi) for y in (lo, hi) for z in (lo, hi)], np.float32)
    faces = [(0, 1, 3, 2), (4, 6, 7, 5), (0, 4, 5, 1), (2, 3, 7, 6), (0, 2, 6, 4), (1, 5, 7, 3)]
    tris = []
    for a, b, c, d in faces:
        tris += [(a, b, c), (a, c, d)]
    return v, np.array(tris, np.uint32), np.full(12, obj, np.int32)


def test_parity_crossing_counts_of_nested_cubes():
    """Crossing counts of the parity rays (the --enable-tracking hit counts):
    a ray from inside the inner of two nested cubes crosses each once, one
    from below both crosses each twice, one between them crosses the outer
    once and the inner not at all."""
    v0, i0, o0 = _lattice_cube(0, 8, 0)
    v1, i1, o1 = _lattice_cube(2, 6, 1)
    T = pg.Geometry.from_arrays(np.concatenate([v0, v1]), np.concatenate([i0, i1 + len(v0)]),
                                np.concatenate([o0, o1]))
    points = np.array([[3, 3, 3], [3, 3, -1], [1, 1, 1], [7, 7, 9], [3, 3, 7]], np.float32)
    src, tgt, hits = O.parity_crossings(points, T)
    got = {(int(s), int(t)): int(h) for s, t, h in zip(src, tgt, hits)}
    assert got == {(0, 0): 1, (0, 1): 1, (1, 0): 2, (1, 1): 2, (2, 0): 1, (4, 0): 1}


def test_parity_crossing_counts_agree_with_parity_pairs():
    """Targets of odd crossing count are exactly the parity pairs, in both
    directions of a dataset pair with nested and touching ellipsoids."""
    A, B = pg.ellipsoid_pair(41, 42, 150, 150, 2, lo=0, hi=60, frac_inside=0.3, frac_contact=0.05)
    for S, T in ((A, B), (B, A)):
        fv = S.first_vertices()
        src, tgt, hits = O.parity_crossings(fv, T)
        assert np.all(hits >= 1)
        keys = (src.astype(np.uint64) << np.uint64(32)) | tgt.astype(np.uint64)
        assert np.all(np.diff(keys.astype(np.int64)) > 0)  # unique, sorted by (source, target)
        odd = keys[(hits & 1) == 1]
        assert np.array_equal(odd, O.parity_keys(fv, T, swap=0))
    assert (hits & 1).sum() > 10


def _cells(rows):
    from pierce_gb300.geometry import GRID_DTYPE
    return np.array(rows, dtype=GRID_DTYPE)


def test_grid_estimate_hand_computed():
    """The grid selectivity estimate on cells whose arithmetic is exact in
    float32: one matched cell contributes 4 * 2 * (0.5 + 0.5)^3 / 2^3 = 1;
    unmatched cells and cells without touches contribute nothing."""
    A = _cells([(0, 0, 0, 1, 4, 0.5, 1.0), (1, 0, 0, 1, 2, 0.5, 1.0), (2, 0, 0, 0, 0, 0.5, 1.0)])
    B = _cells([(0, 0, 0, 1, 2, 0.5, 1.0), (5, 5, 5, 1, 1, 0.5, 1.0), (2, 0, 0, 0, 0, 0.5, 1.0)])
    raw, est, matched = O.grid_estimate(A, B, 2.0, 0.0, 0.8)
    assert (raw, est, matched) == (1.0, 1, 2)
    # cells smaller than the objects: probability capped at 1, alpha = (0.5 + 0.5)^3 / 0.5^3 = 8
    raw, est, matched = O.grid_estimate(A, B, 0.5, 0.0, 0.8)
    assert (raw, est) == (8.0, 1)
    raw, est, _ = O.grid_estimate(A, B, 0.5, 0.0, 0.8, alpha_correction=False)
    assert (raw, est) == (8.0, 8)
    # shape correction: ratios 0.25 and 1 give sqrt(0.25)^1 = 0.5 with gamma 1
    A2 = _cells([(0, 0, 0, 1, 4, 0.5, 0.25)])
    raw, _, _ = O.grid_estimate(A2, B, 2.0, 0.0, 1.0)
    assert raw == 0.5


def test_full_workload_golden_fixture():
    """The stored oracle pair sets of the full benchmark workload (made by
    make_golden.py --full): sorted, unique, containment pairs are
    intersection pairs of B inside A, and the seeds are the benchmark's."""
    g = np.load(GOLDEN / "pairs_ellipsoids_50000.npz")
    inter, cont = g["intersection"], g["containment"]
    assert (len(inter), len(cont)) == (13666, 10122)
    for k in (inter, cont):
        assert k.dtype == np.uint64 and np.all(np.diff(k.astype(np.int64)) > 0)
    assert np.isin(cont, inter).all()
    assert [int(x) for x in g["seeds"]] == [2024, 2025] and int(g["meshes_per_side"]) == 50000
