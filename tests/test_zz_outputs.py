"""Outputs checked against the oracle: the parity-ray tracking tables
(pierce_parity_tracking, pierce_intersection --enable-tracking /
--enable-profiling-stats) against its crossing counts (exact parity rule,
each crossed triangle counted once), the grid selectivity estimate
(pierce_estimate_pairs) against its restatement of the reference's formula,
and the full benchmark workload's pair sets against the stored oracle sets.

Collected after the other GPU files, so that a failure here cannot hide
theirs.
"""
import json
import subprocess
from collections import defaultdict
from pathlib import Path

import numpy as np
import pytest

import pierce_gb300 as pg
from oracle import pyoracle as O

pytestmark = pytest.mark.gpu

LIB = Path(__file__).resolve().parents[1] / "pierce_gb300" / "_lib"


def oracle_tracking(S, T):
    """Per source object: {(target, crossings)} of odd count, and the number
    of targets crossed at all."""
    src, tgt, hits = O.parity_crossings(S.first_vertices(), T)
    odd = defaultdict(set)
    crossed = np.zeros(S.num_objects, np.int64)
    for s, t, h in zip(src, tgt, hits):
        crossed[s] += 1
        if h & 1:
            odd[int(s)].add((int(t), int(h)))
    return dict(odd), crossed


def device_odd(tr):
    odd = defaultdict(set)
    for s in range(tr.ids.shape[0]):
        for i in np.nonzero(tr.ids[s] >= 0)[0]:
            odd[s].add((int(tr.ids[s, i]), int(tr.hits[s, i])))
    return dict(odd)


@pytest.fixture(scope="module")
def pair():
    return pg.ellipsoid_pair(51, 52, 200, 200, 2, lo=0, hi=50, frac_inside=0.3, frac_contact=0.05)


def test_parity_tracking_matches_oracle(ctx, pair):
    from pierce_gb300 import join as J
    A, B = pair
    da, db = J.Dataset.from_geometry(ctx, A), J.Dataset.from_geometry(ctx, B)
    total = 0
    for (S, dS), (T, dT) in (((A, da), (B, db)), ((B, db), (A, da))):
        tr = J.parity_tracking(ctx, dS, dT)
        odd, crossed = oracle_tracking(S, T)
        assert device_odd(tr) == odd
        assert np.array_equal(tr.crossed.astype(np.int64), crossed)
        assert not tr.overflow.any()
        total += sum(len(v) for v in odd.values())
    assert total > 10
    # the odd targets are the parity pairs of the intersection join
    res = J.intersection_join(ctx, da, db)
    keys = set(((res.pairs[:, 0].astype(np.int64) << 32) | res.pairs[:, 1].astype(np.int64)).tolist())
    tr = J.parity_tracking(ctx, da, db)
    for s, t in zip(*np.nonzero(tr.ids >= 0)):
        assert (int(s) << 32 | int(tr.ids[s, t])) in keys


def test_parity_tracking_slot_bound(ctx, pair):
    """With one slot per source, the first odd target fills it and the rest
    count as overflow."""
    from pierce_gb300 import join as J
    A, B = pair
    da, db = J.Dataset.from_geometry(ctx, A), J.Dataset.from_geometry(ctx, B)
    tr = J.parity_tracking(ctx, db, da, max_targets=1)
    odd, crossed = oracle_tracking(B, A)
    for s in range(B.num_objects):
        want = odd.get(s, set())
        if want:
            assert (int(tr.ids[s, 0]), int(tr.hits[s, 0])) in want
        else:
            assert tr.ids[s, 0] == -1
        assert tr.overflow[s] == max(len(want) - 1, 0)
    assert np.array_equal(tr.crossed.astype(np.int64), crossed)


def test_intersection_executable_tracking_outputs(tmp_path, pair):
    A, B = pair
    A.grid_stats(8.0)
    B.grid_stats(8.0)
    A.write_pre(tmp_path / "a.pre")
    B.write_pre(tmp_path / "b.pre")
    cmd = [str(LIB / "pierce_intersection"), "--mesh1", str(tmp_path / "a.pre"), "--mesh2", str(tmp_path / "b.pre"),
           "--output", str(tmp_path / "i.json"), "--pairs-output", str(tmp_path / "i.csv"), "--enable-tracking",
           "--enable-profiling-stats", "--pair-hits-output", str(tmp_path / "hits.csv"),
           "--containment-tracking-output", str(tmp_path / "track.csv"), "--warmup-runs", "0"]
    p = subprocess.run(cmd, capture_output=True, text=True, cwd=tmp_path, timeout=600)
    assert p.returncode == 0, p.stdout + p.stderr
    assert "Pair hit tracking CSV: " in p.stdout and "Containment tracking CSV: " in p.stdout

    hits = (tmp_path / "hits.csv").read_text().strip().splitlines()
    assert hits[0] == "direction,source_object_id,target_object_id,target_ray_hits,final_pair"
    got = {"mesh1_to_mesh2": defaultdict(set), "mesh2_to_mesh1": defaultdict(set)}
    for r in hits[1:]:
        d, s, t, h, f = r.split(",")
        got[d][int(s)].add((int(t), int(h)))
        assert f == "1"  # every odd-parity target is an intersection pair
    odd12, crossed12 = oracle_tracking(A, B)
    odd21, crossed21 = oracle_tracking(B, A)
    assert dict(got["mesh1_to_mesh2"]) == odd12
    assert dict(got["mesh2_to_mesh1"]) == odd21

    track = (tmp_path / "track.csv").read_text().strip().splitlines()
    assert track[0] == ("direction,source_object_id,iterations,candidate_count,tracked_target_count,"
                        "tracked_hit_total,candidate_overflow_events,final_pair_count,tracked_final_pair_count")
    rows = [r.split(",") for r in track[1:]]
    assert len(rows) == A.num_objects + B.num_objects
    for d, s, it, cand, n, htot, ovf, fin, tfin in rows:
        odd, crossed = (odd12, crossed12) if d == "mesh1_to_mesh2" else (odd21, crossed21)
        want = odd.get(int(s), set())
        assert (int(it), int(cand), int(n), int(htot), int(ovf)) == \
            (1, int(crossed[int(s)]), len(want), sum(h for _, h in want), 0)
        assert int(fin) == int(tfin) == len(want)

    counters = json.loads((tmp_path / "i.json").read_text())["counters"]
    assert counters["profile_overlap_iterations_total"] == counters["profile_overlap_trace_calls"] > 0
    assert counters["profile_containment_rays_total"] > 0
    assert counters["profile_containment_iterations_total"] == counters["profile_containment_rays_total"]
    assert counters["profile_containment_candidate_overflow"] == 0


def test_grid_estimate_matches_oracle(ctx):
    """pierce_estimate_pairs against the restated estimator on the grid
    statistics of two generated datasets.  Tolerance: the per-cell float32
    terms may differ in the last bits (powf), so the raw sum agrees to a
    relative 1e-6 and the truncated estimate to 1 + 1e-6 of itself."""
    import ctypes as C
    from pierce_gb300 import capi
    A, B = pg.ellipsoid_pair(61, 62, 3000, 3000, 2, lo=0, hi=150, frac_contact=0.05)
    A.grid_stats(8.0)
    B.grid_stats(8.0)
    ca, cb = A.grid_cells, B.grid_cells
    cs = A.view().grid_cell_size
    L = capi.lib()
    for eps, gamma, alpha in ((0.001, 0.8, 1), (0.0, 1.0, 0), (0.5, 0.5, 1)):
        raw, est, matched = C.c_double(), C.c_int64(), C.c_int32()
        capi.check(L.pierce_estimate_pairs(ctx.handle, ca.ctypes.data, len(ca), cb.ctypes.data, len(cb), cs, eps,
                                           gamma, alpha, C.byref(raw), C.byref(est), C.byref(matched)),
                   "estimate_pairs")
        want_raw, want_est, want_matched = O.grid_estimate(ca, cb, cs, eps, gamma, bool(alpha))
        assert matched.value == want_matched > 50
        assert raw.value == pytest.approx(want_raw, rel=1e-6)
        assert abs(est.value - want_est) <= 1 + 1e-6 * want_est


def test_full_benchmark_workload_matches_golden(ctx):
    """The benchmark's full workload, 2 x 50,000 level-3 ellipsoids (64 M
    triangles and 96 M edges per side, inside copies and exact contacts):
    the intersection and containment pair sets equal the oracle's, stored in
    tests/golden/pairs_ellipsoids_50000.npz by make_golden.py --full."""
    import bench
    from pierce_gb300 import join as J
    g = np.load(Path(__file__).resolve().parent / "golden" / "pairs_ellipsoids_50000.npz")
    A, B, cfg = bench.workload(1.0)
    assert [int(x) for x in g["seeds"]] == cfg["seeds"] and int(g["meshes_per_side"]) == A.num_objects
    t = J.default_tuning(leaf_size=4)
    da, db = J.Dataset.from_geometry(ctx, A, t), J.Dataset.from_geometry(ctx, B, t)
    inter = J.intersection_join(ctx, da, db)
    assert np.array_equal(J.pairs_to_keys(inter.pairs), g["intersection"])
    cont = J.containment_join(ctx, da, db)
    assert np.array_equal(J.pairs_to_keys(cont.pairs), g["containment"])
    da.close()
    db.close()
