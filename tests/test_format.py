"""`.pre` format, edge extraction and generators (CPU only).

The committed fixtures in tests/golden were produced by the reference's own
`.pre` reader/writer and edge extractor (compiled from its sources by
oracle/build_ref.sh); see tests/golden/make_golden.py.
"""
import hashlib
import json
from pathlib import Path

import numpy as np
import pytest

import pierce_gb300 as pg
from pierce_gb300.geometry import HostError

GOLDEN = Path(__file__).resolve().parent / "golden"
sys_path_ok = True


def zero_padding(b: bytes) -> bytes:
    return b[:50] + b"\x00" * 6 + b[56:]


def _make(name):
    import importlib.util
    spec = importlib.util.spec_from_file_location("make_golden", GOLDEN / "make_golden.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod.FORMAT_CASES[name]()


DIGESTS = json.loads((GOLDEN / "ref_digests.json").read_text())


@pytest.mark.parametrize("name", sorted(DIGESTS))
def test_edges_and_writer_match_reference(tmp_path, name):
    geom = _make(name)
    raw = pg.Geometry.from_arrays(geom.vertices, geom.indices, geom.tri_to_object)
    raw.write_pre(tmp_path / "in.pre")
    inp = zero_padding((tmp_path / "in.pre").read_bytes())
    # the generator is bit-identical on every host
    assert hashlib.sha256(inp).hexdigest() == DIGESTS[name]["input_sha256"]
    raw.extract_edges(0)
    raw.write_pre(tmp_path / "out.pre")
    out = zero_padding((tmp_path / "out.pre").read_bytes())
    assert len(out) == DIGESTS[name]["bytes"]
    assert hashlib.sha256(out).hexdigest() == DIGESTS[name]["sha256"]


def test_reference_file_reads_and_rewrites_identically(tmp_path):
    ref = (GOLDEN / "ref_icospheres_l1.pre").read_bytes()
    g = pg.Geometry.read_pre(GOLDEN / "ref_icospheres_l1.pre")
    assert g.has_edges and g.num_objects == 20 and g.num_triangles == 20 * 80
    g.write_pre(tmp_path / "again.pre")
    assert zero_padding((tmp_path / "again.pre").read_bytes()) == ref


def test_object_order_has_the_same_edge_set():
    geom = _make("tubes")
    raw = pg.Geometry.from_arrays(geom.vertices, geom.indices, geom.tri_to_object)
    raw.extract_edges(0)
    a = np.concatenate([raw.edge_starts, raw.edge_ends, raw.edge_src[:, None].view(np.float32)], 1)
    raw.extract_edges(1)
    b = np.concatenate([raw.edge_starts, raw.edge_ends, raw.edge_src[:, None].view(np.float32)], 1)
    sa = np.sort(a.view(np.uint32).view([("", np.uint32)] * 7).ravel())
    sb = np.sort(b.view(np.uint32).view([("", np.uint32)] * 7).ravel())
    assert np.array_equal(sa, sb)
    # object order: source ids non-decreasing
    assert np.all(np.diff(raw.edge_src) >= 0)


def test_unique_edges_of_closed_icospheres():
    g = pg.icospheres(3, 7, 2)
    assert g.num_edges == 7 * 30 * 4 ** 2          # E = 1.5 F for closed 2-manifolds
    assert g.num_triangles == 7 * 20 * 4 ** 2
    assert g.vertices.shape[0] == 7 * (10 * 4 ** 2 + 2)


def test_edge_rules_out_of_range_and_mismatch():
    v = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], np.float32)
    # a triangle with an out-of-range index is skipped
    g = pg.Geometry.from_arrays(v, np.array([[0, 1, 2], [0, 1, 9]], np.uint32), np.array([0, 0], np.int32))
    g.extract_edges(0)
    assert g.num_edges == 3
    # duplicate vertices closer than the 1e-5 quantum collapse into one key
    v2 = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [1.000001, 0, 0]], np.float32)
    g2 = pg.Geometry.from_arrays(v2, np.array([[0, 1, 2], [0, 3, 2]], np.uint32), np.array([0, 0], np.int32))
    g2.extract_edges(0)
    assert g2.num_edges == 3
    # first-seen orientation is kept: edge 1->0 comes from triangle (0,1,2) as 0->1
    assert any(np.array_equal(s, [0, 0, 0]) and np.array_equal(e, [1, 0, 0])
               for s, e in zip(g2.edge_starts, g2.edge_ends))


def test_grid_stats_roundtrip(tmp_path):
    g = pg.icospheres(9, 30, 1, hi=30.0).grid_stats(5.0)
    cells = g.grid_cells
    assert len(cells) > 0 and cells["touch_count"].sum() >= 30 and cells["center_count"].sum() == 30
    assert np.all(cells["vol_ratio"] <= 1.0) and np.all(cells["vol_ratio"] > 0.2)
    g.write_pre(tmp_path / "g.pre")
    h = pg.Geometry.read_pre(tmp_path / "g.pre")
    assert np.array_equal(h.grid_cells, cells)
    assert h.view().grid_cell_size == 5.0


@pytest.mark.parametrize("damage,status", [("magic", 2), ("version", 3), ("truncate", 1), ("header", 1)])
def test_corrupt_files_are_rejected(tmp_path, damage, status):
    g = pg.icospheres(4, 3, 1)
    p = tmp_path / "x.pre"
    g.write_pre(p)
    b = bytearray(p.read_bytes())
    if damage == "magic":
        b[0] ^= 0xFF
    elif damage == "version":
        b[4] = 3
    elif damage == "truncate":
        b = b[: len(b) - 17]
    else:
        b = b[:20]
    p.write_bytes(bytes(b))
    with pytest.raises(HostError) as e:
        pg.Geometry.read_pre(p)
    assert f"status {status}" in str(e.value)


def test_missing_file():
    with pytest.raises(HostError):
        pg.Geometry.read_pre("/nonexistent/dir/none.pre")


def test_generators_are_deterministic():
    a = pg.ellipsoid_pair(3, 4, 20, 20, 1, frac_contact=0.3)
    b = pg.ellipsoid_pair(3, 4, 20, 20, 1, frac_contact=0.3)
    for x, y in zip(a, b):
        assert np.array_equal(x.vertices, y.vertices) and np.array_equal(x.edge_starts, y.edge_starts)
    c = pg.ellipsoid_pair(3, 5, 20, 20, 1)
    assert not np.array_equal(a[1].vertices, c[1].vertices)


def test_inside_copies_are_inside():
    A, B = pg.ellipsoid_pair(11, 12, 40, 200, 1, frac_inside=1.0, frac_contact=0.0, lo=0, hi=100)
    from oracle import pyoracle as O
    cont = O.containment_keys(A, B)
    assert len(cont) == 200     # every B is a scaled copy strictly inside some A


def test_edge_extraction_thread_count_is_per_call():
    """A call with an explicit thread count leaves the process-wide OpenMP
    setting alone (an earlier form set it, so one single-threaded call made
    every later extraction single-threaded)."""
    import ctypes
    try:
        gomp = ctypes.CDLL("libgomp.so.1")
    except OSError:
        pytest.skip("libgomp not loadable")
    before = gomp.omp_get_max_threads()
    G = pg.icospheres(5, 20, 2, hi=20.0)
    G.extract_edges(0, 1)
    assert gomp.omp_get_max_threads() == before
    one = (G.edge_starts.copy(), G.edge_ends.copy(), G.edge_src.copy())
    G.extract_edges(0, 0)
    for a, b in zip(one, (G.edge_starts, G.edge_ends, G.edge_src)):
        assert np.array_equal(a, b)


def test_grid_stats_hand_computed():
    """Grid statistics (generateGridStats semantics) of two closed meshes
    whose values are exact: a 2x2x2 cube at the origin (volume ratio 1, mean
    extent 2) and a corner tetrahedron of the same box moved to (10,10,10)
    (volume 8/6 of an 8 box: ratio 1/6).  A cell counts an object's box
    centre and every cell its box touches (upper bound minus 1e-5)."""
    cube_v = np.array([[x, y, z] for x in (0, 2) for y in (0, 2) for z in (0, 2)], np.float32)
    quads = [(0, 1, 3, 2), (4, 6, 7, 5), (0, 4, 5, 1), (2, 3, 7, 6), (0, 2, 6, 4), (1, 5, 7, 3)]
    cube_t = [t for a, b, c, d in quads for t in ((a, b, c), (a, c, d))]
    tet_v = np.array([[10, 10, 10], [12, 10, 10], [10, 12, 10], [10, 10, 12]], np.float32)
    tet_t = [(0, 2, 1), (0, 1, 3), (0, 3, 2), (1, 2, 3)]
    v = np.concatenate([cube_v, tet_v])
    t = np.array(cube_t + [(a + 8, b + 8, c + 8) for a, b, c in tet_t], np.uint32)
    o = np.array([0] * 12 + [1] * 4, np.int32)
    G = pg.Geometry.from_arrays(v, t, o)
    ratio_tet = float(np.float32(np.float32(8.0) / np.float32(6.0)) / np.float32(8.0))
    G.grid_stats(4.0)
    got = [tuple(c.item()) for c in G.grid_cells]
    assert got == [(0, 0, 0, 1, 1, 2.0, 1.0), (2, 2, 2, 1, 1, 2.0, pytest.approx(ratio_tet))]
    G.grid_stats(1.0)
    cells = {tuple(int(x) for x in c.item()[:3]): c.item()[3:] for c in G.grid_cells}
    cube_cells = {(x, y, z) for x in (0, 1) for y in (0, 1) for z in (0, 1)}
    tet_cells = {(x, y, z) for x in (10, 11) for y in (10, 11) for z in (10, 11)}
    assert set(cells) == cube_cells | tet_cells
    assert cells[(1, 1, 1)][0] == 1 and cells[(11, 11, 11)][0] == 1          # box centres
    assert sum(c[0] for c in cells.values()) == 2
    assert all(c[1] == 1 and c[2] == 2.0 for c in cells.values())


def test_grid_stats_independent_of_thread_count(tmp_path):
    """Grid statistics summed in the serial order: one thread and all
    threads give the same bytes."""
    import os
    import subprocess
    import sys
    code = ("import sys; sys.path.insert(0, sys.argv[1]); import pierce_gb300 as pg; "
            "g = pg.ellipsoid_pair(3, 4, 400, 400, 2, lo=0, hi=80)[0]; g.grid_stats(3.0); "
            "open(sys.argv[2], 'wb').write(g.grid_cells.tobytes())")
    root = str(Path(__file__).resolve().parents[1])
    env = dict(os.environ, OMP_NUM_THREADS="1")
    subprocess.run([sys.executable, "-c", code, root, str(tmp_path / "one.bin")], check=True, env=env)
    g = pg.ellipsoid_pair(3, 4, 400, 400, 2, lo=0, hi=80)[0]
    g.grid_stats(3.0)
    assert len(g.grid_cells) > 100
    assert (tmp_path / "one.bin").read_bytes() == g.grid_cells.tobytes()
