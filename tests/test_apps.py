"""The drop-in executables: CLI, stdout lines the benchmark adapters parse,
timing-JSON keys and pair CSVs."""
import json
import re
import subprocess
from pathlib import Path

import numpy as np
import pytest

import pierce_gb300 as pg
from oracle import pyoracle as O

LIB = Path(__file__).resolve().parents[1] / "pierce_gb300" / "_lib"
APPS = ["pierce_overlap", "pierce_overlap_two_pass", "pierce_intersection", "pierce_containment"]


def run(app, *args, cwd=None, check=True):
    p = subprocess.run([str(LIB / app), *map(str, args)], capture_output=True, text=True, cwd=cwd, timeout=600)
    if check and p.returncode != 0:
        raise AssertionError(f"{app} failed ({p.returncode}):\n{p.stdout}\n{p.stderr}")
    return p


@pytest.mark.parametrize("app", APPS + ["pierce_preprocess"])
def test_help(app):
    p = run(app, "--help")
    assert "Usage:" in p.stdout


@pytest.mark.parametrize("app", APPS)
def test_missing_meshes_is_an_error(app):
    p = run(app, check=False)
    assert p.returncode == 1


def write_obj(path: Path, geom) -> None:
    v, idx, t2o = geom.vertices, geom.indices, geom.tri_to_object
    lines = [f"v {float(x)!r} {float(y)!r} {float(z)!r}" for x, y, z in v]
    cur = -1
    for t in range(idx.shape[0]):
        if t2o[t] != cur:
            cur = t2o[t]
            lines.append(f"o mesh{cur}")
        a, b, c = idx[t] + 1
        lines.append(f"f {a} {b} {c}")
    path.write_text("\n".join(lines) + "\n")


def test_preprocess_obj_to_pre(tmp_path):
    g = pg.icospheres(5, 6, 1, hi=10.0)
    write_obj(tmp_path / "m.obj", g)
    run("pierce_preprocess", "--dataset", tmp_path / "m.obj", "--output-geometry", tmp_path / "m.pre",
        "--generate-grid", "--grid-cell-size", "2.0", "--output-timing", tmp_path / "t.json")
    h = pg.Geometry.read_pre(tmp_path / "m.pre")
    assert h.num_objects == 6 and h.num_triangles == g.num_triangles and h.num_edges == g.num_edges
    assert len(h.grid_cells) > 0
    # same surfaces: per-triangle coordinates agree
    tri_g = g.vertices[g.indices].reshape(-1, 9)
    tri_h = h.vertices[h.indices].reshape(-1, 9)
    assert np.array_equal(tri_g, tri_h)
    # edges in the reference's map order, identical to direct extraction
    d = pg.Geometry.from_arrays(h.vertices, h.indices, h.tri_to_object).extract_edges(0)
    assert np.array_equal(d.edge_starts, h.edge_starts) and np.array_equal(d.edge_src, h.edge_src)
    t = json.loads((tmp_path / "t.json").read_text())
    assert "extracting edges_1" in t["phases"]


def test_preprocess_rejects_dt(tmp_path):
    p = run("pierce_preprocess", "--mode", "dt", "--dataset", tmp_path / "x.dt", check=False)
    assert p.returncode == 1


def keys_of_csv(path, cols=2):
    rows = Path(path).read_text().strip().splitlines()[1:]
    pairs = np.array([[int(x) for x in r.split(",")[:2]] for r in rows], dtype=np.int64).reshape(-1, 2)
    return np.sort((pairs[:, 0].astype(np.uint64) << np.uint64(32)) | pairs[:, 1].astype(np.uint64))


@pytest.fixture(scope="module")
def pre_files(tmp_path_factory):
    d = tmp_path_factory.mktemp("pre")
    A, B = pg.ellipsoid_pair(41, 42, 150, 150, 2, lo=0, hi=45, frac_contact=0.05)
    A.grid_stats(8.0)
    B.grid_stats(8.0)
    A.write_pre(d / "a.pre")
    B.write_pre(d / "b.pre")
    return d, A, B


@pytest.mark.gpu
def test_overlap_executable(pre_files):
    d, A, B = pre_files
    p = run("pierce_overlap", "--mesh1", d / "a.pre", "--mesh2", d / "b.pre", "--output", d / "o.json",
            "--pairs-output", d / "o.csv", "--track-hash-contention", "--runs", "2", cwd=d)
    want, _ = O.overlap_keys(A, B)
    assert np.array_equal(keys_of_csv(d / "o.csv"), want)
    out = p.stdout
    assert f"Unique object pairs: {len(want)}" in out
    assert f"Hash Table Query found {len(want)} unique pairs." in out
    assert re.search(r"Mesh1 objects: 150", out) and re.search(r"Mesh2 objects: 150", out)
    assert re.search(r"Using Direct Estimated Hash Table Size: \d+", out)
    assert re.search(r"Hash contention \(run 2\): \d+/\d+ accesses \([\d.]+%\)", out)
    phases = json.loads((d / "o.json").read_text())["phases"]
    for k in ("selectivity estimation_1", "raytrace_hash_mesh1tomesh2_1", "raytrace_hash_mesh2tomesh1_1",
              "compact_hash_table_pairs_1", "download results_1", "raytrace_hash_mesh1tomesh2_2"):
        assert k in phases, k


@pytest.mark.gpu
def test_overlap_estimate_only(pre_files):
    d, A, B = pre_files
    p = run("pierce_overlap", "--mesh1", d / "a.pre", "--mesh2", d / "b.pre", "--output", d / "e.json",
            "--estimate-only", cwd=d)
    m = re.search(r"Final Estimated Pairs:\s+(\d+)", p.stdout)
    assert m and int(m.group(1)) > 0


@pytest.mark.gpu
def test_two_pass_executable(pre_files):
    d, A, B = pre_files
    p = run("pierce_overlap_two_pass", "--mesh1", d / "a.pre", "--mesh2", d / "b.pre", "--output", d / "t.json",
            cwd=d)
    want, _ = O.overlap_keys(A, B)
    csv = d / "mesh_overlap_results.csv"
    assert np.array_equal(keys_of_csv(csv), want)
    # reference order: sorted by (mesh2 id, mesh1 id)
    rows = [tuple(map(int, r.split(","))) for r in csv.read_text().strip().splitlines()[1:]]
    assert rows == sorted(rows, key=lambda r: (r[1], r[0]))
    assert f"Unique object pairs: {len(want)}" in p.stdout
    phases = json.loads((d / "t.json").read_text())["phases"]
    for k in ("raytrace_mesh1tomesh2_pass1_1", "raytrace_mesh2tomesh1_pass2_1", "gpu deduplication_1",
              "download results_1"):
        assert k in phases, k


@pytest.mark.gpu
def test_intersection_executable(pre_files):
    d, A, B = pre_files
    p = run("pierce_intersection", "--mesh1", d / "a.pre", "--mesh2", d / "b.pre", "--output", d / "i.json",
            "--pairs-output", d / "i.csv", "--enable-profiling-stats", cwd=d)
    want = O.intersection_keys(A, B)
    assert np.array_equal(keys_of_csv(d / "i.csv"), want)
    assert f"Actual Intersection Pairs: {len(want)}" in p.stdout
    data = json.loads((d / "i.json").read_text())
    assert data["counters"]["profile_actual_intersection_pairs"] == len(want)
    for k in ("raytrace_overlap_hash_mesh1tomesh2_1", "raytrace_containment_hash_mesh2tomesh1_1"):
        assert k in data["phases"], k


@pytest.mark.gpu
@pytest.mark.parametrize("include", [False, True])
def test_containment_executable(pre_files, include):
    d, A, B = pre_files
    args = ["--mesh1", d / "a.pre", "--mesh2", d / "b.pre", "--output", d / "c.json"]
    if include:
        args.append("--include-overlap-pairs")
    p = run("pierce_containment", *args, cwd=d)
    cont = O.containment_keys(A, B)
    over, _ = O.overlap_keys(A, B)
    assert f"Containment pairs (B in A): {len(cont)}" in p.stdout
    rows = (d / "mesh_containment_results.csv").read_text().strip().splitlines()
    if include:
        assert rows[0] == "a_object_id,b_object_id,pair_type"
        assert f"Overlap/Touch pairs (A vs B): {len(over)}" in p.stdout
        assert f"Reported pairs: {len(cont) + len(over)}" in p.stdout
        types = [r.split(",")[2] for r in rows[1:]]
        assert types.count("containment") == len(cont) and types.count("overlap") == len(over)
    else:
        assert np.array_equal(keys_of_csv(d / "mesh_containment_results.csv"), cont)
    phases = json.loads((d / "c.json").read_text())["phases"]
    assert "compact_hash_table_pairs (containment)_1" in phases


HARNESS = r"""
#include "tracking_csv.h"
static Tracking make(int n) {
    Tracking t;
    t.num_sources = n;
    t.ids.assign((size_t)n * Tracking::kSlots, -1);
    t.hits.assign((size_t)n * Tracking::kSlots, 0);
    t.crossed.assign(n, 0);
    t.overflow.assign(n, 0);
    t.rays.assign(n, 0);
    return t;
}
int main(int argc, char** argv) {
    if (argc < 3) return 2;
    Tracking a = make(3), b = make(2);
    a.ids[0] = 5; a.hits[0] = 1; a.ids[1] = 7; a.hits[1] = 3; a.overflow[0] = 1;
    a.crossed = {4, 2, 0}; a.rays = {1, 1, 0};
    b.ids[0] = 0; b.hits[0] = 1; b.crossed = {1, 0}; b.rays = {1, 1};
    std::vector<pierce_pair> pairs = {{0, 5}, {0, 0}, {2, 2}};
    return write_tracking(argv[1], argv[2], a, b, pairs) ? 0 : 1;
}
"""


def test_tracking_csv_writer(tmp_path):
    """The --enable-tracking CSVs from given tracking tables (no device):
    final_pair looks the pair up as (source, target) for mesh1's rays and
    (target, source) for mesh2's."""
    from pierce_gb300 import build as B
    B.build(verbose=False)
    src = tmp_path / "harness.cpp"
    src.write_text(HARNESS)
    exe = tmp_path / "harness"
    apps = Path(B.__file__).resolve().parent / "apps"
    subprocess.run(["g++", "-std=c++17", "-I", str(apps), str(src), str(LIB / "obj" / "tracking_csv.host.o"),
                    "-o", str(exe)], check=True)
    subprocess.run([str(exe), str(tmp_path / "hits.csv"), str(tmp_path / "track.csv")], check=True)
    assert (tmp_path / "hits.csv").read_text().splitlines() == [
        "direction,source_object_id,target_object_id,target_ray_hits,final_pair",
        "mesh1_to_mesh2,0,5,1,1",
        "mesh1_to_mesh2,0,7,3,0",
        "mesh2_to_mesh1,0,0,1,1",
    ]
    assert (tmp_path / "track.csv").read_text().splitlines() == [
        "direction,source_object_id,iterations,candidate_count,tracked_target_count,tracked_hit_total,"
        "candidate_overflow_events,final_pair_count,tracked_final_pair_count",
        "mesh1_to_mesh2,0,1,4,2,4,1,1,1",
        "mesh1_to_mesh2,1,1,2,0,0,0,0,0",
        "mesh1_to_mesh2,2,0,0,0,0,0,0,0",
        "mesh2_to_mesh1,0,1,1,1,1,0,1,1",
        "mesh2_to_mesh1,1,1,0,0,0,0,0,0",
    ]
    bad = subprocess.run([str(exe), str(tmp_path / "missing" / "h.csv"), str(tmp_path / "t.csv")])
    assert bad.returncode == 1


def test_preprocess_obj_shapes_polygons_and_relative_indices(tmp_path):
    """OBJ rules of the producer (tinyobjloader's shapes, as the reference's
    loader uses them): a quad becomes a fan of two triangles, `o`/`g` lines
    start a new object only after faces, corners may be negative (relative)
    and carry texture/normal indices, a shape without faces is skipped."""
    (tmp_path / "s.obj").write_text("\n".join([
        "# two objects",
        "v 0 0 0", "v 1 0 0", "v 1 1 0", "v 0 1 0",
        "o first",
        "f 1 2 3 4",
        "g empty_group",
        "g second",
        "v 0 0 1", "v 1 0 1", "v 0 1 1",
        "vt 0 0", "vn 0 0 1",
        "f -3/1 -2/1/1 -1//1",
        "o third_without_faces",
        "",
    ]))
    run("pierce_preprocess", "--dataset", tmp_path / "s.obj", "--output-geometry", tmp_path / "s.pre",
        "--output-timing", tmp_path / "t.json")
    h = pg.Geometry.read_pre(tmp_path / "s.pre")
    assert h.num_objects == 2 and h.num_triangles == 3
    tris = h.vertices[h.indices].reshape(-1, 3, 3).tolist()
    assert tris == [[[0, 0, 0], [1, 0, 0], [1, 1, 0]], [[0, 0, 0], [1, 1, 0], [0, 1, 0]],
                    [[0, 0, 1], [1, 0, 1], [0, 1, 1]]]
    assert h.tri_to_object.tolist() == [0, 0, 1]
    # unique edges per object: the quad's fan has 5, the triangle 3
    assert sorted(np.bincount(h.edge_src).tolist()) == [3, 5]
