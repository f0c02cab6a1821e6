"""Benchmark of the mesh spatial-join path on one GB300.

Default workload: the large tube-mesh overlap join.  Side A is 2,000
branching tube meshes of about 200k triangles each (random-walk skeletons,
step 1.0, branching probability 0.02, radius U[0.5, 3], 12-gon sections swept
and capped) in [0,1000]^3, about 400 M triangles; side B is 100,000 perturbed
ellipsoids (level-3 icospheres, semi-axes U[2,5], random rotation, 5 % radial
value noise) in [0,1000]^3, 128 M triangles; float32, seeded synthetic data.
One step = one overlap join (``pierce_overlap``'s query) from resident device
geometry to the sorted device pair set, per-join hierarchies included.

Printed JSON line (rank 0):
  value      - join queries/s with inputs resident in HBM (CUDA events on the
               library's stream), the tuned form: exact predicates behind an
               FP32 filter, culling, per-join hierarchies, the persistent ray
               queue, learned output sizing;
  e2e        - the same metric through the C ABI from pinned host buffers:
               dataset creation (host to device), the join, the pairs copied
               back, the datasets destroyed, every step;
  plain      - the plain GPU form (dataset hierarchies, FP32
               Moller-Trumbore, two-pass sizing, no culling), device and e2e;
  roofline   - the edge-ray traversal kernel against the measured HBM
               bandwidth, with algorithmic bytes over the units the launches
               process: 28*E_traced + 16*F_tgt + 12*V_tgt + 32*(2*F_tgt - 1)
               + 8*P_raw, E_traced the traced edges and F_tgt the triangles
               of the target's per-join hierarchy;
  cpu_baseline - the CPU oracle (exact restatement, OpenMP) on the first 10
               tubes against every ellipsoid near them, scaled to the join.

``--workload ellipsoids`` runs the intersection + containment line on
2 x 50,000 ellipsoids; ``batched`` the 4,096-query batch; ``preprocess`` the
`.pre` producer.  ``--impl reference`` times the CPU restatement of the
reference path on the same workload (the reference's GPU path needs OptiX
and cannot run here).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "join queries/s & ray-tri tests/s, 1 GB300, exact pair set, tuned vs plain"
UNIT = "join queries/s"


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def workload(scale: float = 1.0, seed_a: int = 2024, seed_b: int = 2025):
    import pierce_gb300 as pg
    n = max(10, int(round(50_000 * scale)))
    hi = 1000.0 * scale ** (1.0 / 3.0)
    A, B = pg.ellipsoid_pair(seed_a, seed_b, n, n, 3, 2.0, 5.0, 0.05, 0.0, hi, 0.2, 0.3, 0.01)
    return A, B, {"workload": "ellipsoids-intersection+containment", "meshes_per_side": n,
                  "subdivision": 3, "box": [0.0, round(hi, 3)], "triangles_per_side": A.num_triangles,
                  "edges_per_side": A.num_edges, "seeds": [seed_a, seed_b],
                  "l2": "inputs larger than L2 (about 9 GB of geometry and BVH per side, 129 MB L2)"}


def clocks_path(name: str) -> Path:
    """Where the nvidia-smi samples of a timed region go: $PIERCE_CLOCKS_DIR
    when set, else the system's temporary directory."""
    d = os.environ.get("PIERCE_CLOCKS_DIR")
    return Path(d) / name if d else Path(tempfile.gettempdir()) / f"pierce_{name}"


class Clocks:
    """nvidia-smi sampling during the timed region."""

    def __init__(self, path: Path):
        self.path = path
        self.proc = None

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={q}", "--format=csv,noheader,nounits",
                                          "-lms", "200"], stdout=self.f, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.f.close()

    def summary(self, device: int = 0):
        if not self.proc or not self.path.exists():
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.path.read_text().splitlines():
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9 or parts[0] != str(device):
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for name, val in zip(names, parts[5:9]):
                if val.lower() == "active":
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        loaded = [s for s in sm if s > 0.5 * max(sm)] or sm
        return {"sm_mhz": statistics.median(loaded), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm)}


def max_over_ranks(value: float, dist) -> float:
    """Largest per-rank time: the job is as slow as its slowest replica."""
    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        return value
    import torch
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(value)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def edge_ray_bytes(src, tgt, raw_hits):
    """Algorithmic bytes of one unculled edge-ray launch (every src edge
    against a hierarchy over every tgt triangle)."""
    E, F, V = src.num_edges, tgt.num_triangles, tgt.vertices.shape[0]
    return 28 * E + 16 * F + 12 * V + 32 * (2 * F - 1) + 8 * raw_hits


# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) per traced
# segment of the two edge-ray launches of one join, from one full-size ncu
# capture of this build (one pass per launch): the tube join's 3.896 GB over
# 67,917,789 segments, the ellipsoid intersection join's 250.3 MB over
# 4,148,442 segments.
EDGE_RAY_DRAM_BYTES_PER_RAY = {"tubes": 57.37, "ellipsoids": 60.34}


def traffic_estimate(rays, workload="tubes"):
    per = EDGE_RAY_DRAM_BYTES_PER_RAY.get(workload)
    return None if per is None else per * rays


def traced_edge_ray_bytes(rays, raw_hits, targets):
    """Algorithmic bytes of the edge-ray launches of one join over the units
    they process: each traced edge read once (28 B), a raw hit written once
    (8 B), and per direction the target's per-join hierarchy over its
    surviving triangles -- indices and object id (16 B per triangle), the
    vertices in proportion to the triangles kept (12 B each) and one 32-B
    node per node of a minimal binary tree.  targets: (dataset, triangles)."""
    b = 28 * rays + 8 * raw_hits
    for G, f in targets:
        v = G.vertices.shape[0] * f / max(G.num_triangles, 1)
        b += 16 * f + 12 * v + 32 * max(2 * f - 1, 0)
    return b


def cpu_sample(A_full, B_full, target_objects: int, seed: int = 7):
    """Spatial sample: objects whose first vertex lies in a sub-cube holding
    about target_objects objects of A; returns (A_sub, B_sub, fraction)."""
    import pierce_gb300 as pg
    nA = A_full.num_objects
    frac = min(1.0, target_objects / max(nA, 1))
    fa = A_full.first_vertices()
    fb = B_full.first_vertices()
    lo = np.minimum(fa.min(0), fb.min(0))
    hi = np.maximum(fa.max(0), fb.max(0))
    side = (hi - lo) * frac ** (1.0 / 3.0)
    sel_hi = lo + side

    def subset(G, fv):
        keep = np.all((fv >= lo) & (fv <= sel_hi), axis=1)
        objs = np.nonzero(keep)[0]
        remap = -np.ones(G.num_objects, np.int64)
        remap[objs] = np.arange(len(objs))
        t2o = G.tri_to_object
        tmask = keep[t2o]
        idx = G.indices[tmask]
        sub = pg.Geometry.from_arrays(G.vertices, idx, remap[t2o[tmask]].astype(np.int32))
        es, ee, src = G.edge_starts, G.edge_ends, G.edge_src
        em = keep[src]
        sub.set_edges(es[em], ee[em], remap[src[em]].astype(np.int32))
        return sub, len(objs)

    As, na = subset(A_full, fa)
    Bs, nb = subset(B_full, fb)
    return As, Bs, na / max(nA, 1)


def cpu_join_seconds(As, Bs) -> float:
    """Exact CPU restatement of the intersection + containment joins."""
    from oracle import pyoracle as O
    t0 = time.perf_counter()
    O.intersection_keys(As, Bs)
    O.containment_keys(As, Bs)
    return time.perf_counter() - t0


# ---- the tube-mesh overlap workload -------------------------------------------

TUBE_SEED, ELLIPSOID_SEED = 5, 6


def tube_counts(scale: float = 1.0):
    return max(2, int(round(2000 * scale))), max(2, int(round(100_000 * scale)))


def tube_geometry(scale: float = 1.0, first: int | None = None):
    """Side A: the branching tubes (all, or only tubes 0 .. first-1)."""
    import pierce_gb300 as pg
    n_tubes, _ = tube_counts(scale)
    return pg.tubes(TUBE_SEED, n_tubes, 200_000, 1.0, 0.02, 0.5, 3.0, 12, 0.0, 1000.0, first=first)


def ellipsoid_instances(scale: float = 1.0):
    """Side B: per-mesh parameters of the 100,000 ellipsoids."""
    import pierce_gb300 as pg
    _, n_ell = tube_counts(scale)
    return pg.instances(ELLIPSOID_SEED, n_ell, pg.ELLIPSOIDS, 3, p0=2.0, p1=5.0, noise_amp=0.05, lo=0.0, hi=1000.0)


def tubes_config(scale: float = 1.0) -> dict:
    n_tubes, n_ell = tube_counts(scale)
    return {"workload": "tubes-vs-ellipsoids-overlap", "predicate": "overlap", "tubes": n_tubes,
            "tube_triangles_target": 200_000, "tube_step": 1.0, "tube_branch_prob": 0.02,
            "tube_radius": [0.5, 3.0], "tube_sides": 12, "ellipsoids": n_ell, "ellipsoid_level": 3,
            "ellipsoid_axes": [2.0, 5.0], "box": [0.0, 1000.0], "seeds": [TUBE_SEED, ELLIPSOID_SEED],
            "l2": "inputs larger than L2 (about 40 GB of geometry resident, 129 MB L2)"}


def _cell_keys(c: np.ndarray) -> np.ndarray:
    c = c.astype(np.int64) + (1 << 20)
    return (c[:, 0] << 42) | (c[:, 1] << 21) | c[:, 2]


def boxes_near(tri_lo, tri_hi, obj_lo, obj_hi, cell: float = 8.0) -> np.ndarray:
    """Objects whose box shares a grid cell with the box of one of the given
    triangles: a superset of the objects whose box meets one of those
    triangle boxes (two boxes that meet share the cell of a common point)."""
    t0 = np.floor(tri_lo / cell).astype(np.int64)
    t1 = np.floor(tri_hi / cell).astype(np.int64)
    ext = t1 - t0
    keys = []
    for dx in range(int(ext[:, 0].max(initial=0)) + 1):
        for dy in range(int(ext[:, 1].max(initial=0)) + 1):
            for dz in range(int(ext[:, 2].max(initial=0)) + 1):
                sel = (ext[:, 0] >= dx) & (ext[:, 1] >= dy) & (ext[:, 2] >= dz)
                keys.append(np.unique(_cell_keys(t0[sel] + np.array([dx, dy, dz]))))
    cells = np.unique(np.concatenate(keys)) if keys else np.zeros(0, np.int64)
    o0 = np.floor(obj_lo / cell).astype(np.int64)
    o1 = np.floor(obj_hi / cell).astype(np.int64)
    oext = o1 - o0
    near = np.zeros(len(obj_lo), bool)
    for dx in range(int(oext[:, 0].max(initial=0)) + 1):
        for dy in range(int(oext[:, 1].max(initial=0)) + 1):
            for dz in range(int(oext[:, 2].max(initial=0)) + 1):
                sel = (oext[:, 0] >= dx) & (oext[:, 1] >= dy) & (oext[:, 2] >= dz) & ~near
                idx = np.nonzero(sel)[0]
                hit = np.isin(_cell_keys(o0[idx] + np.array([dx, dy, dz])), cells)
                near[idx[hit]] = True
    return near


def mesh_boxes(G):
    """Box (lo, hi) of every object of G whose vertices are stored object by
    object (generated and instanced meshes)."""
    vobj = np.empty(G.vertices.shape[0], np.int64)
    vobj[G.indices.reshape(-1)] = np.repeat(G.tri_to_object.astype(np.int64), 3)
    if np.any(vobj[1:] < vobj[:-1]):
        raise AssertionError("vertices are not stored object by object")
    starts = np.searchsorted(vobj, np.arange(G.num_objects))
    return np.minimum.reduceat(G.vertices, starts), np.maximum.reduceat(G.vertices, starts)


def instance_boxes(inst, batch: int = 8192):
    """Box (lo, hi) of every instanced mesh, from its host expansion in
    batches (the vertices of mesh m are contiguous)."""
    import pierce_gb300 as pg
    lo = np.empty((len(inst), 3), np.float32)
    hi = np.empty((len(inst), 3), np.float32)
    for s0 in range(0, len(inst), batch):
        part = inst[s0:s0 + batch].copy()
        part["group"] = 0
        lo[s0:s0 + len(part)], hi[s0:s0 + len(part)] = mesh_boxes(pg.expand_instances(part))
    return lo, hi


def tube_sample(k: int, scale: float = 1.0, inst_b=None, boxes=None):
    """The first k tubes and the ellipsoids whose boxes share a grid cell
    with the box of one of their triangles: every ellipsoid that can meet
    those tubes.  Returns (tubes, ellipsoids, ellipsoid ids)."""
    import pierce_gb300 as pg
    As = tube_geometry(scale, first=k)
    if inst_b is None:
        inst_b = ellipsoid_instances(scale)
    lo, hi = boxes if boxes is not None else instance_boxes(inst_b)
    tri = As.vertices[As.indices]
    near = np.nonzero(boxes_near(tri.min(1), tri.max(1), lo, hi))[0]
    del tri
    sub = inst_b[near].copy()
    sub["group"] = 0
    Bs = pg.expand_instances(sub)
    return As, Bs, near


def sample_keys_global(keys: np.ndarray, near: np.ndarray) -> np.ndarray:
    """Pair keys (a << 32 | local b) of a sample -> keys with global b ids, sorted."""
    a = keys >> np.uint64(32)
    b = near.astype(np.uint64)[(keys & np.uint64(0xFFFFFFFF)).astype(np.int64)]
    return np.sort((a << np.uint64(32)) | b)


def run_reference_tubes(args):
    """CPU restatement of the reference's overlap join (the oracle port, all
    host threads) on the tube workload: each step joins the first
    --cpu-sample-tubes tubes with every ellipsoid near them; the join
    queries/s of the whole join are the sample's time scaled by the tube
    count (every tube holds the same triangle budget)."""
    from oracle import pyoracle as O
    O.build()
    n_tubes, _ = tube_counts(args.scale)
    k = max(1, min(n_tubes, args.cpu_sample_tubes))
    t0 = time.perf_counter()
    As, Bs, near = tube_sample(k, args.scale)
    prep_s = time.perf_counter() - t0
    for _ in range(max(args.warmup, 0)):
        O.overlap_keys(As, Bs)
    times, npairs = [], 0
    for _ in range(args.steps):
        t1 = time.perf_counter()
        keys, _ = O.overlap_keys(As, Bs)
        times.append(time.perf_counter() - t1)
        npairs = len(keys)
    step_s = statistics.mean(times)
    full_s = step_s * n_tubes / k
    value = 1.0 / full_s
    sample = (f"tubes 0..{k - 1} ({As.num_triangles} triangles) of {n_tubes} against the {len(near)} ellipsoids "
              f"near them ({Bs.num_triangles} triangles): {step_s:.3f} s per step ({npairs} pairs), "
              f"scaled by {n_tubes}/{k}; sample set-up {prep_s:.1f} s untimed")
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 * step_s,
            "ms_per_join_extrapolated": 1000.0 * full_s, "sample_fraction": k / n_tubes,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32 (exact predicates)",
            "data": "synthetic", "config": tubes_config(args.scale),
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": O.max_threads(), "kind": "port",
                             "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


def run_reference(args):
    """CPU restatement of the reference path (the oracle port), all host
    threads, on the workload of --workload; rank 0 only."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    if args.workload == "tubes":
        return run_reference_tubes(args)
    from oracle import pyoracle as O
    O.build()
    A, B, cfg = workload(args.scale)
    As, Bs, frac = cpu_sample(A, B, args.cpu_sample_objects)
    threads = O.max_threads()
    for _ in range(max(args.warmup, 0)):
        cpu_join_seconds(As, Bs)
    times = [cpu_join_seconds(As, Bs) for _ in range(args.steps)]
    step_s = statistics.mean(times)
    full_s = step_s / max(frac, 1e-12)   # seconds for the full workload's 2 joins
    value = 2.0 / full_s
    sample = (f"spatial sub-cube holding {As.num_objects}+{Bs.num_objects} of "
              f"{A.num_objects}+{B.num_objects} objects (fraction {frac:.4f}); time scaled by 1/fraction")
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 * step_s,
            "ms_per_step_extrapolated": 1000.0 * full_s, "sample_fraction": frac,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32/exact",
            "data": "synthetic", "config": cfg,
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


def main_batched(args):
    """4,096 independent overlap joins: waves of partitioned joins, each wave
    captured as a CUDA graph with autotuned settings, against the same
    queries run one join call each (plain form and tuned form)."""
    import torch
    from pierce_gb300 import batched as BT
    from pierce_gb300 import join as J
    log = lambda m: print(m, file=sys.stderr, flush=True)
    ctx = J.Context(0)
    n_queries = max(1, int(round(4096 * args.scale)))
    t0 = time.perf_counter()
    qs = BT.workload(seed=3, queries=n_queries)
    waves = BT.make_waves(qs, budget_tris=args.wave_tris)
    gen_s = time.perf_counter() - t0
    tris = sum(w.tris for w in waves)
    log(f"{n_queries} queries, {tris / 1e9:.2f} G triangles, {len(waves)} waves ({gen_s:.1f} s host parameters)")

    # autotune on the first wave
    t = J.default_tuning(defer_build=1)
    A0 = J.Dataset.from_instances(ctx, waves[0].a, t)
    B0 = J.Dataset.from_instances(ctx, waves[0].b, t)
    base = J.make_opts(predicate="overlap", expected_pairs=BT.expected_pairs(waves[0]))
    best, trials = J.autotune(ctx, A0, B0, base, repeats=2)
    A0.close()
    B0.close()
    log(f"autotuned: {best}")

    def opts_fn(w):
        return J.tuned_opts(J.make_opts(predicate="overlap", expected_pairs=BT.expected_pairs(w)), best)

    clocks = Clocks(clocks_path("clocks_batched.csv"))
    with clocks:
        bat = BT.run_batched(ctx, waves, opts_fn, warmup=max(1, args.warmup), replays=max(1, args.steps),
                             log=log, keep_pairs=True)
    value = n_queries / (bat["ms"] / 1000.0)
    log(f"batched: {bat['ms']:.1f} ms for {n_queries} queries")
    # the same queries one join call each: the plain form, and the tuned form
    plain_opts = J.make_opts(predicate="overlap", sizing="two_pass", precision="fp32", cull_objects=False,
                             defer_exact=False, active_bvh=False)
    plain = BT.run_per_query(ctx, qs, plain_opts, build_leaf=args.plain_leaf_size, log=log, keep_pairs=True)
    log(f"plain per query: {plain['s']:.2f} s")
    tuned_q = J.tuned_opts(J.make_opts(predicate="overlap", sizing="hash"), best)
    per_q = BT.run_per_query(ctx, qs, tuned_q, log=log, keep_pairs=True)
    log(f"tuned per query: {per_q['s']:.2f} s")
    empty = np.zeros((0, 2), np.int32)
    mism_plain = sum(not np.array_equal(bat["results"].get(i, empty), plain["results"].get(i, empty))
                     for i in range(n_queries))
    mism_tuned = sum(not np.array_equal(bat["results"].get(i, empty), per_q["results"].get(i, empty))
                     for i in range(n_queries))
    launches_per_wave = [w["launches"] for w in bat["waves"]]
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": 1, "steps": args.steps,
        "warmup": max(1, args.warmup), "ms_per_step": bat["ms"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32 (exact predicates)", "data": "synthetic",
        "config": {"workload": "batched-overlap-4096-queries", "queries": n_queries, "triangles": tris,
                   "meshes_per_side": "log-uniform [10, 10000]", "levels": "1..5", "waves": len(waves),
                   "wave_triangle_budget": args.wave_tris,
                   "l2": "inputs larger than L2 (every wave holds >100 MB of geometry)",
                   "timing": "per wave: mean of the timed replays of its CUDA graph (CUDA events); "
                             "device expansion of the inputs not timed"},
        "autotuned": best, "autotune_trials": len(trials),
        "pairs": bat["pairs"],
        "plain_per_query": {"value": n_queries / plain["s"], "unit": UNIT, "s": plain["s"],
                            "form": "dataset BVH builds + fp32 two-pass join, no culling, one join call per query",
                            "mismatching_queries": int(mism_plain),
                            "batched_speedup": (n_queries / (bat["ms"] / 1000.0)) / (n_queries / plain["s"])},
        "tuned_per_query": {"value": n_queries / per_q["s"], "unit": UNIT, "s": per_q["s"],
                            "mismatching_queries": int(mism_tuned),
                            "batched_speedup": (n_queries / (bat["ms"] / 1000.0)) / (n_queries / per_q["s"])},
        "expand_s": bat["expand_s"], "plan_and_capture_s": bat["plan_s"],
        "gpu_launches": int(sum(launches_per_wave) * max(1, args.steps)),
        "graph_launches_per_step": len(waves), "clocks": clocks.summary(0),
    }
    print(json.dumps(line))
    return 0


TRIANGLE_FIELDS = ("vertices", "indices", "tri_to_object")


def pinned_view(G, keep: list, edges: bool = True, ranges: bool = False):
    """A pierce_mesh_view over pinned host copies of G's arrays (the copies
    are appended to keep; without `edges`, the edge arrays are left out and
    the view holds none; with `ranges` and a mesh stored object by object,
    the objects go as triangle offsets instead of per-triangle ids).
    Returns (view, bytes of the triangle arrays, bytes of the edge arrays)."""
    import torch
    from pierce_gb300 import capi
    from pierce_gb300 import join as J
    off = J.object_offsets(G.tri_to_object, G.num_objects) if ranges else None
    ptr, nbytes = {}, {}
    for field in ("vertices", "indices", "tri_to_object", "edge_starts", "edge_ends", "edge_src"):
        if (not edges and field not in TRIANGLE_FIELDS) or (field == "tri_to_object" and off is not None):
            ptr[field], nbytes[field] = 0, 0
            continue
        src = np.ascontiguousarray(getattr(G, field))
        pin = torch.empty(max(src.nbytes, 1), dtype=torch.uint8, pin_memory=True)
        pin.numpy()[:src.nbytes] = src.view(np.uint8).reshape(-1)
        keep.append(pin)
        ptr[field] = pin.data_ptr()
        nbytes[field] = src.nbytes
    v = capi.MeshView()
    v.vertices, v.num_vertices = ptr["vertices"], G.vertices.shape[0]
    v.indices, v.num_triangles = ptr["indices"], G.num_triangles
    v.tri_to_object = ptr["tri_to_object"]
    v.edge_starts, v.edge_ends, v.edge_src = ptr["edge_starts"], ptr["edge_ends"], ptr["edge_src"]
    v.num_edges, v.num_objects = (G.num_edges if edges else 0), G.num_objects
    tri = sum(nbytes[f] for f in TRIANGLE_FIELDS)
    if off is not None:
        keep.append(off)
        v.object_offsets = off.ctypes.data
        tri += off.nbytes
    return v, tri, sum(nbytes.values()) - tri + (off.nbytes if off is not None else 0)


def range_view(v, G, keep: list):
    """A copy of view v (over the same pinned arrays) without edges and, when
    G is stored object by object, with its objects as triangle offsets
    instead of per-triangle ids.  Returns (view, bytes it uploads)."""
    from pierce_gb300 import capi
    from pierce_gb300 import join as J
    r = capi.MeshView.from_buffer_copy(v)
    r.edge_starts = r.edge_ends = r.edge_src = None
    r.num_edges = 0
    nbytes = 12 * G.vertices.shape[0] + 12 * G.num_triangles
    off = J.object_offsets(G.tri_to_object, G.num_objects)
    if off is None:
        return r, nbytes + 4 * G.num_triangles
    keep.append(off)
    r.tri_to_object = None
    r.object_offsets = off.ctypes.data
    return r, nbytes + off.nbytes


class E2E:
    """One end-to-end join through the C ABI: both datasets created from
    pinned host buffers (views with every `.pre` array), the join, the pairs
    copied to pinned host memory, the datasets destroyed."""

    def __init__(self, ctx, views, out_pairs: int):
        import torch
        from pierce_gb300 import capi
        self.ctx, self.views = ctx, views
        self.L = capi.lib()
        self.out = torch.empty(8 * out_pairs, dtype=torch.uint8, pin_memory=True)

    def step(self, opts, upload, build_tuning=None, want_keys=False):
        """upload: the datasets' pierce_tuning (skip_edges = 1: the edge
        arrays are neither read nor copied)."""
        import ctypes as C
        from pierce_gb300 import capi
        from pierce_gb300 import join as J
        L, ctx = self.L, self.ctx
        ha, hb = C.c_void_p(), C.c_void_p()
        capi.check(L.pierce_dataset_create(ctx.handle, C.byref(self.views[0]), capi.HOST_MEMORY, C.byref(upload),
                                           C.byref(ha)), "dataset A")
        capi.check(L.pierce_dataset_create(ctx.handle, C.byref(self.views[1]), capi.HOST_MEMORY, C.byref(upload),
                                           C.byref(hb)), "dataset B")
        if build_tuning is not None:
            capi.check(L.pierce_dataset_build(ctx.handle, ha, C.byref(build_tuning)), "build A")
            capi.check(L.pierce_dataset_build(ctx.handle, hb, C.byref(build_tuning)), "build B")
        r = C.c_void_p()
        st = capi.Stats()
        capi.check(L.pierce_join(ctx.handle, ha, hb, C.byref(opts), C.byref(r), C.byref(st)), "join")
        n = C.c_uint64()
        L.pierce_result_count(r, C.byref(n))
        cap = min(n.value, self.out.numel() // 8)
        capi.check(L.pierce_result_copy(ctx.handle, r, self.out.data_ptr(), cap), "copy")
        keys = J.pairs_to_keys(self.out.numpy()[:8 * cap].view(np.int32).reshape(-1, 2).copy()) if want_keys else None
        L.pierce_result_destroy(r)
        L.pierce_dataset_destroy(ha)
        L.pierce_dataset_destroy(hb)
        return st.as_dict(), keys, 8 * cap


def tubes_replica_tail(args, ctx, da, db, A, B, tuned_o, tuned_ms, keys_t, launches, clocks, rank, world,
                       local_rank, dist):
    """The tube line under torchrun: every rank has timed its replica of the
    device-resident join; each now times the end-to-end join from pinned
    host buffers without edges (the tuned form's upload), the times are
    maxed over ranks, and rank 0 prints the line."""
    import torch
    from pierce_gb300 import capi
    from pierce_gb300 import join as J
    da.close()
    db.close()
    ctx.release_scratch()
    keep = []
    va, a_tri, _ = pinned_view(A, keep, edges=False, ranges=True)
    vb, b_tri, _ = pinned_view(B, keep, edges=False, ranges=True)
    e2e = E2E(ctx, (va, vb), out_pairs=max(1 << 22, 2 * len(keys_t)))
    upload_tri = J.default_tuning(leaf_size=args.leaf_size, defer_build=1, skip_edges=1)
    tri_o = capi.JoinOpts.from_buffer_copy(tuned_o)
    if tri_o.edge_source == capi.EDGES_DATASET:
        tri_o.edge_source = capi.EDGES_AUTO
    _, keys_e, d2h = e2e.step(tri_o, upload_tri, want_keys=True)
    ctx.synchronize()
    dist.barrier()
    n = max(1, min(args.steps, 5))
    t1 = time.perf_counter()
    for _ in range(n):
        e2e.step(tri_o, upload_tri, None)
    e2e_s = max_over_ranks((time.perf_counter() - t1) / n, dist)
    identical = bool(np.array_equal(keys_e, keys_t))
    if rank == 0:
        line = {
            "metric": METRIC, "value": world * 1000.0 / tuned_ms, "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": max(args.warmup, 3), "ms_per_step": tuned_ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32 (exact predicates)", "data": "synthetic",
            "config": tubes_config(args.scale),
            "settings": {"parallelism": f"replicas x{world}", "sizing": "learned",
                         "precision": "exact (fp32 filter, fp64, expansions)"},
            "pairs": len(keys_t), "identical_e2e": identical,
            "e2e": {"value": world / e2e_s, "unit": UNIT, "h2d_bytes_per_step": int(world * (a_tri + b_tri)),
                    "d2h_bytes_per_step": int(world * d2h), "ms_per_step": 1000.0 * e2e_s, "edges_uploaded": False},
            "gpu_launches": int(launches) * world, "clocks": clocks.summary(local_rank),
        }
        print(json.dumps(line))
    dist.destroy_process_group()
    return 0


def main_tubes(args):
    """Large tube-mesh overlap join (the default line): the tuned form with
    inputs resident in HBM (value), end to end through the C ABI (e2e), the
    plain GPU form, the edge-ray roofline and the CPU oracle on a sample.
    Under torchrun every rank runs a replica of the join on its own GPU
    (weak scaling, max time over ranks); rank 0 alone adds the plain form,
    the CPU sample and the upload with edges, and prints the line."""
    import torch
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local_rank)
        dist.init_process_group("nccl")
    import pierce_gb300 as pg
    from pierce_gb300 import capi
    from pierce_gb300 import join as J
    from pierce_gb300 import sizing as S
    from oracle import pyoracle as O
    log = lambda m: print(m, file=sys.stderr, flush=True)
    n_tubes, n_ell = tube_counts(args.scale)
    t0 = time.perf_counter()
    A = tube_geometry(args.scale)
    inst_b = ellipsoid_instances(args.scale)
    inst_b_host = inst_b.copy()
    inst_b_host["group"] = 0
    B = pg.expand_instances(inst_b_host)
    log(f"tubes {A.num_triangles / 1e6:.0f} M tris, ellipsoids {B.num_triangles / 1e6:.0f} M tris "
        f"({time.perf_counter() - t0:.1f} s host generation)")

    # CPU oracle on a sample: the first k tubes against every ellipsoid near them
    cpu, cpu_touch, sample_keys, ref_sem = None, None, None, None
    k = max(1, min(n_tubes, args.cpu_sample_tubes))
    if not (args.no_cpu_baseline or args.only_tuned or rank != 0):
        tb = time.perf_counter()
        As, Bs, near = tube_sample(k, args.scale, inst_b, boxes=mesh_boxes(B))
        prep_s = time.perf_counter() - tb
        tc = time.perf_counter()
        cpu_keys, _ = O.overlap_keys(As, Bs)
        cpu_s = time.perf_counter() - tc
        sample_keys = sample_keys_global(cpu_keys, near)
        cpu = {"value": 1.0 / (cpu_s * n_tubes / k), "unit": UNIT, "cores": O.max_threads(), "kind": "port",
               "sample": (f"tubes 0..{k - 1} of {n_tubes} against the {len(near)} ellipsoids near them: "
                          f"{cpu_s:.2f} s, scaled by {n_tubes}/{k}")}
        # the reference's second CPU baseline, TOUCH, on the same sample
        tt = time.perf_counter()
        touch_keys, touch_cand = O.touch_keys(As, Bs)
        touch_s = time.perf_counter() - tt
        cpu_touch = {"value": 1.0 / (touch_s * n_tubes / k), "unit": UNIT, "cores": O.max_threads(),
                     "kind": "port (TOUCH: STR tree fanout 2, exact refinement)",
                     "sample": f"the same sample: {touch_s:.2f} s, {touch_cand} candidates, scaled by {n_tubes}/{k}",
                     "pairs_equal_oracle": bool(np.array_equal(touch_keys, cpu_keys))}
        # |exact set Δ the reference's edge-ray semantics| on the same sample
        ref_sem = O.reference_semantics_diff(As, Bs, 100)
        ref_sem["sample"] = f"tubes 0..{k - 1} against the {len(near)} ellipsoids near them"
        log(f"cpu sample: {k} tubes vs {len(near)} ellipsoids: {cpu_s:.2f} s ({prep_s:.1f} s set-up), "
            f"{len(sample_keys)} pairs; TOUCH {touch_s:.2f} s; reference semantics {ref_sem}")

    ctx = J.Context(local_rank)
    upload = J.default_tuning(leaf_size=args.leaf_size, defer_build=1)
    model = S.SizingModel.load(ctx, S.TRAINED_MODEL)
    tuned_o = J.make_opts(predicate="overlap", sizing="learned", sizing_model=model)
    plain_o = J.make_opts(predicate="overlap", sizing="two_pass", precision="fp32", cull_objects=False,
                          defer_exact=False, active_bvh=False)
    plain_build = J.default_tuning(leaf_size=args.plain_leaf_size)
    stream = torch.cuda.ExternalStream(ctx.stream, device=torch.device("cuda", local_rank))

    # device-resident legs: inputs already in HBM (profiling runs skip the
    # edge arrays, which only the plain form reads)
    resident = J.default_tuning(leaf_size=args.leaf_size, defer_build=1, skip_edges=1 if args.only_tuned else 0)
    da = J.Dataset.from_geometry(ctx, A, resident)
    db = J.Dataset.from_geometry(ctx, B, resident)
    # the library's autotuner picks leaf size, rays per fetch, stack depth,
    # hash load factor and traversal form for this join (untimed)
    autotuned, n_trials = None, 0
    if not args.no_autotune:
        ta = time.perf_counter()
        autotuned, trials = J.autotune(ctx, da, db, tuned_o, repeats=2)
        n_trials = len(trials)
        tuned_o = J.tuned_opts(tuned_o, autotuned)
        ctx.release_scratch()
        log(f"autotuned in {time.perf_counter() - ta:.1f} s over {n_trials} trials: {autotuned}")
    for _ in range(max(args.warmup, 3)):
        r = J.run_join(ctx, da, db, tuned_o, download=False)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    clocks = Clocks(clocks_path(f"clocks_tubes_rank{rank}.csv" if world > 1 else "clocks_tubes.csv"))
    l0 = ctx.kernel_launches
    stats = []
    with clocks:
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        if args.only_tuned:
            torch.cuda.nvtx.range_push("timed")  # profilers select the timed joins by this range
        e0.record(stream)
        for _ in range(args.steps):
            r = J.run_join(ctx, da, db, tuned_o, download=False)
            stats.append(r.stats)
        e1.record(stream)
        e1.synchronize()
        if args.only_tuned:
            torch.cuda.nvtx.range_pop()
    launches = ctx.kernel_launches - l0
    tuned_ms = max_over_ranks(e0.elapsed_time(e1), dist) / args.steps
    st = stats[-1]
    if args.only_tuned and world == 1:
        print(json.dumps({"metric": METRIC, "value": 1000.0 / tuned_ms, "unit": UNIT, "ms_per_step": tuned_ms,
                          "partial": "only the tuned device-resident joins", "config": tubes_config(args.scale),
                          "autotuned": autotuned,
                          "stats": {k2: st[k2] for k2 in ("ms_total", "ms_build", "ms_edge_rays", "ms_dedup",
                                                          "ms_sizing", "rays", "tri_tests", "node_visits",
                                                          "raw_hits", "active_triangles", "launches")},
                          "gpu_launches": int(launches)}))
        return 0
    tuned = J.run_join(ctx, da, db, tuned_o)
    keys_t = J.pairs_to_keys(tuned.pairs)
    ctx.release_scratch()
    if world > 1:
        return tubes_replica_tail(args, ctx, da, db, A, B, tuned_o, tuned_ms, keys_t, launches, clocks, rank,
                                  world, local_rank, dist)

    # plain form on the same resident data: dataset hierarchies + two-pass join
    def plain_dev():
        da.build(plain_build)
        db.build(plain_build)
        return J.run_join(ctx, da, db, plain_o, download=False)

    plain_dev()
    torch.cuda.synchronize()
    p0, p1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    plain_steps = max(1, min(args.steps, 3))
    p0.record(stream)
    for _ in range(plain_steps):
        plain_dev()
    p1.record(stream)
    p1.synchronize()
    plain_ms = p0.elapsed_time(p1) / plain_steps
    keys_p = J.pairs_to_keys(J.run_join(ctx, da, db, plain_o).pairs)
    identical = bool(np.array_equal(keys_t, keys_p))
    sample_match = None
    if sample_keys is not None:
        sample_match = bool(np.array_equal(np.sort(keys_t[(keys_t >> np.uint64(32)) < np.uint64(k)]), sample_keys))
    log(f"tuned {tuned_ms:.2f} ms, plain {plain_ms:.2f} ms; {len(keys_t)} pairs; tuned == plain: {identical}; "
        f"sample == oracle: {sample_match}")
    da.close()
    db.close()
    ctx.release_scratch()

    # end to end through the C ABI from pinned host buffers.  The tuned form
    # traces its kept triangles' edges, so its datasets skip the edge arrays
    # (skip_edges); the plain form traces the edge list and uploads it.
    keep = []
    va, a_tri, a_edge = pinned_view(A, keep)
    vb, b_tri, b_edge = pinned_view(B, keep)
    e2e = E2E(ctx, (va, vb), out_pairs=max(1 << 22, 2 * len(keys_t)))
    upload_tri = J.default_tuning(leaf_size=args.leaf_size, defer_build=1, skip_edges=1)
    # the tuned form's upload: the same pinned arrays, no edges, and the
    # objects as triangle offsets (both meshes are stored object by object)
    ra, ra_tri = range_view(va, A, keep)
    rb, rb_tri = range_view(vb, B, keep)
    e2e_tri = E2E(ctx, (ra, rb), out_pairs=max(1 << 22, 2 * len(keys_t)))

    def timed(opts, up, build, n, runner=e2e):
        runner.step(opts, up, build)
        ctx.synchronize()
        t1 = time.perf_counter()
        for _ in range(n):
            runner.step(opts, up, build)
        dt = (time.perf_counter() - t1) / n
        ctx.release_scratch()
        return dt

    # datasets uploaded without edges trace the kept triangles' edges
    tri_o = capi.JoinOpts.from_buffer_copy(tuned_o)
    if tri_o.edge_source == capi.EDGES_DATASET:
        tri_o.edge_source = capi.EDGES_AUTO
    _, keys_e, d2h = e2e_tri.step(tri_o, upload_tri, want_keys=True)
    e2e_identical = bool(np.array_equal(keys_e, keys_t))
    e2e_s = timed(tri_o, upload_tri, None, max(1, min(args.steps, 5)), e2e_tri)
    e2e_edges_s = timed(tuned_o, upload, None, max(1, min(args.steps, 2)))
    plain_e2e_s = timed(plain_o, upload, plain_build, max(1, min(args.steps, 2)))
    log(f"e2e tuned {1000 * e2e_s:.1f} ms ({1000 * e2e_edges_s:.1f} ms uploading the edges too), "
        f"plain {1000 * plain_e2e_s:.1f} ms")

    # roofline of the dominant kernel: the edge rays of both directions
    edge_ms = st["ms_edge_rays"][0] + st["ms_edge_rays"][1]
    act = st["active_triangles"]
    traced_bytes = traced_edge_ray_bytes(st["rays"], st["raw_hits"], [(B, act[1]), (A, act[0])])
    achieved = traced_bytes / (edge_ms / 1000.0) / 1e9 if edge_ms > 0 else 0.0
    peak, peak_kind = peaks()
    cfg = tubes_config(args.scale)
    line = {
        "metric": METRIC, "value": 1000.0 / tuned_ms, "unit": UNIT, "n_gpus": 1, "steps": args.steps,
        "warmup": max(args.warmup, 3), "ms_per_step": tuned_ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32 (exact predicates)", "data": "synthetic", "config": cfg,
        "settings": {"leaf_size": args.leaf_size, "plain_leaf_size": args.plain_leaf_size, "sizing": "learned",
                     "precision": "exact (fp32 filter, fp64, expansions)", "parallelism": "single GPU",
                     "autotuned": autotuned, "autotune_trials": n_trials},
        "sizes": {"tube_triangles": A.num_triangles, "tube_edges": A.num_edges,
                  "ellipsoid_triangles": B.num_triangles, "ellipsoid_edges": B.num_edges},
        "ray_tri_tests_per_s": st["tri_tests"] / (st["ms_total"] / 1000.0) if st["ms_total"] > 0 else None,
        "rays_per_s": st["rays"] / (edge_ms / 1000.0) if edge_ms > 0 else None,
        "pairs": len(keys_t), "identical_tuned_plain": identical, "identical_e2e": e2e_identical,
        "sample_matches_oracle": sample_match,
        "phase_ms": {"total": st["ms_total"], "builds_and_culling": st["ms_build"],
                     "edge_rays": st["ms_edge_rays"], "dedup": st["ms_dedup"], "sizing": st["ms_sizing"]},
        "tuned_stats": {k2: st[k2] for k2 in ("rays", "tri_tests", "node_visits", "raw_hits", "fp32_ambiguous",
                                              "fp64_ambiguous", "predicted_pairs", "sizing_overflow", "hash_slots",
                                              "active_triangles", "launches")},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak if peak else None, "traffic": traffic_estimate(st["rays"], "tubes"),
                     "kernel": "k_edge_rays, both directions of the tube join", "peak_kind": peak_kind,
                     "algorithmic_bytes": traced_bytes, "kernel_ms": edge_ms},
        "plain": {"value": 1000.0 / plain_ms, "unit": UNIT, "ms_per_step": plain_ms,
                  "form": "dataset BVH builds + fp32 Moller-Trumbore two-pass join, no culling",
                  "tuned_speedup": plain_ms / tuned_ms,
                  "e2e": {"value": 1.0 / plain_e2e_s, "ms_per_step": 1000.0 * plain_e2e_s,
                          "h2d_bytes_per_step": int(a_tri + b_tri + a_edge + b_edge)},
                  "e2e_speedup_tuned": plain_e2e_s / e2e_s},
        "e2e": {"value": 1.0 / e2e_s, "unit": UNIT, "h2d_bytes_per_step": int(ra_tri + rb_tri),
                "d2h_bytes_per_step": int(d2h), "ms_per_step": 1000.0 * e2e_s,
                "edges_uploaded": False, "objects_as_ranges": True,
                "with_edge_upload": {"value": 1.0 / e2e_edges_s, "ms_per_step": 1000.0 * e2e_edges_s,
                                     "h2d_bytes_per_step": int(a_tri + b_tri + a_edge + b_edge)}},
        "reference_semantics_diff": ref_sem,
        "cpu_baseline": cpu, "cpu_baseline_touch": cpu_touch, "gpu_launches": int(launches),
        "clocks": clocks.summary(0),
    }
    print(json.dumps(line))
    return 0


def main_preprocess(args):
    """Edge extraction of the `.pre` producer (host code, no GPU): read a
    `.pre` file, extract the unique per-object edges in the reference's map
    order, write the file.  This repository's extractor (all host threads,
    and one thread) against the reference's own EdgePreprocessor::extractEdges
    with its BinaryIO reader and writer, compiled from the reference sources
    into oracle/_ref/ref_pre_tool where they are present.  Workload: side A
    of the plain overlap configuration, 2,000 level-3 icospheres (2.56 M
    triangles, 3.84 M unique edges)."""
    import pierce_gb300 as pg
    log = lambda m: print(m, file=sys.stderr, flush=True)
    n = max(10, int(round(2000 * args.scale)))
    G = pg.icospheres(2024, n, 3, hi=200.0 * args.scale ** (1.0 / 3.0))
    tris = G.num_triangles
    work = Path(tempfile.mkdtemp(prefix="pierce_pre_"))
    src = work / "in.pre"
    G.write_pre(src)

    def ours(threads):
        t0 = time.perf_counter()
        H = pg.Geometry.read_pre(src)
        H.extract_edges(0, threads)
        H.write_pre(work / "ours.pre")
        return time.perf_counter() - t0

    def reference():
        tool = ROOT / "oracle" / "_ref" / "ref_pre_tool"
        if not tool.exists():
            return None
        t0 = time.perf_counter()
        r = subprocess.run([str(tool), str(src), str(work / "ref.pre")], capture_output=True, text=True)
        if r.returncode != 0:
            return None
        return time.perf_counter() - t0

    for _ in range(max(args.warmup, 0)):
        ours(0)
    t_all = min(ours(0) for _ in range(max(args.steps, 1)))
    t_one = min(ours(1) for _ in range(max(args.steps, 1)))
    ref = [reference() for _ in range(max(args.steps, 1))]
    t_ref = None if any(r is None for r in ref) else min(ref)
    identical = None
    if t_ref is not None:
        a, b = (work / "ref.pre").read_bytes(), (work / "ours.pre").read_bytes()
        identical = len(a) == len(b) and a[:50] == b[:50] and a[56:] == b[56:]  # header padding excluded
    def grid_seconds():
        H = pg.Geometry.read_pre(src)
        t0 = time.perf_counter()
        H.grid_stats(8.0)
        return time.perf_counter() - t0

    t_grid = min(grid_seconds() for _ in range(max(args.steps, 1)))
    threads = os.cpu_count() or 1
    log(f"preprocess: {tris} triangles; ours {t_all:.3f} s ({threads} threads), {t_one:.3f} s (1 thread); "
        f"reference {t_ref if t_ref is None else round(t_ref, 3)} s; identical {identical}")
    line = {"metric": "edge extraction of the .pre producer (read, extract, write)", "unit": "triangles/s",
            "value": tris / t_all, "value_one_thread": tris / t_one, "threads": threads,
            "reference": None if t_ref is None else {"value": tris / t_ref, "threads": 1,
                                                     "kind": "reference (EdgePreprocessor, BinaryIO)"},
            "byte_identical_to_reference": identical, "grid_stats_s": t_grid, "steps": args.steps,
            "warmup": args.warmup,
            "higher_is_better": True, "data": "synthetic",
            "config": {"workload": "pre-edge-extraction", "meshes": n, "subdivision": 3,
                       "triangles": tris, "edges": G.num_edges, "seed": 2024}}
    print(json.dumps(line))
    for f in ("in.pre", "ours.pre", "ref.pre"):
        (work / f).unlink(missing_ok=True)
    work.rmdir()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="pierce", choices=["pierce", "reference"])
    ap.add_argument("--scale", type=float, default=1.0, help="fraction of the full workload (debug only)")
    ap.add_argument("--cpu-sample-objects", type=int, default=3000)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--leaf-size", type=int, default=4, help="leaf size of the tuned form's per-join hierarchies")
    ap.add_argument("--plain-leaf-size", type=int, default=8, help="leaf size of the plain form's dataset hierarchies")
    ap.add_argument("--workload", default="tubes", choices=["tubes", "ellipsoids", "batched", "preprocess"],
                    help="tubes (default): 2,000 tubes against 100,000 ellipsoids, overlap; ellipsoids: "
                         "intersection + containment of 2 x 50,000 ellipsoids; batched: 4,096 overlap queries; "
                         "preprocess: edge extraction of the .pre producer on the host cores")
    ap.add_argument("--cpu-sample-tubes", type=int, default=10)
    ap.add_argument("--no-autotune", action="store_true", help="tubes: keep the default tuning values")
    ap.add_argument("--only-tuned", action="store_true",
                    help="tubes, ellipsoids: only the device-resident tuned joins (profiling runs; prints a "
                         "partial line)")
    ap.add_argument("--wave-tris", type=float, default=1.0e9, help="batched: triangles per wave (both sides)")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)
    if args.workload == "batched":
        return main_batched(args)
    if args.workload == "tubes":
        return main_tubes(args)
    if args.workload == "preprocess":
        return main_preprocess(args)
    return main_ellipsoids(args)


def main_ellipsoids(args):
    """Intersection + containment joins of 2 x 50,000 ellipsoids; under
    torchrun every rank runs a replica (weak scaling, max time over ranks)."""
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist
        import torch
        torch.cuda.set_device(local_rank)
        dist.init_process_group("nccl")
    import torch
    from pierce_gb300 import capi
    from pierce_gb300 import join as J
    import ctypes as C

    A, B, cfg = workload(args.scale)
    ctx = J.Context(local_rank)
    tuning = J.default_tuning(leaf_size=args.leaf_size)
    da = J.Dataset.from_geometry(ctx, A, tuning)
    db = J.Dataset.from_geometry(ctx, B, tuning)
    opts_i = J.make_opts(predicate="intersection", sizing="hash", expected_pairs=4 * A.num_objects)
    opts_c = J.make_opts(predicate="containment", sizing="hash", expected_pairs=4 * A.num_objects)
    L = capi.lib()
    stream = torch.cuda.ExternalStream(ctx.stream, device=torch.device("cuda", local_rank))

    def device_step(collect=None):
        # the joins build their own BVHs over the triangles of objects that
        # meet the other side (active_bvh), so no dataset build is needed
        ri = J.run_join(ctx, da, db, opts_i, download=False)
        rc = J.run_join(ctx, da, db, opts_c, download=False)
        if collect is not None:
            collect.append((ri, rc))
        return ri, rc

    for _ in range(args.warmup):
        device_step()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    clocks = Clocks(clocks_path(f"clocks_rank{rank}.csv"))
    collected = []
    l0 = ctx.kernel_launches
    with clocks:
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        if args.only_tuned:
            torch.cuda.nvtx.range_push("timed")  # profilers select the timed joins by this range
        e0.record(stream)
        for _ in range(args.steps):
            device_step(collected)
        e1.record(stream)
        e1.synchronize()
        if args.only_tuned:
            torch.cuda.nvtx.range_pop()
    launches = ctx.kernel_launches - l0
    ms_total = e0.elapsed_time(e1)
    ms_total = max_over_ranks(ms_total, dist)
    ms_step = ms_total / args.steps
    queries = 2 * args.steps * world
    value = queries / (ms_total / 1000.0)
    ri, rc = collected[-1]
    containment_phases = {"by_candidate_pairs": bool(rc.stats["containment_by_pairs"]),
                          "builds": rc.stats["ms_build"], "parity": sum(rc.stats["ms_parity"]),
                          "edge_rays": sum(rc.stats["ms_edge_rays"]), "total": rc.stats["ms_total"]}
    if args.only_tuned:
        if rank == 0:
            print(json.dumps({"metric": METRIC, "value": value, "unit": UNIT, "ms_per_step": ms_step,
                              "partial": "only the tuned device-resident joins", "config": cfg,
                              "intersection": {"total": ri.stats["ms_total"], "builds": ri.stats["ms_build"],
                                               "edge_rays": sum(ri.stats["ms_edge_rays"]), "rays": ri.stats["rays"]},
                              "containment": containment_phases,
                              "gpu_launches": int(launches)}))
        return 0

    # roofline of the dominant kernel: edge rays (both directions, both joins)
    edge_ms = ri.stats["ms_edge_rays"][0] + ri.stats["ms_edge_rays"][1]
    raw_hits = ri.stats["raw_hits"]
    act = ri.stats["active_triangles"]
    traced_bytes = traced_edge_ray_bytes(ri.stats["rays"], raw_hits, [(B, act[1]), (A, act[0])])
    achieved = traced_bytes / (edge_ms / 1000.0) / 1e9 if edge_ms > 0 else 0.0
    unculled_bytes = edge_ray_bytes(A, B, raw_hits / 2) + edge_ray_bytes(B, A, raw_hits / 2)
    peak, peak_kind = peaks()
    tri_tests = ri.stats["tri_tests"] + rc.stats["tri_tests"]
    join_ms = ri.stats["ms_total"] + rc.stats["ms_total"]

    # plain GPU form on the same data: float32 Moller-Trumbore without
    # fallback, no object culling, two-pass sizing (one step, same shape)
    opts_pi = J.make_opts(predicate="intersection", sizing="two_pass", precision="fp32", cull_objects=False,
                          defer_exact=False, active_bvh=False)
    opts_pc = J.make_opts(predicate="containment", sizing="two_pass", precision="fp32", cull_objects=False,
                          defer_exact=False, active_bvh=False)
    J.run_join(ctx, da, db, opts_pi, download=False)
    torch.cuda.synchronize()
    p0 = torch.cuda.Event(enable_timing=True)
    p1 = torch.cuda.Event(enable_timing=True)
    plain_tuning = J.default_tuning(leaf_size=args.plain_leaf_size)
    p0.record(stream)
    da.build(plain_tuning)
    db.build(plain_tuning)
    rpi = J.run_join(ctx, da, db, opts_pi)
    rpc = J.run_join(ctx, da, db, opts_pc)
    p1.record(stream)
    p1.synchronize()
    plain_ms = p0.elapsed_time(p1)
    exact_i = J.run_join(ctx, da, db, opts_i)
    exact_c = J.run_join(ctx, da, db, opts_c)
    ki, kpi = J.pairs_to_keys(exact_i.pairs), J.pairs_to_keys(rpi.pairs)
    kc, kpc = J.pairs_to_keys(exact_c.pairs), J.pairs_to_keys(rpc.pairs)
    plain = {"value": 2.0 / (plain_ms / 1000.0), "unit": UNIT, "ms_per_step": plain_ms,
             "form": "fp32 Moller-Trumbore, no culling, two-pass sizing",
             "mismatch_vs_exact": {"intersection": int(len(np.setxor1d(ki, kpi))),
                                   "containment": int(len(np.setxor1d(kc, kpc)))},
             "tuned_speedup": (2.0 / (ms_step / 1000.0)) / (2.0 / (plain_ms / 1000.0))}

    # e2e through the C ABI from pinned host buffers
    e2e = None
    if rank == 0:
        arrs = {}
        for name, G in (("A", A), ("B", B)):
            for field in ("vertices", "indices", "tri_to_object", "edge_starts", "edge_ends", "edge_src"):
                src = np.ascontiguousarray(getattr(G, field))
                pin = torch.empty(src.nbytes, dtype=torch.uint8, pin_memory=True)
                pin.numpy()[:] = src.view(np.uint8).reshape(-1)
                arrs[(name, field)] = (pin, src.shape)
        # the tuned joins trace their kept triangles' edges: the datasets
        # skip the edge arrays (skip_edges), so only the triangle arrays move
        h2d = sum(p.numel() for (nm, f), (p, _) in arrs.items() if f in TRIANGLE_FIELDS)

        def view_of(name, G):
            v = capi.MeshView()
            v.vertices = arrs[(name, "vertices")][0].data_ptr()
            v.num_vertices = G.vertices.shape[0]
            v.indices = arrs[(name, "indices")][0].data_ptr()
            v.num_triangles = G.num_triangles
            v.tri_to_object = arrs[(name, "tri_to_object")][0].data_ptr()
            v.edge_starts = arrs[(name, "edge_starts")][0].data_ptr()
            v.edge_ends = arrs[(name, "edge_ends")][0].data_ptr()
            v.edge_src = arrs[(name, "edge_src")][0].data_ptr()
            v.num_edges = G.num_edges
            v.num_objects = G.num_objects
            return v

        # both meshes are stored object by object: the objects go as
        # triangle offsets (the library writes the per-triangle ids)
        keep_off = []
        va, ha_bytes = range_view(view_of("A", A), A, keep_off)
        vb, hb_bytes = range_view(view_of("B", B), B, keep_off)
        h2d = ha_bytes + hb_bytes
        upload_only = J.default_tuning(leaf_size=args.leaf_size, defer_build=1, skip_edges=1)
        out_pairs = torch.empty(8 * (1 << 22), dtype=torch.uint8, pin_memory=True)

        def e2e_step():
            ha, hb = C.c_void_p(), C.c_void_p()
            capi.check(L.pierce_dataset_create(ctx.handle, C.byref(va), capi.HOST_MEMORY, C.byref(upload_only),
                                               C.byref(ha)), "e2e dataset A")
            capi.check(L.pierce_dataset_create(ctx.handle, C.byref(vb), capi.HOST_MEMORY, C.byref(upload_only),
                                               C.byref(hb)), "e2e dataset B")
            d2h = 0
            for o in (opts_i, opts_c):
                r = C.c_void_p()
                capi.check(L.pierce_join(ctx.handle, ha, hb, C.byref(o), C.byref(r), None), "e2e join")
                n = C.c_uint64()
                L.pierce_result_count(r, C.byref(n))
                cap = out_pairs.numel() // 8
                capi.check(L.pierce_result_copy(ctx.handle, r, out_pairs.data_ptr(), min(n.value, cap)),
                           "e2e copy")
                d2h += 8 * min(n.value, cap)
                L.pierce_result_destroy(r)
            L.pierce_dataset_destroy(ha)
            L.pierce_dataset_destroy(hb)
            return d2h

        e2e_step()
        t0 = time.perf_counter()
        d2h_total = 0
        e2e_steps = max(1, min(args.steps, 3))
        for _ in range(e2e_steps):
            d2h_total += e2e_step()
        e2e_s = (time.perf_counter() - t0) / e2e_steps
        e2e = {"value": 2.0 / e2e_s, "unit": UNIT, "h2d_bytes_per_step": int(h2d),
               "d2h_bytes_per_step": int(d2h_total // e2e_steps), "ms_per_step": 1000.0 * e2e_s,
               "edges_uploaded": False, "objects_as_ranges": len(keep_off) == 2}

    cpu, ref_sem = None, None
    if rank == 0 and not args.no_cpu_baseline:
        from oracle import pyoracle as O
        As, Bs, frac = cpu_sample(A, B, args.cpu_sample_objects)
        secs = cpu_join_seconds(As, Bs)
        ref_sem = O.reference_semantics_diff(As, Bs, 100)
        ref_sem["sample"] = f"overlap pairs of the spatial sub-cube sample (fraction {frac:.4f})"
        full = secs / max(frac, 1e-12)
        cpu = {"value": 2.0 / full, "unit": UNIT, "cores": O.max_threads(), "kind": "port",
               "sample": (f"intersection+containment joins of the objects in a spatial sub-cube "
                          f"({As.num_objects}+{Bs.num_objects} of {A.num_objects}+{B.num_objects} objects, "
                          f"fraction {frac:.4f}) took {secs:.2f} s; scaled by 1/fraction")}

    if dist:
        dist.barrier()
    if rank != 0:
        return 0
    clk = clocks.summary(local_rank)
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32 (exact predicates)", "data": "synthetic", "config": cfg,
        "settings": {"leaf_size": args.leaf_size, "plain_leaf_size": args.plain_leaf_size, "sizing": "hash",
                     "precision": "exact (fp32 filter, fp64, expansions)",
                     "parallelism": f"replicas x{world}" if world > 1 else "single GPU"},
        "ray_tri_tests_per_s": tri_tests / (join_ms / 1000.0) if join_ms > 0 else None,
        "rays_per_s": (ri.stats["rays"]) / (edge_ms / 1000.0) if edge_ms > 0 else None,
        "pairs": {"intersection": ri.stats["num_pairs"], "containment": rc.stats["num_pairs"]},
        "ambiguous": {"fp32": ri.stats["fp32_ambiguous"], "fp64": ri.stats["fp64_ambiguous"],
                      "tests": ri.stats["tri_tests"]},
        "phase_ms": {"intersection": ri.stats["ms_total"], "containment": rc.stats["ms_total"],
                     "edge_rays": edge_ms, "parity": sum(ri.stats["ms_parity"]), "dedup": ri.stats["ms_dedup"],
                     "join_bvh_builds": ri.stats["ms_build"] + rc.stats["ms_build"],
                     "full_dataset_bvh_build": da.info().ms_build + db.info().ms_build},
        "containment_phases": containment_phases,
        "query_only": {"value": 2.0 / ((join_ms - ri.stats["ms_build"] - rc.stats["ms_build"]) / 1000.0),
                       "unit": UNIT, "note": "BVH builds excluded, as in the reference benchmark adapters"},
        "active_triangles": list(ri.stats["active_triangles"]),
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak if peak else None,
                     "traffic": traffic_estimate(ri.stats["rays"], "ellipsoids"),
                     "kernel": "k_edge_rays (exact, hash mode), both directions of the intersection join",
                     "peak_kind": peak_kind, "algorithmic_bytes": traced_bytes,
                     "unculled_equivalent_gbs": unculled_bytes / (edge_ms / 1000.0) / 1e9 if edge_ms > 0 else None},
        "plain": plain, "cpu_baseline": cpu, "reference_semantics_diff": ref_sem, "e2e": e2e,
        "gpu_launches": int(launches), "clocks": clk,
    }
    print(json.dumps(line))
    if dist:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
