"""Batches of independent overlap joins (4,096 queries of uneven size).

Workload: per query, meshes per side log-uniform in [10, 10,000]; every mesh
an icosphere of subdivision level uniform in 1..5 (80 .. 20,480 triangles)
with radius lognormal(ln 1.5, 0.4); centres uniform in a per-query cube
whose side gives a mean of 0.5 overlapping partners per mesh (expected pairs
0.25 (nA + nB), from the shell of centre distances in which two spheres'
surfaces meet).

The batched form runs many queries as one partitioned join: each side of a
wave of queries is one dataset whose objects are partitioned by query, so
one hierarchy build (a subtree per query), one culling pass, one persistent
edge-ray launch fed from a device ray queue and one de-duplication serve
every query of the wave.  The wave's whole join is captured as a CUDA graph
and replayed.  Waves bound the device memory: the full batch holds tens of
billions of triangles, far more than one GPU holds at once.
"""
from __future__ import annotations

import math
import time
from dataclasses import dataclass

import numpy as np

from .capi import INSTANCE_DTYPE
from .geometry import SPHERES, instances

LN_MU, SIGMA = math.log(1.5), 0.4


@dataclass
class Query:
    seed_a: int
    seed_b: int
    n_a: int
    n_b: int
    extent: float


def shell_volume(rng: np.random.Generator, k: int = 1 << 16) -> float:
    ra = np.exp(LN_MU + SIGMA * rng.standard_normal(k))
    rb = np.exp(LN_MU + SIGMA * rng.standard_normal(k))
    return float((4.0 / 3.0) * math.pi * np.mean((ra + rb) ** 3 - np.abs(ra - rb) ** 3))


def workload(seed: int = 3, queries: int = 4096, n_lo: int = 10, n_hi: int = 10_000,
             overlaps_per_mesh: float = 0.5) -> list[Query]:
    rng = np.random.default_rng(seed)
    shell = shell_volume(np.random.default_rng(seed + 1))
    out = []
    for _ in range(queries):
        n_a = int(round(math.exp(rng.uniform(math.log(n_lo), math.log(n_hi)))))
        n_b = int(round(math.exp(rng.uniform(math.log(n_lo), math.log(n_hi)))))
        pairs = overlaps_per_mesh * 0.5 * (n_a + n_b)
        sel = pairs / (n_a * n_b)
        out.append(Query(int(rng.integers(1, 2**62)), int(rng.integers(1, 2**62)), n_a, n_b,
                         (shell / sel) ** (1.0 / 3.0)))
    return out


def side_instances(q: Query, side: int, level_lo: int = 1, level_hi: int = 5) -> np.ndarray:
    seed, n = (q.seed_a, q.n_a) if side == 0 else (q.seed_b, q.n_b)
    return instances(seed, n, SPHERES, level_lo, level_hi, p0=LN_MU, p1=SIGMA, hi=q.extent)


def triangles(inst: np.ndarray) -> int:
    return int((20 * 4 ** inst["level"].astype(np.int64)).sum())


@dataclass
class Wave:
    queries: list[int]
    a: np.ndarray          # instances of side A, group = query index within the wave
    b: np.ndarray
    tris: int


def make_waves(qs: list[Query], budget_tris: float = 1.0e9) -> list[Wave]:
    """Consecutive queries packed into waves of at most budget_tris triangles
    (both sides together; a query larger than the budget gets a wave alone)."""
    waves: list[Wave] = []
    cur_q, cur_a, cur_b, cur_t = [], [], [], 0
    for i, q in enumerate(qs):
        ia, ib = side_instances(q, 0), side_instances(q, 1)
        t = triangles(ia) + triangles(ib)
        if cur_q and cur_t + t > budget_tris:
            waves.append(_wave(cur_q, cur_a, cur_b, cur_t))
            cur_q, cur_a, cur_b, cur_t = [], [], [], 0
        cur_q.append(i)
        cur_a.append(ia)
        cur_b.append(ib)
        cur_t += t
    if cur_q:
        waves.append(_wave(cur_q, cur_a, cur_b, cur_t))
    return waves


def _wave(qs, parts_a, parts_b, t) -> Wave:
    for g, (pa, pb) in enumerate(zip(parts_a, parts_b)):
        pa["group"] = g
        pb["group"] = g
    cat = lambda p: np.concatenate(p) if p else np.zeros(0, INSTANCE_DTYPE)
    return Wave(list(qs), cat(parts_a), cat(parts_b), t)


def split_pairs(pairs: np.ndarray, wave: Wave) -> dict[int, np.ndarray]:
    """Global (a, b) object ids of a wave's result -> {query: local pairs}."""
    offs_a = np.concatenate([[0], np.cumsum(np.bincount(wave.a["group"], minlength=len(wave.queries)))])
    offs_b = np.concatenate([[0], np.cumsum(np.bincount(wave.b["group"], minlength=len(wave.queries)))])
    qa = wave.a["group"][pairs[:, 0]] if len(pairs) else np.zeros(0, np.int64)
    out = {}
    for g in np.unique(qa):
        sel = pairs[qa == g]
        out[wave.queries[int(g)]] = np.stack([sel[:, 0] - offs_a[g], sel[:, 1] - offs_b[g]], 1)
    return out


def expected_pairs(wave: Wave, per_mesh: float = 0.5) -> int:
    return int(per_mesh * 0.5 * (len(wave.a) + len(wave.b))) + 1


def run_batched(ctx, waves: list[Wave], opts_fn, warmup: int = 1, replays: int = 3, log=None,
                keep_pairs: bool = False) -> dict:
    """Each wave: expand both sides on the device (untimed), capture the
    wave's join as a CUDA graph, replay it `warmup` + `replays` times; the
    wave's time is the mean of the timed replays (CUDA events around the
    graph launch)."""
    from .join import Dataset, JoinGraph, default_tuning
    t = default_tuning(defer_build=1)
    total_ms, pairs_total, expand_s, plan_s = 0.0, 0, 0.0, 0.0
    launches, per_wave, results = 0, [], {}
    for w, wave in enumerate(waves):
        t0 = time.perf_counter()
        A = Dataset.from_instances(ctx, wave.a, t)
        B = Dataset.from_instances(ctx, wave.b, t)
        t1 = time.perf_counter()
        g = JoinGraph(ctx, A, B, opts_fn(wave))
        t2 = time.perf_counter()
        for _ in range(warmup):
            g.launch()
        ms = []
        for _ in range(replays):
            st = g.launch()
            ms.append(st["ms_total"])
        launches = st["launches"]
        wave_ms = float(np.mean(ms))
        total_ms += wave_ms
        expand_s += t1 - t0
        plan_s += t2 - t1
        pairs = g.pairs()
        pairs_total += len(pairs)
        if keep_pairs:
            results.update(split_pairs(pairs, wave))
        per_wave.append({"queries": len(wave.queries), "tris": wave.tris, "ms": wave_ms, "pairs": len(pairs),
                         "launches": launches})
        g.close()
        A.close()
        B.close()
        if log:
            log(f"wave {w + 1}/{len(waves)}: {len(wave.queries)} queries, {wave.tris / 1e6:.0f} M tris, "
                f"{wave_ms:.1f} ms, {len(pairs)} pairs")
    return {"ms": total_ms, "pairs": pairs_total, "expand_s": expand_s, "plan_s": plan_s, "waves": per_wave,
            "results": results}


def run_per_query(ctx, qs: list[Query], opts, build_leaf: int = 0, log=None, keep_pairs: bool = False,
                  subset: list[int] | None = None) -> dict:
    """The same queries one join call each.  Timed: the datasets' own
    hierarchy builds (when `build`) and the join, wall clock (both are
    synchronous calls); the device expansion of the inputs is not timed.
    build_leaf > 0 builds each dataset's own hierarchy with that leaf size
    inside the timed region (the plain form)."""
    from .join import Dataset, default_tuning, run_join
    t = default_tuning(defer_build=1)
    total_s, pairs_total, results = 0.0, 0, {}
    idx = subset if subset is not None else range(len(qs))
    for n, i in enumerate(idx):
        q = qs[i]
        A = Dataset.from_instances(ctx, side_instances(q, 0), t)
        B = Dataset.from_instances(ctx, side_instances(q, 1), t)
        ctx.synchronize()
        t0 = time.perf_counter()
        if build_leaf > 0:
            A.build(default_tuning(leaf_size=build_leaf))
            B.build(default_tuning(leaf_size=build_leaf))
        r = run_join(ctx, A, B, opts)
        total_s += time.perf_counter() - t0
        pairs_total += len(r.pairs)
        if keep_pairs:
            results[i] = r.pairs
        A.close()
        B.close()
        if log and (n % 512 == 0):
            log(f"query {n + 1}/{len(idx)}: {total_s:.2f} s so far")
    return {"s": total_s, "pairs": pairs_total, "results": results}
