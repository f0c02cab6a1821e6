"""Generate the committed golden fixtures (run in the development container,
where the reference sources are present).

* ``ref_*.pre`` / ``ref_digests.json`` — outputs of the reference's own
  `.pre` tool (``oracle/_ref/ref_pre_tool``: the reference's BinaryIO.h and
  EdgePreprocessor.cpp compiled from their sources) for seeded meshes written
  without edges by this repository.  They pin this repository's writer and
  edge extractor byte for byte (header padding bytes 50..55 excluded: the
  reference leaves them uninitialised).
* ``pairs_*.npz`` — oracle pair sets for small joins (overlap, intersection,
  containment, FP32 plain overlap), so the GPU tests also compare against
  stored answers.
* ``pairs_ellipsoids_50000.npz`` (``--full``) — the oracle's intersection and
  containment pair sets of the full benchmark workload, 2 x 50,000 level-3
  ellipsoids (the datasets of ``bench.workload(1.0)``), a few minutes of
  host time.
* ``pairs_tubes_head50.npz`` (``--tubes``) — the oracle's overlap pairs of
  the first 50 tubes of the tube workload (``bench.tube_geometry``) against
  every one of the 100,000 ellipsoids (``bench.ellipsoid_instances``) whose
  box shares a grid cell with one of those tubes' triangle boxes, with
  global ellipsoid ids: the full tube join restricted to tubes 0..49 must
  equal it.
* ``pairs_batched_64.npz`` (``--batched``) — the oracle's overlap pairs of 64
  queries drawn (seed 64) from the 4,096-query batched workload
  (``pierce_gb300.batched.workload(seed=3)``), at their full mesh sizes.

Usage:  python tests/golden/make_golden.py [--full | --tubes | --batched]
"""
from __future__ import annotations

import hashlib
import json
import subprocess
import sys
import tempfile
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
sys.path.insert(0, str(ROOT))

import pierce_gb300 as pg  # noqa: E402
from oracle import pyoracle as O  # noqa: E402

REF_TOOL = ROOT / "oracle" / "_ref" / "ref_pre_tool"

# Datasets whose reference `.pre` output is pinned.  (name, builder)
FORMAT_CASES = {
    "icospheres_l1": lambda: pg.icospheres(7, 20, 1, hi=20.0),
    "icospheres_l3": lambda: pg.icospheres(8, 40, 3, hi=40.0),
    "ellipsoids_l2": lambda: pg.ellipsoid_pair(1, 2, 30, 30, 2, lo=0, hi=30, frac_contact=0.2)[1],
    "tubes": lambda: pg.tubes(3, 2, 3000),
}
STORE_FULL = {"icospheres_l1"}   # small enough to commit the reference file itself

JOIN_CASES = {
    "icospheres": lambda: (pg.icospheres(101, 200, 2, hi=45.0), pg.icospheres(202, 200, 2, hi=45.0)),
    "ellipsoid_contacts": lambda: pg.ellipsoid_pair(5, 6, 150, 150, 2, lo=0, hi=50, frac_contact=0.1),
}


def zero_padding(b: bytes) -> bytes:
    return b[:50] + b"\x00" * 6 + b[56:]


def raw_without_edges(geom) -> "pg.Geometry":
    return pg.Geometry.from_arrays(geom.vertices, geom.indices, geom.tri_to_object)


def full_workload() -> None:
    """Intersection and containment pairs of the benchmark's 2 x 50,000
    ellipsoids, as the oracle computes them."""
    import time
    import bench
    A, B, cfg = bench.workload(1.0)
    t0 = time.perf_counter()
    inter = O.intersection_keys(A, B)
    cont = O.containment_keys(A, B)
    np.savez_compressed(HERE / "pairs_ellipsoids_50000.npz", intersection=inter, containment=cont,
                        seeds=np.array(cfg["seeds"]), meshes_per_side=cfg["meshes_per_side"])
    print("ellipsoids_50000", len(inter), len(cont), f"{time.perf_counter() - t0:.1f} s")


TUBE_HEAD = 50
BATCHED_SEED, BATCHED_QUERIES = 64, 64


def tubes_head() -> None:
    """Overlap pairs of tubes 0..TUBE_HEAD-1 against every ellipsoid."""
    import time
    import bench
    t0 = time.perf_counter()
    As, Bs, near = bench.tube_sample(TUBE_HEAD)
    t1 = time.perf_counter()
    keys, _ = O.overlap_keys(As, Bs)
    glob = bench.sample_keys_global(keys, near)
    np.savez_compressed(HERE / "pairs_tubes_head50.npz", overlap=glob, first=TUBE_HEAD,
                        near=near.astype(np.int32), seeds=np.array([bench.TUBE_SEED, bench.ELLIPSOID_SEED]))
    print(f"tubes head {TUBE_HEAD}: {As.num_triangles} + {Bs.num_triangles} triangles ({len(near)} ellipsoids), "
          f"{len(glob)} pairs, set-up {t1 - t0:.1f} s, oracle {time.perf_counter() - t1:.1f} s")


def batched_queries() -> list[int]:
    return sorted(np.random.default_rng(BATCHED_SEED).choice(4096, BATCHED_QUERIES, replace=False).tolist())


def batched_subset() -> None:
    """Overlap pairs of 64 queries of the batched workload, one join each."""
    import time
    from pierce_gb300 import batched as BT
    qs = BT.workload(seed=3, queries=4096)
    out = {}
    t0 = time.perf_counter()
    for i in batched_queries():
        q = qs[i]
        A = pg.expand_instances(BT.side_instances(q, 0))
        B = pg.expand_instances(BT.side_instances(q, 1))
        keys, _ = O.overlap_keys(A, B)
        out[f"q{i}"] = keys
        print(f"query {i}: {A.num_triangles} + {B.num_triangles} triangles, {len(keys)} pairs, "
              f"{time.perf_counter() - t0:.0f} s", flush=True)
    np.savez_compressed(HERE / "pairs_batched_64.npz", queries=np.array(batched_queries()), **out)


def main() -> None:
    if "--full" in sys.argv[1:]:
        full_workload()
        return
    if "--tubes" in sys.argv[1:]:
        tubes_head()
        return
    if "--batched" in sys.argv[1:]:
        batched_subset()
        return
    if not REF_TOOL.exists():
        raise SystemExit("oracle/_ref/ref_pre_tool missing: run oracle/build_ref.sh first")
    digests = {}
    with tempfile.TemporaryDirectory() as td:
        td = Path(td)
        for name, make in FORMAT_CASES.items():
            raw = raw_without_edges(make())
            raw.write_pre(td / "in.pre")
            subprocess.run([str(REF_TOOL), str(td / "in.pre"), str(td / "out.pre")], check=True,
                           stdout=subprocess.DEVNULL)
            ref = zero_padding((td / "out.pre").read_bytes())
            digests[name] = {"sha256": hashlib.sha256(ref).hexdigest(), "bytes": len(ref),
                             "input_sha256": hashlib.sha256(zero_padding((td / "in.pre").read_bytes())).hexdigest()}
            if name in STORE_FULL:
                (HERE / f"ref_{name}.pre").write_bytes(ref)
    (HERE / "ref_digests.json").write_text(json.dumps(digests, indent=1, sort_keys=True) + "\n")

    for name, make in JOIN_CASES.items():
        A, B = make()
        over, _ = O.overlap_keys(A, B)
        fp32, _ = O.overlap_keys(A, B, mode=1)
        inter = O.intersection_keys(A, B)
        cont = O.containment_keys(A, B)
        np.savez_compressed(HERE / f"pairs_{name}.npz", overlap=over, overlap_fp32=fp32,
                            intersection=inter, containment=cont)
        print(name, len(over), len(fp32), len(inter), len(cont))


if __name__ == "__main__":
    main()
