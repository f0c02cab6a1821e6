"""bench.py on the CPU: multi-rank aggregation with world_size 2 over gloo,
and the reference arm's JSON line."""
import os
import socket
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, out):
    sys.path.insert(0, str(ROOT))
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    v = bench.max_over_ranks(10.0 + 5.0 * rank, dist)
    dist.barrier()
    out.put((rank, v))
    dist.destroy_process_group()


def test_max_over_ranks_gloo_world2():
    torch = pytest.importorskip("torch")
    mp = torch.multiprocessing.get_context("spawn")
    q = mp.Queue()
    port = _free_port()
    procs = [mp.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = dict(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert got == {0: 15.0, 1: 15.0}


def test_max_over_ranks_single_process():
    sys.path.insert(0, str(ROOT))
    import bench
    assert bench.max_over_ranks(3.5, None) == 3.5


@pytest.mark.parametrize("workload", ["tubes", "ellipsoids"])
def test_reference_arm_json_line(workload):
    """bench.py --impl reference (the oracle port on the host cores, no GPU)
    prints one JSON line of the bench contract on a small workload, with the
    config our arm prints for the same workload."""
    import json
    import subprocess
    import bench
    root = ROOT
    p = subprocess.run([sys.executable, str(root / "bench.py"), "--impl", "reference", "--workload", workload,
                        "--scale", "0.02", "--steps", "1", "--warmup", "0", "--cpu-sample-objects", "200",
                        "--cpu-sample-tubes", "2"],
                       capture_output=True, text=True, cwd=root, timeout=600)
    assert p.returncode == 0, p.stderr
    lines = [ln for ln in p.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["value"] > 0 and d["unit"] == "join queries/s"
    assert d["higher_is_better"] is True and d["n_gpus"] == 1 and d["steps"] == 1
    assert d["cpu_baseline"]["kind"] == "port" and d["cpu_baseline"]["cores"] >= 1
    assert d["cpu_baseline"]["value"] == d["value"]
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    if workload == "tubes":
        assert d["config"] == bench.tubes_config(0.02)
        assert d["sample_fraction"] == pytest.approx(2 / 40)
    else:
        assert d["config"] == bench.workload(0.02)[2]
        assert d["config"]["meshes_per_side"] == 1000


def test_boxes_near_is_a_superset_of_box_overlap():
    """The sample selection keeps every object whose box meets a triangle box."""
    import bench
    rng = np.random.default_rng(3)
    tri_lo = rng.uniform(0, 100, (400, 3)).astype(np.float32)
    tri_hi = tri_lo + rng.uniform(0, 5, (400, 3)).astype(np.float32)
    obj_lo = rng.uniform(0, 100, (3000, 3)).astype(np.float32)
    obj_hi = obj_lo + rng.uniform(0, 12, (3000, 3)).astype(np.float32)
    meets = np.any(np.all((obj_lo[:, None, :] <= tri_hi[None]) & (tri_lo[None] <= obj_hi[:, None, :]), axis=2), axis=1)
    near = bench.boxes_near(tri_lo, tri_hi, obj_lo, obj_hi, cell=8.0)
    assert np.all(near[meets]) and meets.sum() > 50 and near.sum() < len(near)


def test_preprocess_workload_json_line():
    """bench.py --workload preprocess (host code only) prints its JSON line;
    where the reference's extractor was built, the output files are
    byte-identical to its own (header padding excluded)."""
    import json
    import subprocess
    p = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--workload", "preprocess", "--scale", "0.05",
                        "--steps", "1", "--warmup", "0"], capture_output=True, text=True, cwd=ROOT, timeout=600)
    assert p.returncode == 0, p.stderr
    d = json.loads([ln for ln in p.stdout.splitlines() if ln.startswith("{")][-1])
    assert d["unit"] == "triangles/s" and d["value"] > 0 and d["value_one_thread"] > 0
    assert d["config"]["triangles"] == 100 * 1280
    if d["reference"] is not None:
        assert d["byte_identical_to_reference"] is True


def test_roofline_algorithmic_bytes():
    """bench.py's algorithmic bytes of the edge-ray launches: 28 B per traced
    edge, 8 B per raw hit, and per target hierarchy 16 B per kept triangle,
    12 B per vertex in proportion to the triangles kept and 32 B per node of
    a minimal binary tree."""
    import types
    import numpy as np
    import bench
    G = types.SimpleNamespace(vertices=np.zeros((600, 3), np.float32), num_triangles=1000)
    got = bench.traced_edge_ray_bytes(10, 2, [(G, 500), (G, 0)])
    assert got == 28 * 10 + 8 * 2 + 16 * 500 + 12 * 300 + 32 * 999
    assert bench.traffic_estimate(100, "tubes") == pytest.approx(bench.EDGE_RAY_DRAM_BYTES_PER_RAY["tubes"] * 100)
