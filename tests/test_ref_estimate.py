"""The oracle's grid selectivity estimate (oracle/pyoracle.py grid_estimate,
which the GPU's pierce_estimate_pairs is tested against) pinned to the
reference's own estimate: its kernel (pierce/query/src/cuda/
estimated_overlap.cu:8-41), global averages and estimatePairs lambda
(pierce/query/src/applications/pierce_overlap_main.cpp:189-219, 376-471),
compiled from their sources into oracle/_ref/ref_estimate_tool by
oracle/build_ref.sh where the reference is present (skipped elsewhere).

The matched-cell count and the truncated estimate must be equal; the raw
sum is a float reduction whose order differs (the reference reduces on the
device, the oracle exactly): within 1e-6 relative."""
import subprocess
from pathlib import Path

import numpy as np
import pytest

import pierce_gb300 as pg
from oracle import pyoracle as O

ROOT = Path(__file__).resolve().parents[1]
TOOL = ROOT / "oracle" / "_ref" / "ref_estimate_tool"

pytestmark = pytest.mark.skipif(not TOOL.exists(), reason="reference sources not compiled here")

CASES = {
    "icospheres": (lambda: (pg.icospheres(1, 400, 2, hi=50.0), pg.icospheres(2, 300, 2, hi=50.0)), 4.0),
    "ellipsoids": (lambda: pg.ellipsoid_pair(3, 4, 300, 300, 2, lo=0, hi=60), 6.0),
    "tubes_vs_spheres": (lambda: (pg.tubes(3, 3, 20000, hi=50.0), pg.icospheres(5, 200, 2, hi=50.0)), 3.0),
    "disjoint": (lambda: (pg.icospheres(6, 50, 1, hi=10.0), pg.icospheres(7, 50, 1, lo=500.0, hi=510.0)), 2.0),
}


@pytest.mark.parametrize("name", sorted(CASES))
@pytest.mark.parametrize("eps,gamma,alpha", [(0.001, 0.8, True), (0.001, 0.8, False), (0.5, 1.3, True)])
def test_grid_estimate_matches_reference(tmp_path, name, eps, gamma, alpha):
    make, cell = CASES[name]
    A, B = make()
    A.grid_stats(cell)
    B.grid_stats(cell)
    A.write_pre(tmp_path / "a.pre")
    B.write_pre(tmp_path / "b.pre")
    out = subprocess.run([str(TOOL), str(tmp_path / "a.pre"), str(tmp_path / "b.pre"), str(eps), str(gamma),
                          "1" if alpha else "0"], capture_output=True, text=True, check=True).stdout.split()
    raw, est, matched = float(out[0]), int(out[1]), int(out[2])
    o_raw, o_est, o_matched = O.grid_estimate(A.grid_cells, B.grid_cells, cell, eps, gamma, alpha)
    assert matched == o_matched
    assert est == o_est
    assert raw == pytest.approx(o_raw, rel=1e-6, abs=0.0)
    if name == "disjoint":
        assert matched == 0 and est == 0
