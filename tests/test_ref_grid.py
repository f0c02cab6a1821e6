"""Grid statistics (pierce_preprocess --generate-grid) against the
reference's own generateGridStats (pierce/preprocess/src/
pierce_preprocess.cpp:49-167), compiled from its sources into
oracle/_ref/ref_grid_tool by oracle/build_ref.sh where the reference is
present (skipped elsewhere).

The sparse cells' indices, CenterCount and TouchCount must be equal.  The
two float means (AvgSizeMean, VolRatio) are sums over a cell's objects
divided by TouchCount; the reference adds the objects in the iteration
order of its std::unordered_map, this repository in object order, so they
may differ in the last bits: within 5e-7 relative."""
import subprocess
from pathlib import Path

import numpy as np
import pytest

import pierce_gb300 as pg

ROOT = Path(__file__).resolve().parents[1]
TOOL = ROOT / "oracle" / "_ref" / "ref_grid_tool"

pytestmark = pytest.mark.skipif(not TOOL.exists(), reason="reference sources not compiled here")

CASES = {
    "icospheres": lambda: pg.icospheres(7, 300, 3, hi=60.0),
    "ellipsoids": lambda: pg.ellipsoid_pair(1, 2, 200, 200, 2, lo=0, hi=40)[1],
    "tubes": lambda: pg.tubes(3, 3, 20000, hi=50.0),
    "negative_coordinates": lambda: pg.icospheres(9, 80, 2, lo=-30.0, hi=10.0),
}


def _sorted(c):
    return c[np.lexsort((c["iz"], c["iy"], c["ix"]))]


@pytest.mark.parametrize("name", sorted(CASES))
@pytest.mark.parametrize("cell", [2.5, 8.0])
def test_grid_stats_match_reference(tmp_path, name, cell):
    G = CASES[name]()
    G.write_pre(tmp_path / "in.pre")
    subprocess.run([str(TOOL), str(tmp_path / "in.pre"), str(cell), str(tmp_path / "ref.pre")], check=True,
                   capture_output=True)
    ref = _sorted(pg.Geometry.read_pre(tmp_path / "ref.pre").grid_cells)
    H = pg.Geometry.read_pre(tmp_path / "in.pre")
    H.grid_stats(cell)
    ours = _sorted(H.grid_cells)
    assert len(ref) == len(ours) and len(ref) > 10
    for f in ("ix", "iy", "iz", "center_count", "touch_count"):
        assert np.array_equal(ref[f], ours[f]), f
    for f in ("avg_size_mean", "vol_ratio"):
        np.testing.assert_allclose(ours[f], ref[f], rtol=5e-7, atol=0, err_msg=f)
