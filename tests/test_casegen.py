"""The input generator's compressed beds (lbm-dem_gb300/casegen.py): volume
fraction reached, no two spheres and no sphere and wall closer than the
generator's gap, the same packing from the same seed, and the files in the
reference's format (20-column particles.dat with the reader's -0.05 shift,
src/DEM.cpp:88-134)."""
import math
import os

import numpy as np
import pytest
from scipy.spatial import cKDTree

import casegen


def _min_gaps(pk, lo, hi):
    r, x = pk[:, 0], pk[:, 1:]
    p = cKDTree(x).query_pairs(2.0 * r.max() + 0.5, output_type="ndarray")
    pair = np.linalg.norm(x[p[:, 0]] - x[p[:, 1]], axis=1) - r[p[:, 0]] - r[p[:, 1]]
    wall = min(float(np.min(x - r[:, None] - np.asarray(lo))),
               float(np.min(np.asarray(hi) - x - r[:, None])))
    return float(pair.min()), wall


@pytest.mark.parametrize("phi", [0.50, 0.55])
def test_compressed_bed_reaches_fraction_without_overlap(phi):
    rng = np.random.default_rng(7)
    n = 1500
    rs = np.array([4.2] * (n - n // 2) + [3.0] * (n // 2))
    lo, hi = (0.5, 0.5, 0.5), (78.5, 200.0, 78.5)
    pk, H = casegen.compress_pack(rng, lo, hi, rs, phi)
    vol = float(np.sum(4.0 / 3.0 * math.pi * rs ** 3))
    top = float(np.max(pk[:, 2] + pk[:, 0]))
    assert top <= lo[1] + H + 1e-9
    assert vol / (78.0 * 78.0 * (top - 0.5)) >= phi - 1e-9
    pair, wall = _min_gaps(pk, lo, (hi[0], lo[1] + H, hi[2]))
    assert pair > 0.015 and wall >= -1e-12
    # the same seed gives the same packing, bit for bit
    pk2, _ = casegen.compress_pack(np.random.default_rng(7), lo, hi, rs, phi)
    assert np.array_equal(pk, pk2)


def test_bed_taller_than_the_box_is_refused():
    rs = np.full(400, 4.2)
    with pytest.raises(ValueError, match="above the box"):
        casegen.compress_pack(np.random.default_rng(1), (0.5, 0.5, 0.5), (30.5, 30.0, 30.5),
                              rs, 0.5)


def test_c2_workload_bed(tmp_path):
    """The 256x320x256 workload: 25 000 spheres (radii 3.0 / 4.2, half each)
    in a bed of volume fraction 0.50 below the fill height 240, written in
    the reference's format."""
    case = casegen.named_case("c2")
    assert len(case.particles) == 25000
    assert sorted(set(case.particles[:, 0])) == [3.0, 4.2]
    phi = casegen.bed_fraction(case)
    assert phi >= 0.49
    p = case.particles
    assert float(np.max(p[:, 2] + p[:, 0])) < 240.0
    pair, wall = _min_gaps(p[:, :4], (0.5, 0.5, 0.5), (254.5, 240.0, 254.5))
    assert pair > 0.0 and wall >= -1e-12
    cfg = case.write(str(tmp_path / "c2"))
    rows = open(os.path.join(os.path.dirname(cfg), "input", "particles.dat")).read().split("\n")
    assert int(rows[0]) == 25000
    first = rows[1].split()
    assert len(first) == 20
    assert float(first[3]) == pytest.approx(p[0, 1] + 0.05, rel=0, abs=1e-12)
