"""The reference's fluid recycle file: lbdem_export_recycle_fluid (writer,
IO::exportRecycleFluid) and lbRestart / lbRestartFile at lbdem_create
(reader, LB::restartInterface / restartVariables), against files and states
the pinned reference wrote (tests/golden/recycle/, made by
tests/golden/make_recycle_golden.py).

- CPU: lbRestartFile is parsed into the configuration (with -key overrides).
- GPU, plain FP64 form, tiny_direct:
  * after 8 cycles the exported file equals the reference's recycle file of
    cycle 8: the size line and the type line exactly, the same number of
    records, mass, viscosity and the 19 populations of every record within
    RTOL_PRINT relative (six printed digits of values that agree to 1e-10)
    or ATOL_PRINT absolute. The density and velocity columns hold the
    moments of the record's own populations (the reference writes the
    collision's force-shifted values, which a restart does not read):
    checked against the printed populations within ATOL_MOMENTS;
  * a run started from the reference's file holds exactly the file's types
    (type counts equal to the reference's restart) and, at every active
    node in index order, exactly the file's populations and mass;
  * after 6 cycles from that start, particle, impactor and wall state agree
    with the reference's restarted run within RTOL relative of each array's
    largest value (the order of atomic force sums differs), node type
    counts are equal and the total mass agrees within 1e-12.
- GPU, mixed form: the same start (populations within FP32 rounding).
- GPU, driver with fluidRecycleExpTime 8: the recycle files of cycles 0 and
  8 in data/fluidData, the one of cycle 8 equal to the reference's as above.
"""
import gzip
import os
import shutil
import subprocess

import numpy as np
import pytest

from conftest import GOLDEN, REPO

REC = os.path.join(GOLDEN, "recycle")
CASE = "tiny_direct"
RTOL_PRINT, ATOL_PRINT = 2e-5, 1e-9
ATOL_MOMENTS = 2e-6  # 19 populations printed to six digits
RTOL = 1e-10


def _cfg(overrides=None):
    import lbdem
    return lbdem.LoadedConfig(os.path.join(GOLDEN, CASE, "parameters.cfg"), overrides=overrides)


def _reference_file(tmp_path):
    path = tmp_path / "fluidRecycle_step8.dat"
    with gzip.open(os.path.join(REC, f"{CASE}_step8.dat.gz"), "rb") as src:
        path.write_bytes(src.read())
    return path


def _records(path):
    with open(path) as fh:
        lines = fh.read().split("\n")
    return lines[0], lines[1], [l for l in lines[2:] if l]


def test_restart_file_key_is_parsed(lib):
    c = _cfg({"lbRestart": 1, "lbRestartFile": "some/dir/fluidRecycle.dat"})
    try:
        assert c.cfg.lbRestart == 1
        assert c.cfg.lbRestartFile == b"some/dir/fluidRecycle.dat"
    finally:
        c.close()


def _compare_recycle(mine, tmp_path):
    size_m, types_m, recs_m = _records(mine)
    size_r, types_r, recs_r = _records(_reference_file(tmp_path))
    assert size_m == size_r
    assert types_m == types_r
    assert len(recs_m) == len(recs_r)
    a = np.array([[float(v) for v in l.split()] for l in recs_m])
    b = np.array([[float(v) for v in l.split()] for l in recs_r])
    assert a.shape == b.shape == (len(recs_r), 25)
    assert all(l.endswith(" ") for l in recs_m)
    np.testing.assert_allclose(a[:, 4:], b[:, 4:], rtol=RTOL_PRINT, atol=ATOL_PRINT)
    # D3Q19 directions in the reference's order (src/lattice.h)
    cx = np.array([0, 1, -1, 0, 0, 0, 0, 1, -1, -1, 1, 0, 0, 0, 0, 1, -1, 1, -1])
    cy = np.array([0, 0, 0, 1, -1, 0, 0, 1, -1, 1, -1, 1, -1, -1, 1, 0, 0, 0, 0])
    cz = np.array([0, 0, 0, 0, 0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 1, -1, -1, 1])
    f = a[:, 6:]
    n = f.sum(axis=1)
    np.testing.assert_allclose(a[:, 0], n - 1.0, rtol=0, atol=ATOL_MOMENTS)
    for col, c in ((1, cx), (2, cy), (3, cz)):
        np.testing.assert_allclose(a[:, col], (f * c).sum(axis=1) / n, rtol=0, atol=ATOL_MOMENTS)


@pytest.mark.gpu
def test_export_matches_the_reference_recycle_file(lib, tmp_path):
    import lbdem
    cfg = _cfg()
    s = lbdem.Solver(cfg, precision=lbdem.PLAIN_FP64)
    try:
        s.cycle(8)
        s.export_recycle_fluid(tmp_path / "mine.dat")
    finally:
        s.close()
        cfg.close()
    _compare_recycle(tmp_path / "mine.dat", tmp_path)


@pytest.mark.gpu
def test_driver_writes_recycle_files_at_the_reference_cycles(lib, tmp_path):
    d = tmp_path / CASE
    shutil.copytree(os.path.join(GOLDEN, CASE), d)
    driver = os.path.join(REPO, "lbm-dem_gb300", "lbdem_run")
    r = subprocess.run([driver, "-c", "parameters.cfg", "-steps", "8", "-fluidRecycleExpTime",
                        "8", "-d", "out"], cwd=d, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    names = sorted(os.listdir(d / "out" / "fluidData"))
    assert names == ["fluidRecycle0000000000.dat", "fluidRecycle0000000008.dat"]
    _compare_recycle(d / "out" / "fluidData" / "fluidRecycle0000000008.dat", tmp_path)


@pytest.mark.gpu
@pytest.mark.parametrize("form", ["fp64", "mixed"])
def test_restart_holds_the_file_state(form, lib, tmp_path):
    import lbdem
    path = _reference_file(tmp_path)
    cfg = _cfg({"lbRestart": 1, "lbRestartFile": str(path)})
    s = lbdem.Solver(cfg, precision=lbdem.PLAIN_FP64 if form == "fp64" else lbdem.MIXED)
    try:
        g = s.lattice()
    finally:
        s.close()
        cfg.close()
    ref = np.load(os.path.join(REC, f"{CASE}_restart.npz"))
    np.testing.assert_array_equal(np.bincount(g["type"], minlength=13), ref["s0/type_counts"])
    _, types_r, recs = _records(path)
    ftypes = np.array([int(v) for v in types_r.split()])
    fluid_now = (g["type"] == ftypes)
    assert fluid_now.mean() > 0.9  # walls and impactor keep their geometry types
    vals = np.array([[float(v) for v in l.split()] for l in recs])
    act = np.flatnonzero((g["type"] == 0) | (g["type"] == 3))
    assert len(act) == len(vals)
    tol = 0.0 if form == "fp64" else 1e-7
    np.testing.assert_allclose(g["f"][:, act].T, vals[:, 6:], rtol=0, atol=tol)
    np.testing.assert_allclose(g["mass"][act], vals[:, 4] + 1.0, rtol=0, atol=tol)


@pytest.mark.gpu
def test_restarted_run_matches_the_reference_restart(lib, tmp_path):
    import lbdem
    path = _reference_file(tmp_path)
    cfg = _cfg({"lbRestart": 1, "lbRestartFile": str(path)})
    s = lbdem.Solver(cfg, precision=lbdem.PLAIN_FP64)
    ref = np.load(os.path.join(REC, f"{CASE}_restart.npz"))
    try:
        for step in range(1, 7):
            s.cycle(1)
            st = s.state()
            np.testing.assert_array_equal(np.bincount(st["type"], minlength=13),
                                          ref[f"s{step}/type_counts"], err_msg=f"step {step}")
            assert st["mass"].sum() == pytest.approx(float(ref[f"s{step}/mass_sum"][0]),
                                                     rel=1e-12)
            for key in ("p_x0", "p_x1", "p_w1", "p_FHydro", "p_FContact", "p_FLub", "p_FTotal",
                        "o_x0", "o_x1", "o_FHydro", "o_FTotal", "w_FHydro", "w_FTotal"):
                want = ref[f"s{step}/{key}"].reshape(st[key].shape)
                scale = max(float(np.max(np.abs(want))), 1e-300)
                np.testing.assert_allclose(st[key], want, rtol=0, atol=RTOL * scale,
                                           err_msg=f"{key} step {step}")
    finally:
        s.close()
        cfg.close()
