"""The command-line driver lbdem_run (the reference's main, src/main.cpp,
on top of the C ABI): usage, loud failure without a GPU, and on a GPU an
impactor trajectory equal to the FP64 oracle's."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from conftest import GOLDEN, REPO, gpu_available

DRIVER = os.path.join(REPO, "lbm-dem_gb300", "lbdem_run")


def _case_dir(tmp_path, name):
    d = tmp_path / name
    shutil.copytree(os.path.join(GOLDEN, name), d)
    return d


def _read_impactor(path):
    rows = [l.split() for l in open(path) if not l.startswith("#")]
    return np.array([[float(v) for v in r] for r in rows])


def test_driver_usage(lib):
    r = subprocess.run([DRIVER, "-h"], capture_output=True, text=True)
    assert r.returncode == 0 and "Usage" in r.stdout


@pytest.mark.skipif(gpu_available(), reason="checks the no-device path")
def test_driver_fails_loudly_without_gpu(lib, tmp_path):
    d = _case_dir(tmp_path, "tiny_direct")
    r = subprocess.run([DRIVER, "-c", "parameters.cfg", "-steps", "2"], cwd=d,
                       capture_output=True, text=True)
    assert r.returncode != 0
    assert "no CUDA device" in r.stderr


def test_driver_rejects_unknown_precision(lib, tmp_path):
    d = _case_dir(tmp_path, "tiny_direct")
    r = subprocess.run([DRIVER, "-c", "parameters.cfg", "-precision", "fp16"], cwd=d,
                       capture_output=True, text=True)
    assert r.returncode != 0 and "precision" in r.stderr


@pytest.mark.gpu
def test_driver_trajectory_matches_oracle(lib, oracle_lib, tmp_path):
    """Plain FP64 form, 12 cycles reported every 4: the impactor position and
    velocity written by the driver equal the oracle's within 1e-10 relative."""
    import lbdem
    import oracle_ffi
    d = _case_dir(tmp_path, "tiny_direct")
    r = subprocess.run([DRIVER, "-c", "parameters.cfg", "-steps", "12", "-every", "4",
                        "-d", "out"], cwd=d, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    got = _read_impactor(d / "out" / "impactor.dat")
    assert [int(s) for s in got[:, 0]] == [0, 4, 8, 12]
    cfg = lbdem.LoadedConfig(str(d / "parameters.cfg"))
    orc = oracle_ffi.Oracle(cfg)
    for k, step in enumerate([0, 4, 8, 12]):
        if step:
            orc.cycle(4)
        ref = np.array(orc.object0())  # x0 (3), x1 (3)
        np.testing.assert_allclose(got[k, 3:9], ref, rtol=1e-10, atol=1e-14)
    orc.close()
    cfg.close()


@pytest.mark.gpu
def test_driver_resumes_from_a_snapshot(lib, tmp_path):
    """Plain FP64 form: 5 cycles with -snapshot, then -resume up to cycle 12,
    against one uninterrupted 12-cycle run. The resumed run's impactor lines
    continue the file and agree with the uninterrupted run within 1e-10
    relative (the order of atomic force sums differs between runs)."""
    d = _case_dir(tmp_path, "tiny_direct")
    base = [DRIVER, "-c", "parameters.cfg", "-every", "4"]
    r = subprocess.run(base + ["-steps", "12", "-d", "whole"], cwd=d, capture_output=True,
                       text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run(base + ["-steps", "5", "-d", "split", "-snapshot", "s.lbdemck"], cwd=d,
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert (d / "s.lbdemck").exists()
    r = subprocess.run(base + ["-steps", "12", "-d", "split", "-resume", "s.lbdemck"], cwd=d,
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert "resumed at cycle 5" in r.stdout
    whole = _read_impactor(d / "whole" / "impactor.dat")
    split = _read_impactor(d / "split" / "impactor.dat")
    assert [int(s) for s in whole[:, 0]] == [0, 4, 8, 12]
    assert [int(s) for s in split[:, 0]] == [0, 4, 5, 9, 12]
    np.testing.assert_allclose(split[-1, 1:], whole[-1, 1:], rtol=1e-10, atol=1e-14)
