"""The reference's screen-phase output files (lbdem_output_open /
lbdem_output_close, and the driver with screenExpTime > 0) against the files
the reference's own IO code wrote for the same inputs
(tests/golden/io/<case>/, made by tests/golden/make_io_golden.py).

- CPU: the committed files hold a line exactly at the cycles the
  reference's screen counter picks ((unsigned)(t / screenExpTime) + 1
  advancing, t summed one unitTime per cycle), and their header lines.
- GPU, plain FP64 form through the driver: the same files line for line.
  Header lines and the layout of every line (tabs, number of fields) are
  equal; numbers agree to the printed precision: RTOL_PRINT relative (six
  significant digits on both sides of values that agree to 1e-10), with an
  absolute floor of ATOL_FRAC of the file's largest value for sums that
  cancel to near zero.
- GPU, mixed form through the Python API: the same layout, numbers within
  MIXED_FRAC of each file's largest value.
- The stress files (the DEM stress sums over the DEM volume) and the
  particle recycle files (particleData/partRecycle*.dat, the driver with
  partRecycleExpTime: per-particle total stresslets and displacements) are
  compared the same way; bodyPosition.dat is header-only in both.
"""
import json
import os
import shutil
import subprocess

import numpy as np
import pytest

from conftest import GOLDEN, REPO

DRIVER = os.path.join(REPO, "lbm-dem_gb300", "lbdem_run")
IO = os.path.join(GOLDEN, "io")
STRESS = ("stressTensor.dat", "normalStressCont.dat", "shearStressCont.dat")
FILLED = ("export.dat", "objPosition.dat", "objForce.dat", "wallForce.dat",
          "bodyPosition.dat") + STRESS
RTOL_PRINT = 2e-5
ATOL_FRAC = 1e-9
MIXED_FRAC = 1e-3


def _cases():
    with open(os.path.join(IO, "cases.json")) as fh:
        return json.load(fh)


def _lines(path):
    with open(path) as fh:
        return fh.read().split("\n")


def _num(tok):
    try:
        return float(tok)
    except ValueError:
        return None


def _scale(lines):
    vals = [abs(v) for l in lines for v in map(_num, l.split()) if v is not None]
    return max(vals) if vals else 0.0


def _compare(got_path, ref_path, rtol, atol_frac):
    got, ref = _lines(got_path), _lines(ref_path)
    name = os.path.basename(ref_path)
    assert len(got) == len(ref), (name, len(got), len(ref))
    atol = atol_frac * _scale(ref)
    for n, (lg, lr) in enumerate(zip(got, ref)):
        assert lg.count("\t") == lr.count("\t"), (name, n, lg, lr)
        assert lg.count(" ") == lr.count(" "), (name, n, lg, lr)
        tg, tr = lg.split(), lr.split()
        assert len(tg) == len(tr), (name, n, lg, lr)
        for a, b in zip(tg, tr):
            fa, fb = _num(a), _num(b)
            if fa is None or fb is None:
                assert a == b, (name, n, a, b)
            else:
                assert abs(fa - fb) <= rtol * max(abs(fa), abs(fb)) + atol, (name, n, a, b)


def test_golden_files_follow_the_reference_schedule():
    for name, c in _cases().items():
        steps, screen = c["steps"], c["screenExpTime"]
        want, t, last = [], 0.0, 0
        for s in range(steps + 1):
            if s:
                t += 1.0  # unitTime of the golden cases
            counter = int(t / screen) + 1
            if counter > last:
                last = counter
                want.append(s)
        lines = [l for l in _lines(os.path.join(IO, name, "export.dat")) if l]
        assert [int(l.split(";")[0]) for l in lines] == want, name
        pos = [l for l in _lines(os.path.join(IO, name, "objPosition.dat")) if l]
        assert pos[0].startswith("position(x)") and len(pos) == len(want) + 1
        for f in STRESS + ("bodyPosition.dat",):
            assert _lines(os.path.join(IO, name, f))[0].endswith(" ")


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["tiny_direct", "small_cells", "c1", "bodies"])
def test_driver_writes_the_reference_files(name, lib, tmp_path):
    c = _cases()[name]
    d = tmp_path / name
    shutil.copytree(os.path.join(GOLDEN, name), d)
    r = subprocess.run([DRIVER, "-c", "parameters.cfg", "-steps", str(c["steps"]),
                        "-screenExpTime", repr(c["screenExpTime"]), "-partRecycleExpTime",
                        repr(c["partRecycleExpTime"]), "-d", "out"], cwd=d,
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    for f in FILLED:
        _compare(d / "out" / f, os.path.join(IO, name, f), RTOL_PRINT, ATOL_FRAC)
    want = sorted(os.listdir(os.path.join(IO, name, "particleData")))
    assert sorted(os.listdir(d / "out" / "particleData")) == want
    for f in want:
        _compare(d / "out" / "particleData" / f, os.path.join(IO, name, "particleData", f),
                 RTOL_PRINT, ATOL_FRAC)


@pytest.mark.gpu
def test_mixed_form_output_through_the_api(lib, tmp_path):
    import lbdem
    name = "small_cells"
    c = _cases()[name]
    cfg = lbdem.LoadedConfig(os.path.join(GOLDEN, name, "parameters.cfg"))
    s = lbdem.Solver(cfg, precision=lbdem.MIXED)
    try:
        s.output_open(tmp_path, c["screenExpTime"])
        s.cycle(c["steps"] - 5)  # the lines of these cycles may still be in flight
        s.cycle(5)
        s.output_close()
    finally:
        s.close()
        cfg.close()
    for f in FILLED:
        _compare(tmp_path / f, os.path.join(IO, name, f), 0.0, MIXED_FRAC)
