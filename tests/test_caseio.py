"""The pure-Python case reader (tests/caseio.py, used by the CPU baseline and
the reference arm of the bench) and the library's reader (csrc/config.cpp,
lbdem_config_load) fill identical lbdem_config structures from the same
files, for every committed case and with command-line overrides."""
import ctypes as C
import glob
import os

import pytest

from conftest import GOLDEN

import caseio


def _same(a, b):
    """Field-by-field equality of two lbdem_config structures, tables included."""
    import lbdem_types
    diffs = []
    for name, ctype in lbdem_types.Config._fields_:
        va, vb = getattr(a, name), getattr(b, name)
        if name in ("particles", "objects", "bodies"):
            n = {"particles": a.n_particles, "objects": a.n_objects, "bodies": a.n_bodies}[name]
            rt = {"particles": lbdem_types.ParticleIn, "objects": lbdem_types.ObjectIn,
                  "bodies": lbdem_types.BodyIn}[name]
            sz = C.sizeof(rt) * n
            if n and C.string_at(va, sz) != C.string_at(vb, sz):
                diffs.append(name)
        elif name == "lbRestartFile":
            if (va or b"") != (vb or b""):
                diffs.append(name)
        elif hasattr(va, "_length_"):
            if list(va) != list(vb):
                diffs.append(name)
        elif va != vb:
            diffs.append(name)
    return diffs


CASES = sorted(os.path.dirname(p) for p in glob.glob(os.path.join(GOLDEN, "*", "parameters.cfg")))


@pytest.mark.parametrize("case", CASES, ids=[os.path.basename(c) for c in CASES])
def test_python_reader_matches_library_reader(lib, case):
    import lbdem
    ref = lbdem.LoadedConfig(os.path.join(case, "parameters.cfg"))
    ours = caseio.CaseConfig(os.path.join(case, "parameters.cfg"))
    assert _same(ref.cfg, ours.cfg) == []
    ref.close()


def test_python_reader_overrides(lib):
    import lbdem
    case = os.path.join(GOLDEN, "small_cells", "parameters.cfg")
    ov = {"demInitialRepeat": "7.5", "objWaitTime": "11", "lbRestart": "TRUE",
          "boundary3": "8", "unitLength": "0.25"}
    ref = lbdem.LoadedConfig(case, overrides=ov)
    ours = caseio.CaseConfig(case, overrides=ov)
    assert ours.cfg.objWaitTime == 11 and ours.cfg.lbRestart == 1
    assert _same(ref.cfg, ours.cfg) == []
    ref.close()


def test_getpot_value_rules(tmp_path):
    """Integer keys take the leading integer, failed conversions keep the
    default, quoted strings keep their spaces, the last definition wins."""
    (tmp_path / "input").mkdir()
    (tmp_path / "input" / "particles.dat").write_text("0\n")
    (tmp_path / "input" / "objects.dat").write_text("0\n")
    (tmp_path / "input" / "body.dat").write_text("0\n")
    (tmp_path / "p.cfg").write_text(
        "objWaitTime = 12.7 # comment\nintervalTime = abc\nlbRestartFile = \" a b \"\n"
        "unitLength = 0.5\nunitLength = 0.25\nlbSizeX = 1e1\n")
    c = caseio.CaseConfig(str(tmp_path / "p.cfg")).cfg
    assert c.objWaitTime == 12 and c.intervalTime == 0
    assert c.lbRestartFile == b" a b "
    assert c.unitLength == 0.25 and c.lbSizeX == 10.0
    assert c.unitTime == 1.0 and list(c.boundary) == [1] * 6
