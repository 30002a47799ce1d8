"""lbdem_checkpoint / lbdem_restore through the C ABI.

A run is snapshotted after some cycles and the snapshot is loaded into a
second run created from the same configuration.

- Right after the restore the two runs' downloaded states are equal: no
  tolerance, the snapshot copies every byte of the device state.
- Both runs then advance the same number of cycles. Integer state (node
  types, particle flags and indices, neighbour lists, step counters) stays
  equal; floating-point state agrees within what two uninterrupted runs of
  one configuration differ by, since the order of the atomic floating-point
  sums (particle, wall and impactor forces, the extra mass) differs from
  launch to launch: RTOL_FP64 relative per element in the plain FP64 form;
  in the mixed form NORM_MIXED of each field's largest magnitude, because
  its per-step force and torque sums are FP32 sums of terms that largely
  cancel, whose order noise is about 1e-4 of their value.
- Snapshots of another configuration or form, and truncated files, are
  refused before the run's state is touched.

An odd number of cycles before the snapshot leaves the run on its second
lattice buffer, so the restore of the buffer parity is exercised.
"""
import os

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu

RTOL_FP64, ATOL_FP64 = 1e-10, 1e-14
NORM_MIXED = 1e-4
INTEGER_KEYS = ("type", "pflag", "solid", "p_list", "step", "demTimeStep")


def _cfg(name):
    import lbdem
    return lbdem.LoadedConfig(os.path.join(GOLDEN, name, "parameters.cfg"))


def _prec(form):
    import lbdem
    return lbdem.PLAIN_FP64 if form == "fp64" else lbdem.MIXED


def _assert_same(a, b, rtol=0.0, atol=0.0, norm=0.0):
    assert a.keys() == b.keys()
    for k in a:
        if k in INTEGER_KEYS or (rtol == 0.0 and atol == 0.0 and norm == 0.0):
            np.testing.assert_array_equal(a[k], b[k], err_msg=k)
        elif norm:
            scale = float(np.max(np.abs(a[k]))) if a[k].size else 0.0
            np.testing.assert_allclose(a[k], b[k], rtol=0.0, atol=norm * scale, err_msg=k)
        else:
            np.testing.assert_allclose(a[k], b[k], rtol=rtol, atol=atol, err_msg=k)


@pytest.mark.parametrize("form", ["fp64", "mixed"])
def test_restored_run_continues_the_snapshotted_one(form, tmp_path, lib):
    import lbdem
    cfg = _cfg("small_cells")
    a = lbdem.Solver(cfg, precision=_prec(form))
    b = lbdem.Solver(cfg, precision=_prec(form))
    try:
        path = tmp_path / "run.lbdemck"
        a.cycle(7)
        a.checkpoint(path)
        assert os.path.getsize(path) >= a.get_info().device_bytes
        b.restore(path)
        sa, sb = a.state(), b.state()
        assert int(sa["step"][0]) == 7
        _assert_same(sa, sb)
        # a device sum whose atomic order differs from call to call
        assert a.mass_total() == pytest.approx(b.mass_total(), rel=1e-13)
        # the state is live: the next cycles move it
        a.cycle(6)
        b.cycle(6)
        ta, tb = a.state(), b.state()
        assert not np.array_equal(ta["f"], sa["f"])
        if form == "fp64":
            _assert_same(ta, tb, RTOL_FP64, ATOL_FP64)
        else:
            _assert_same(ta, tb, norm=NORM_MIXED)
        assert int(tb["step"][0]) == 13
    finally:
        a.close()
        b.close()
        cfg.close()


def test_snapshot_of_another_run_or_a_truncated_file_is_refused(tmp_path, lib):
    import lbdem
    small, tiny = _cfg("small_cells"), _cfg("tiny_direct")
    a = lbdem.Solver(small, precision=lbdem.MIXED)
    other_form = lbdem.Solver(small, precision=lbdem.PLAIN_FP64)
    other_cfg = lbdem.Solver(tiny, precision=lbdem.MIXED)
    try:
        path = tmp_path / "run.lbdemck"
        a.cycle(2)
        a.checkpoint(path)
        before = other_form.state()
        with pytest.raises(RuntimeError, match="precision"):
            other_form.restore(path)
        _assert_same(before, other_form.state())
        with pytest.raises(RuntimeError, match="differs"):
            other_cfg.restore(path)
        cut = tmp_path / "cut.lbdemck"
        data = path.read_bytes()
        cut.write_bytes(data[: len(data) - 4096])
        target = lbdem.Solver(small, precision=lbdem.MIXED)
        try:
            before = target.state()
            with pytest.raises(RuntimeError, match="wrong length"):
                target.restore(cut)
            _assert_same(before, target.state())
            # the intact snapshot still loads into it
            target.restore(path)
            _assert_same(a.state(), target.state())
        finally:
            target.close()
        bad = tmp_path / "bad.lbdemck"
        bad.write_bytes(b"not a snapshot" * 8)
        with pytest.raises(RuntimeError, match="not a snapshot"):
            a.restore(bad)
        with pytest.raises(RuntimeError, match="cannot open"):
            a.restore(tmp_path / "missing.lbdemck")
    finally:
        a.close()
        other_form.close()
        other_cfg.close()
        small.close()
        tiny.close()


def test_output_continues_from_the_restored_cycle(tmp_path, lib):
    """Output open on the target run: after a restore to cycle 5 its lines
    continue with the reference's output cycles after 5 (screenExpTime 3.5:
    7 and 11), numbered by the restored cycle count."""
    import lbdem
    cfg = _cfg("tiny_direct")
    a = lbdem.Solver(cfg, precision=lbdem.PLAIN_FP64)
    b = lbdem.Solver(cfg, precision=lbdem.PLAIN_FP64)
    try:
        a.cycle(5)
        a.checkpoint(tmp_path / "run.lbdemck")
        out = tmp_path / "out"
        out.mkdir()
        b.output_open(out, 3.5)  # writes the line of cycle 0
        b.restore(tmp_path / "run.lbdemck")
        b.cycle(7)
        b.output_close()
        steps = [int(l.split(";")[0]) for l in (out / "export.dat").read_text().splitlines()]
        assert steps == [0, 7, 11]
    finally:
        a.close()
        b.close()
        cfg.close()
