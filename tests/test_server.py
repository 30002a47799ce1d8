"""The run server (lbdem_server_*): many impact runs resident on one GPU.

Each run's result must be the same alone and in the mix, whether the runs
in the mix share launches (the batch: one launch per kernel for all runs in
their steady cycle) or advance on their own streams:
- plain FP64 form: the impactor state to 1e-10 relative, the tolerance of
  the FP64 parity tests;
- mixed form: the impactor displacement to 1e-3 relative, the mixed form's
  stated tolerance.
Admission follows the memory budget.
"""
import os

import numpy as np
import pytest

from conftest import GOLDEN

CASES = ["small_cells", "tiny_direct", "small_dup"]
CYCLES = 20


def _cfg(name):
    import lbdem
    return lbdem.LoadedConfig(os.path.join(GOLDEN, name, "parameters.cfg"))


def test_estimate_scales_with_lattice_and_form(lib):
    import lbdem
    small = _cfg("tiny_direct")
    big = _cfg("c1")
    for prec in (lbdem.MIXED, lbdem.PLAIN_FP64):
        assert lbdem.estimate_device_bytes(big, prec) > lbdem.estimate_device_bytes(small, prec)
    # the plain form keeps FP64 populations: more bytes per node
    assert lbdem.estimate_device_bytes(big, lbdem.PLAIN_FP64) > \
        lbdem.estimate_device_bytes(big, lbdem.MIXED)
    small.close()
    big.close()


def _solo(name, precision):
    import lbdem
    cfg = _cfg(name)
    s = lbdem.Solver(cfg, precision=precision)
    x0 = np.array(s.objects()["o_x0"][0])
    s.cycle(CYCLES)
    o = s.objects()
    out = x0, np.array(o["o_x0"][0]), np.array(o["o_x1"][0])
    s.close()
    cfg.close()
    return out


@pytest.mark.gpu
@pytest.mark.parametrize("solo", [False, True], ids=["batched", "solo"])
@pytest.mark.parametrize("prec_name", ["fp64", "mixed"])
def test_runs_in_the_mix_equal_runs_alone(prec_name, solo, lib):
    import lbdem
    prec = lbdem.PLAIN_FP64 if prec_name == "fp64" else lbdem.MIXED
    srv = lbdem.Server(precision=prec, max_active=len(CASES), slice_cycles=7,
                       batch_runs=0 if solo else 2)
    cfgs = [_cfg(n) for n in CASES]
    ids = {srv.submit(c, CYCLES): n for c, n in zip(cfgs, CASES)}
    res = srv.drain()
    srv.close()
    for c in cfgs:
        c.close()
    assert len(res) == len(CASES)
    # the runs overlapped: every run started before the first one ended
    first_end = min(r["end_time"] for r in res)
    assert all(r["start_time"] < first_end for r in res)
    for r in res:
        name = ids[r["job_id"]]
        assert r["status"] == 0 and r["cycles"] == CYCLES, name
        # shared launches carried most of the cycles of the runs that reach
        # their steady cycle (small_dup spends these cycles in its initial
        # DEM-only phase, which runs on its own stream)
        if solo:
            assert r["batched_cycles"] == 0, name
        elif name != "small_dup":
            assert r["batched_cycles"] >= CYCLES // 2, (name, r["batched_cycles"])
        y0, x0, x1 = _solo(name, prec)
        got0, got1 = np.array(r["impactor_x0"]), np.array(r["impactor_x1"])
        if prec == lbdem.PLAIN_FP64:
            np.testing.assert_allclose(got0, x0, rtol=1e-10, atol=0)
            np.testing.assert_allclose(got1, x1, rtol=1e-10, atol=1e-300)
        else:
            disp, ref = got0 - y0, x0 - y0
            err = np.max(np.abs(disp - ref)) / max(np.max(np.abs(ref)), 1e-12)
            assert err <= 1e-3, f"{name}: impactor displacement rel err {err:.2e}"


@pytest.mark.gpu
def test_budget_admits_one_run_at_a_time(lib):
    import lbdem
    # three runs of one size and a budget that holds one of them, not two
    cfgs = [_cfg("small_cells") for _ in range(3)]
    need = lbdem.estimate_device_bytes(cfgs[0], lbdem.MIXED)
    srv = lbdem.Server(precision=lbdem.MIXED, max_active=8, slice_cycles=5,
                       device_budget_bytes=int(need * 1.5))
    for c in cfgs:
        srv.submit(c, 10)
    res = sorted(srv.drain(), key=lambda r: r["job_id"])
    srv.close()
    for c in cfgs:
        c.close()
    assert [r["status"] for r in res] == [0, 0, 0]
    # with room for one run, each starts after the previous one ended
    for a, b in zip(res, res[1:]):
        assert b["start_time"] >= a["end_time"]


@pytest.mark.gpu
def test_estimate_bounds_the_allocation(lib):
    import lbdem
    for name in ("tiny_direct", "c1"):
        cfg = _cfg(name)
        for prec in (lbdem.MIXED, lbdem.PLAIN_FP64):
            est = lbdem.estimate_device_bytes(cfg, prec)
            s = lbdem.Solver(cfg, precision=prec)
            got = int(s.get_info().device_bytes)
            s.close()
            assert got <= est <= got + 64 * 1024, (name, prec, got, est)
        cfg.close()


@pytest.mark.gpu
def test_tuner_picks_a_candidate_schedule(lib):
    import lbdem
    cfgs = [_cfg(n) for n in ("small_cells", "tiny_direct")]
    b, c, t = lbdem.tune_server(cfgs, cycles=4, precision=lbdem.MIXED, slice_cycles=2)
    for cf in cfgs:
        cf.close()
    assert b in (0, 2, 4, 8) and c in (8, 32) and t > 0.0


def _diverging_case(tmp_path):
    """A run that diverges within 200 cycles: relaxation time 0.501 and an
    initial fluid velocity of 0.2 across a 24x32x24 box (the oracle's
    populations turn non-finite at cycle 156, its spheres leave the domain
    at cycle 192)."""
    import casegen
    import lbdem
    c = casegen.impact_case((24, 32, 24), 20.0, 6, (3.0, 3.4), 4.0, 26.0, -0.05, 5.0, 0.501,
                            1.0e-4, 1, overrides={"objWaitTime": "2", "initVelocityX": "0.2"},
                            name="diverge")
    return lbdem.LoadedConfig(c.write(str(tmp_path / "diverge")))


@pytest.mark.gpu
@pytest.mark.parametrize("solo", [False, True], ids=["batched", "solo"])
@pytest.mark.parametrize("prec_name", ["fp64"])
def test_diverged_run_ends_at_its_slice(prec_name, solo, lib, tmp_path):
    """A run that diverges ends at the slice whose read-back shows it, with a
    non-finite (or out-of-domain) status and a message; the runs beside it
    finish with the results they have alone.

    The plain form only: its trajectory is the reference's arithmetic and
    the same in every run, so the run diverges at the same cycle every time.
    The mixed form's trajectory of this unstable run changes from run to run
    (FP32 atomic sums in another order), and with it whether and when it
    turns non-finite; the check after each slice is the same code for both
    forms."""
    import lbdem
    prec = lbdem.PLAIN_FP64 if prec_name == "fp64" else lbdem.MIXED
    bad_cfg = _diverging_case(tmp_path)
    good_cfg = _cfg("small_cells")
    srv = lbdem.Server(precision=prec, max_active=2, slice_cycles=8,
                       batch_runs=0 if solo else 2)
    bad_id = srv.submit(bad_cfg, 400)
    good_id = srv.submit(good_cfg, CYCLES)
    res = {r["job_id"]: r for r in srv.drain()}
    err = srv.last_error()
    srv.close()
    bad, good = res[bad_id], res[good_id]
    assert bad["status"] in (lbdem.ERR_NONFINITE, lbdem.ERR_DEVICE_STATE), bad
    assert bad["cycles"] < 260, bad["cycles"]
    assert "after a slice" in err and "failed in a" in err, err
    if not solo:
        assert bad["batched_cycles"] > 0
    assert good["status"] == 0 and good["cycles"] == CYCLES
    y0, x0, x1 = _solo("small_cells", prec)
    got0 = np.array(good["impactor_x0"])
    if prec == lbdem.PLAIN_FP64:
        np.testing.assert_allclose(got0, x0, rtol=1e-10, atol=0)
    else:
        disp, ref = got0 - y0, x0 - y0
        assert np.max(np.abs(disp - ref)) <= 1e-3 * max(np.max(np.abs(ref)), 1e-12)
    bad_cfg.close()
    good_cfg.close()
