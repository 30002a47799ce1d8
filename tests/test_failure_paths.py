"""Failure paths of the C ABI: each fault becomes an error status that the host
reads, and the context stays destroyable (the GPU stays usable).

None of these tests faults, traps or hangs the GPU:
- non-finite state: a NaN initial fluid velocity (set in the configuration
  structure) makes the populations NaN in the first lattice step; the
  NaN/Inf guard (check_every = 1) reports LBDEM_ERR_NONFINITE at lbdem_sync.
  Particle positions stay finite within that cycle, so no index is ever
  computed from a NaN.
- neighbour-list overflow: sixty small spheres packed around one large
  sphere give it more than 49 neighbours; the list build clamps the list at
  49 entries and reports LBDEM_ERR_OVERFLOW (at lbdem_create, or at
  lbdem_sync with asynchronous initialisation), in the direct-sum and in the
  cell-list branch.
- copy-pipeline timeout: with LBDEM_DEBUG_NO_LATTICE_COPIES the mixed
  lattice step issues none of its bulk copies, so its bounded waits give up
  (after a short limit, with nothing in flight) and the step reports
  LBDEM_ERR_DEVICE_STATE.
"""
import math
import os

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu


def _forms():
    import lbdem
    return [("fp64", lbdem.PLAIN_FP64), ("mixed", lbdem.MIXED)]


@pytest.mark.parametrize("form", ["fp64", "mixed"])
def test_nonfinite_state_is_reported(form, lib):
    import lbdem
    prec = dict(_forms())[form]
    cfg = lbdem.LoadedConfig(os.path.join(GOLDEN, "tiny_direct", "parameters.cfg"))
    cfg.cfg.initVelocity[0] = float("nan")
    s = lbdem.Solver(cfg, precision=prec, check_every=1)
    try:
        s.cycle(1)
        with pytest.raises(RuntimeError, match="non-finite"):
            s.sync()
        # the readback without allocation still returns the state at the fault
        f, _ = s.nodes_noalloc(int(s.info.nodes) // 2, 64)
        assert np.isnan(f).any()
    finally:
        s.close()
        cfg.close()


def _crowded_case(tmp_path, cells: bool):
    """One sphere of radius 4.2 (the last index) with sixty spheres of radius
    0.5 on a shell of radius 5.6 around it: every small sphere is within the
    neighbour cut-off r1 + r2 + 2 of the large one (src/DEM.cpp:473-652)."""
    import casegen
    nx, ny, nz = (40, 44, 40) if cells else (24, 28, 24)
    fill = 36.0 if cells else 20.0
    c = np.array([0.5 * (nx - 1), 10.0, 0.5 * (nz - 1)])
    n = 60
    k = np.arange(n) + 0.5
    phi = np.arccos(1.0 - 2.0 * k / n)
    th = math.pi * (1.0 + 5.0 ** 0.5) * k
    shell = c + 5.6 * np.stack([np.cos(th) * np.sin(phi), np.cos(phi),
                                np.sin(th) * np.sin(phi)], axis=1)
    d = np.linalg.norm(shell[:, None] - shell[None], axis=-1)
    assert d[~np.eye(n, dtype=bool)].min() > 1.05  # no two small spheres overlap
    parts = np.zeros((n + 1, 10))
    parts[:n, 0] = 0.5
    parts[:n, 1:4] = shell
    parts[n, 0] = 4.2
    parts[n, 1:4] = c
    case = casegen.impact_case((nx, ny, nz), fill, 0, (3.0, 4.2), 1.5, fill + 3.0, -0.01, 5.0,
                               0.8, 1.0e-5, 1, name="crowded")
    case.particles = parts
    return case.write(str(tmp_path / ("cells" if cells else "direct")))


@pytest.mark.parametrize("cells", [False, True], ids=["direct", "cells"])
def test_neighbour_overflow_is_reported(cells, lib, tmp_path):
    import lbdem
    path = _crowded_case(tmp_path, cells)
    cfg = lbdem.LoadedConfig(path)
    with pytest.raises(RuntimeError, match="list overflow"):
        lbdem.Solver(cfg, precision=lbdem.PLAIN_FP64)
    # asynchronous initialisation: the same fault at the first lbdem_sync,
    # and the context is still destroyable
    s = lbdem.Solver(cfg, precision=lbdem.MIXED, async_init=True)
    try:
        with pytest.raises(RuntimeError, match="neighbour-list-overflow"):
            s.sync()
    finally:
        s.close()
    cfg.close()


def test_pipeline_timeout_is_reported(lib):
    import lbdem
    cfg = lbdem.LoadedConfig(os.path.join(GOLDEN, "tiny_direct", "parameters.cfg"))
    s = lbdem.Solver(cfg, precision=lbdem.MIXED, debug_flags=lbdem.DEBUG_NO_LATTICE_COPIES)
    try:
        s.cycle(1)
        with pytest.raises(RuntimeError, match="lattice-copy-pipeline-timeout") as e:
            s.sync()
        assert "device-side error" in str(e.value)
    finally:
        s.close()
    # the GPU is still usable: a normal run of the same case steps cleanly
    s = lbdem.Solver(cfg, precision=lbdem.MIXED)
    s.cycle(3)
    s.sync()
    s.close()
    cfg.close()
