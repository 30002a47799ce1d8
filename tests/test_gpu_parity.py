"""Plain FP64 GPU path against the oracle, step by step (CUDA path via the C ABI).

Tolerance: 1e-10 relative for every floating-point field, both against the
field's scale and element by element (tests/parity.py), identical node
types, particle flags, solid indices and neighbour lists, at every step of
the 60-step golden cases, over the 100-step config-1 horizon, and on the
reference's own example input in physical units. The oracle is pinned bit
for bit to the compiled reference on every one of these cases
(tests/test_oracle_golden.py).
"""
import os
import tempfile

import numpy as np
import pytest

from conftest import GOLDEN
from parity import compare

RTOL = 1e-10

pytestmark = pytest.mark.gpu


def _pair(name):
    import lbdem
    import oracle_ffi
    cfg = lbdem.LoadedConfig(os.path.join(GOLDEN, name, "parameters.cfg"))
    return cfg, lbdem.Solver(cfg, precision=lbdem.PLAIN_FP64), oracle_ffi.Oracle(cfg)


@pytest.mark.parametrize("name", ["tiny_direct", "small_cells", "small_dup", "units_dyn",
                                  "rheo_bingham", "rheo_frictional", "rheo_voellmy",
                                  "rheo_turbulent", "bodies", "bodies_lj", "slip_stat",
                                  "slip_dyn", "uncover_mid", "uncover_wide"])
def test_fp64_matches_oracle_every_step(name, lib, oracle_lib):
    cfg, gpu, orc = _pair(name)
    steps = 40 if name.startswith("uncover") else 60
    with tempfile.TemporaryDirectory() as tmp:
        bad = compare(gpu.state(), orc.state(tmp), RTOL)
        assert not bad, f"{name} after init: {bad}"
        for s in range(1, steps + 1):
            gpu.cycle(1)
            orc.cycle(1)
            bad = compare(gpu.state(), orc.state(tmp), RTOL)
            assert not bad, f"{name} step {s}: {bad}"
    gpu.close()
    orc.close()
    cfg.close()


def test_fp64_phase_by_phase(lib, oracle_lib):
    """Each reference entry point on its own (dem, coupling, lb, free surface)."""
    cfg, gpu, orc = _pair("small_cells")
    with tempfile.TemporaryDirectory() as tmp:
        for s in range(1, 11):
            for phase in ("dem_step", "coupling_step", "lb_step", "free_surface_step"):
                getattr(gpu, phase)()
                getattr(orc, phase)()
                bad = compare(gpu.state(), orc.state(tmp), RTOL,
                              fluid_mass=phase != "lb_step")
                assert not bad, f"step {s} after {phase}: {bad}"
    gpu.close()
    orc.close()
    cfg.close()


def test_fp64_config1_100_steps(lib, oracle_lib):
    """The c1 case (64x80x64 lattice, 376 spheres): 100-step horizon."""
    cfg, gpu, orc = _pair("c1")
    with tempfile.TemporaryDirectory() as tmp:
        for s in range(10, 101, 10):
            gpu.cycle(10)
            orc.cycle(10)
            g, o = gpu.state(), orc.state(tmp)
            bad = compare(g, o, RTOL)
            assert not bad, f"config 1 step {s}: {bad}"
        m0 = float(np.sum(o["mass"]))
        mg = float(np.sum(g["mass"]))
        assert abs(mg - m0) <= 1e-12 * abs(m0)
    gpu.close()
    orc.close()
    cfg.close()


def test_fp64_reference_example(lib, oracle_lib):
    """The reference's example input (unitLength 0.2, unitTime 1e-3,
    unitDensity 1; 123x200x123 lattice, 962 spheres of radius 1.0/1.2, one
    impactor; demInitialRepeat 0, objWaitTime 2): every physical/lattice unit
    conversion of the coupling, the lubrication coefficient pi nu a dt and
    the DEM in physical units, over 20 steps."""
    cfg, gpu, orc = _pair("example")
    with tempfile.TemporaryDirectory() as tmp:
        done = 0
        for s in (1, 2, 3, 4, 5, 10, 15, 20):
            gpu.cycle(s - done)
            orc.cycle(s - done)
            done = s
            g, o = gpu.state(), orc.state(tmp)
            bad = compare(g, o, RTOL)
            assert not bad, f"example step {s}: {bad}"
        act = (o["type"] == 0) | (o["type"] == 3)
        m0 = float(np.sum(o["mass"][act]))
        mg = float(np.sum(g["mass"][act]))
        assert abs(mg - m0) <= 1e-12 * abs(m0)
    gpu.close()
    orc.close()
    cfg.close()
