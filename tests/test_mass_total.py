"""lbdem_mass_total: mass of every active node (inside particles included)
against the oracle's state after the same cycles, plain FP64 form (1e-12
relative, the mass tolerance of the FP64 parity tests)."""
import os
import tempfile

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", ["small_cells", "c1"])
def test_mass_total_matches_oracle(name, lib, oracle_lib):
    import lbdem
    import oracle_ffi
    cfg = lbdem.LoadedConfig(os.path.join(GOLDEN, name, "parameters.cfg"))
    gpu = lbdem.Solver(cfg, precision=lbdem.PLAIN_FP64)
    orc = oracle_ffi.Oracle(cfg)
    gpu.cycle(10)
    orc.cycle(10)
    with tempfile.TemporaryDirectory() as tmp:
        o = orc.state(tmp)
    act = (o["type"] == 0) | (o["type"] == 3)
    ref = float(np.sum(o["mass"][act]))
    got = gpu.mass_total()
    assert abs(got - ref) <= 1e-12 * abs(ref), (got, ref)
    # the particle interiors are part of it
    assert got > gpu.mass_summary()[0]
    gpu.close()
    orc.close()
    cfg.close()
