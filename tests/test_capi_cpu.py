"""Host-side checks of the C ABI that need no GPU: the library loads, exports
every entry point include/lbdem.h declares, parses the reference's input
format, and refuses to run without a device instead of falling back."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from conftest import REPO, GOLDEN


def header_functions():
    src = open(os.path.join(REPO, "include", "lbdem.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(lbdem_[a-z_0-9]+)\s*\(", src)))


def test_every_declared_symbol_is_exported(lib):
    names = header_functions()
    assert len(names) >= 19
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, f"not exported: {missing}"


def test_config_load_reads_reference_format(lib):
    import lbdem
    cfg = lbdem.LoadedConfig(os.path.join(GOLDEN, "small_cells", "parameters.cfg"))
    c = cfg.cfg
    assert (c.lbSizeX, c.lbSizeY, c.lbSizeZ) == (28.0, 40.0, 28.0)
    assert c.n_particles == 16 and c.n_objects == 1 and c.n_bodies == 0
    assert c.objWaitTime == 3 and c.freeSurfaceSolve == 1
    assert list(c.boundary) == [7] * 6
    # particles.dat coordinates are shifted by -0.05 on read (src/DEM.cpp:101)
    raw = open(os.path.join(GOLDEN, "small_cells", "input", "particles.dat")).read().split()
    x_file = float(raw[1 + 3])
    assert c.particles[0].x[0] == pytest.approx(x_file - 0.05, abs=0, rel=0)
    assert c.particles[0].size == 1
    cfg.close()


def test_config_command_line_overrides(lib):
    import lbdem
    cfg = lbdem.LoadedConfig(os.path.join(GOLDEN, "small_cells", "parameters.cfg"),
                             overrides={"demInitialRepeat": 7.5, "objWaitTime": 11})
    assert cfg.cfg.demInitialRepeat == 7.5
    assert cfg.cfg.objWaitTime == 11
    cfg.close()


def test_config_errors_are_reported(lib, tmp_path):
    import lbdem
    with pytest.raises(RuntimeError, match="cannot open"):
        lbdem.LoadedConfig(str(tmp_path / "missing.cfg"))
    (tmp_path / "p.cfg").write_text("lbSizeX = 10\n")
    with pytest.raises(RuntimeError, match="particles.dat"):
        lbdem.LoadedConfig(str(tmp_path / "p.cfg"))


def test_create_without_gpu_fails_loudly(lib):
    from conftest import gpu_available
    if gpu_available():
        pytest.skip("a GPU is present")
    import lbdem
    cfg = lbdem.LoadedConfig(os.path.join(GOLDEN, "tiny_direct", "parameters.cfg"))
    with pytest.raises(RuntimeError, match="no CUDA device|CUDA"):
        lbdem.Solver(cfg)
    cfg.close()


def test_mixed_form_refuses_a_per_node_viscosity(lib):
    """Non-Newtonian rheology and the Smagorinsky term run in the plain FP64
    form; the mixed form refuses them before any device use."""
    import lbdem
    for name in ("rheo_bingham", "rheo_turbulent"):
        cfg = lbdem.LoadedConfig(os.path.join(GOLDEN, name, "parameters.cfg"))
        with pytest.raises(RuntimeError, match="mixed form runs NEWTONIAN"):
            lbdem.Solver(cfg, precision=lbdem.MIXED)
        cfg.close()


def test_unsupported_inputs_are_rejected_before_device_use(lib):
    import lbdem
    cfg = lbdem.LoadedConfig(os.path.join(GOLDEN, "tiny_direct", "parameters.cfg"),
                             overrides={"boundary0": 4, "boundary1": 4})
    with pytest.raises(RuntimeError, match="only walls on every face"):
        lbdem.Solver(cfg)
    cfg.close()
