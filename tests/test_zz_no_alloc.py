"""lbdem_download_nodes_noalloc, the readback that allocates no device
memory, against lbdem_download_lattice on the same nodes.

Both go through the C ABI. Each check makes two calls of the no-allocation
entry point in a row, in both precision forms, and again after more steps.
Tolerance: none. Both exports compute the same per-node values, so they are
compared for equality. The file name makes it the last file collected, so it
runs after every other GPU test in one process; it passes alone as well.
"""
import os

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu

RTOL = 0.0  # identical per-node arithmetic in both exports


def _compare(s, ranges):
    full = s.lattice()
    for first, count in ranges:  # consecutive calls of the entry point
        f, mass = s.nodes_noalloc(first, count)
        np.testing.assert_allclose(f, full["f"][:, first:first + count], rtol=RTOL, atol=0)
        np.testing.assert_allclose(mass, full["mass"][first:first + count], rtol=RTOL, atol=0)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_noalloc_readback_matches_full_download(precision, lib):
    import lbdem
    cfg = lbdem.LoadedConfig(os.path.join(GOLDEN, "small_cells", "parameters.cfg"))
    s = lbdem.Solver(cfg, precision=lbdem.PLAIN_FP64 if precision == "fp64" else lbdem.MIXED)
    try:
        N = int(s.info.nodes)
        big = lbdem.NOALLOC_MAX_NODES
        assert N > big
        s.cycle(3)
        _compare(s, [(N // 3, big), (N - 1000, 1000)])
        s.cycle(2)
        _compare(s, [(0, 517), (N - big, big)])
        # the populations read back are not all zero (a live lattice)
        f, _ = s.nodes_noalloc(N // 2, 256)
        assert np.count_nonzero(f) > 0
    finally:
        s.close()
        cfg.close()


def test_noalloc_makes_no_device_allocation(lib):
    """Consecutive calls leave the library's allocation count, the context's
    device footprint and the device's free memory where they were. The
    first call (which looks up the staging buffer and may load the module)
    is made before the counts are taken."""
    import torch

    import lbdem
    cfg = lbdem.LoadedConfig(os.path.join(GOLDEN, "small_cells", "parameters.cfg"))
    s = lbdem.Solver(cfg, precision=lbdem.MIXED)
    try:
        N = int(s.info.nodes)
        big = lbdem.NOALLOC_MAX_NODES
        s.cycle(2)
        s.nodes_noalloc(0, 64)
        torch.cuda.synchronize()
        allocs = lbdem.device_allocations()
        footprint = int(s.get_info().device_bytes)
        free0, _ = torch.cuda.mem_get_info()
        for i in range(12):
            first = (i * 7919) % (N - big)
            s.nodes_noalloc(first, big if i % 2 else 1 + i * 1000)
        free1, _ = torch.cuda.mem_get_info()
        assert lbdem.device_allocations() == allocs
        assert int(s.get_info().device_bytes) == footprint
        assert free1 == free0
        # the counter does move for a call that allocates (the full download)
        s.lattice()
        assert lbdem.device_allocations() > allocs
    finally:
        s.close()
        cfg.close()


def test_noalloc_rejects_oversized_and_outside_ranges(lib):
    import lbdem
    cfg = lbdem.LoadedConfig(os.path.join(GOLDEN, "small_cells", "parameters.cfg"))
    s = lbdem.Solver(cfg, precision=lbdem.MIXED)
    try:
        N = int(s.info.nodes)
        with pytest.raises(RuntimeError, match="LBDEM_NOALLOC_MAX_NODES"):
            s.nodes_noalloc(0, lbdem.NOALLOC_MAX_NODES + 1)
        with pytest.raises(RuntimeError, match="outside the lattice"):
            s.nodes_noalloc(N - 10, 11)
        with pytest.raises(RuntimeError, match="outside the lattice"):
            s.nodes_noalloc(-1, 5)
        # the context stays usable after a rejected call
        s.cycle(1)
        _compare(s, [(100, 300), (N - 300, 300)])
    finally:
        s.close()
        cfg.close()
