"""An impactor that reaches through the box walls (GPU, both forms).

The impactor (radius 5) starts with its centre at x = 2, so the sphere
covers nodes of the x = 0 wall layer, which become impactor nodes, and it
moves away at 0.1 per step. The reference then turns the uncovered wall
nodes with fluid neighbours into fluid nodes (the oracle: 56 such nodes
after 60 steps), which stream through neighbour offsets that leave the
node array. Here they become gas, so no node of the outer layer is ever
fluid or interface, and the run stays finite.
"""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _case(tmp_path):
    import casegen
    import lbdem
    c = casegen.impact_case((24, 32, 24), 20.0, 4, (3.0, 3.4), 5.0, 12.0, 0.0, 5.0, 0.8,
                            1.0e-4, 1, overrides={"objWaitTime": "0"}, name="wallimp")
    c.objects[0, 1] = 2.0  # centre x: the sphere reaches through the x = 0 layer
    c.objects[0, 4] = 0.1  # moving away from it
    # spheres well clear of the impactor
    c.particles[:, 1] = np.clip(c.particles[:, 1], 12.0, 19.0)
    return lbdem.LoadedConfig(c.write(str(tmp_path / "wallimp")))


def _outer(t, lb_size):
    X, Y, Z = (int(v) for v in lb_size)
    t = t.reshape(Z, Y, X)
    b = np.zeros_like(t, bool)
    b[0], b[-1] = True, True
    b[:, 0], b[:, -1] = True, True
    b[:, :, 0], b[:, :, -1] = True, True
    return t[b]


@pytest.mark.parametrize("prec_name", ["fp64", "mixed"])
def test_uncovered_wall_nodes_stay_gas(prec_name, lib, tmp_path):
    import lbdem
    prec = lbdem.PLAIN_FP64 if prec_name == "fp64" else lbdem.MIXED
    cfg = _case(tmp_path)
    s = lbdem.Solver(cfg, precision=prec)
    st = s.state()
    first = _outer(st["type"], s.info.lb_size)
    assert np.sum(first == 12) > 0  # wall nodes covered by the impactor
    for _ in range(6):
        s.cycle(10)
        st = s.state()
        outer = _outer(st["type"], s.info.lb_size)
        assert not np.any((outer == 0) | (outer == 3)), np.unique(outer, return_counts=True)
        assert np.all(np.isfinite(st["f"])) and np.all(np.isfinite(st["o_x0"]))
    # the impactor moved away: wall nodes it covered were uncovered, as gas
    assert np.sum(outer == 2) > 0
    assert np.sum(outer == 12) < np.sum(first == 12)
    s.close()
    cfg.close()
