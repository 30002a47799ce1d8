"""The CPU restatement (oracle) against the pinned reference's golden dumps.

The golden fixtures hold, per step, the SHA-256 of every array of the
reference's state dump (tests/golden/make_golden.py). The oracle must
reproduce each of them exactly: node types and flags, solid indices,
distributions, densities, velocities, masses, particle and impactor state,
neighbour lists and tangential springs.
"""
import hashlib
import json
import os

import numpy as np
import pytest

from conftest import golden_case
from dumpio import read_dump


def _hash(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def _run(name, lib, oracle_lib, tmp_path):
    import lbdem
    import oracle_ffi
    cfg_path, gold = golden_case(name)
    hashes = json.loads(bytes(gold["hashes"]).decode())
    steps = sorted(int(s) for s in hashes)
    cfg = lbdem.LoadedConfig(cfg_path)
    orc = oracle_ffi.Oracle(cfg)
    done = 0
    for s in steps:
        if s > done:
            orc.cycle(s - done)
            done = s
        p = os.path.join(tmp_path, "o.bin")
        orc.dump(p)
        d = read_dump(p)
        ref = hashes[str(s)]
        bad = [k for k in ref if k in d and _hash(d[k]) != ref[k]]
        if bad:
            detail = {k: (d[k].ravel()[:3].tolist(), gold[f"s{s}/{k}"].ravel()[:3].tolist())
                      for k in bad if f"s{s}/{k}" in gold}
            pytest.fail(f"{name} step {s}: arrays differ from the reference: {bad} {detail}")
        assert set(ref) <= set(d), f"missing arrays {set(ref) - set(d)}"
    orc.close()
    cfg.close()


@pytest.mark.parametrize("name", ["tiny_direct", "small_cells", "small_dup", "units_dyn"])
def test_oracle_bitwise_equal_to_reference(name, lib, oracle_lib, tmp_path):
    _run(name, lib, oracle_lib, tmp_path)


def test_oracle_bitwise_equal_to_reference_config1(lib, oracle_lib, tmp_path):
    """The c1 case (64x80x64 lattice, 376 spheres), 100 steps, every 10th."""
    _run("c1", lib, oracle_lib, tmp_path)


@pytest.mark.parametrize("name", ["rheo_bingham", "rheo_frictional", "rheo_voellmy",
                                  "rheo_turbulent"])
def test_oracle_bitwise_equal_to_reference_rheology(name, lib, oracle_lib, tmp_path):
    """Bingham, frictional and Voellmy apparent viscosity and the Smagorinsky
    term (node::computeApparentViscosity), per-node viscosity included."""
    _run(name, lib, oracle_lib, tmp_path)


@pytest.mark.parametrize("name", ["bodies", "bodies_lj", "slip_stat", "slip_dyn"])
def test_oracle_bitwise_equal_to_reference_bodies(name, lib, oracle_lib, tmp_path):
    """Bodies joined to the impactor by springs (DEM::bodyObjectInteraction):
    spring-dashpot-cubic and Lennard-Jones repulsion, body state included."""
    _run(name, lib, oracle_lib, tmp_path)


def test_oracle_bitwise_equal_to_reference_example(lib, oracle_lib, tmp_path):
    """The reference's own example input in physical units (unitLength 0.2,
    unitTime 1e-3, 123x200x123 lattice, 962 spheres), 20 steps."""
    _run("example", lib, oracle_lib, tmp_path)


@pytest.mark.parametrize("name", ["uncover_mid", "uncover_wide"])
def test_oracle_bitwise_equal_to_reference_uncover(name, lib, oracle_lib, tmp_path):
    """A large, fast impactor: 36-80 (mid) and 200-350 (wide) nodes uncovered
    per step, resolved together (LB::findNewActiveObject)."""
    _run(name, lib, oracle_lib, tmp_path)


def test_uncover_cases_reach_many_nodes(lib, oracle_lib, tmp_path):
    """The uncover cases free more than 32, more than 64 and more than 256
    nodes in single steps (type 12, an impactor node, becoming another type),
    the sizes at which the resolution of uncovered nodes changes method."""
    import lbdem
    import oracle_ffi
    per_step = []
    for name in ("uncover_mid", "uncover_wide"):
        cfg_path, _ = golden_case(name)
        cfg = lbdem.LoadedConfig(cfg_path)
        orc = oracle_ffi.Oracle(cfg)
        prev = orc.state(str(tmp_path))["type"].copy()
        for _ in range(40):
            orc.cycle(1)
            t = orc.state(str(tmp_path))["type"]
            per_step.append(int(np.sum((prev == 12) & (t != 12))))
            prev = t.copy()
        orc.close()
        cfg.close()
    assert any(32 < n <= 64 for n in per_step), per_step
    assert any(64 < n <= 256 for n in per_step), per_step
    assert any(n > 256 for n in per_step), per_step


def test_golden_cases_exercise_every_branch():
    """The small cases must cover the reference's branches the GPU path
    reimplements: fill/empty conversions, impactor cover/uncover, contacts,
    lubrication, electrostatics, impactor-particle contact."""
    seen = dict(filled=0, emptied=0, uncover=0, contact=0, lub=0, rep=0, objcontact=0)
    for name in ("tiny_direct", "small_cells", "small_dup"):
        _, g = golden_case(name)
        for s in range(1, 61):
            tc = g[f"s{s}/type_counts"]
            seen["contact"] += int(np.any(g[f"s{s}/p_FContact"] != 0))
            seen["lub"] += int(np.any(g[f"s{s}/p_FLub"] != 0))
            seen["rep"] += int(np.any(g[f"s{s}/p_FRep"] != 0))
            seen["objcontact"] += int(np.any(g[f"s{s}/o_FContact"] != 0))
            prev = g[f"s{s-1}/type_counts"]
            seen["uncover"] += int(tc[12] != prev[12])
            seen["filled"] += int(tc[0] != prev[0])
            seen["emptied"] += int(tc[2] != prev[2])
    for k, v in seen.items():
        assert v > 0, f"golden cases never exercise {k}"
