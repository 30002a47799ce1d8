"""Generate the golden fixtures from the pinned reference build.

Run here (where the reference tree exists):
    make -C oracle ref REF=<reference>/src && python tests/golden/make_golden.py

For every case it writes tests/golden/<case>/ (parameters.cfg + input/*.dat,
the exact inputs the reference read) and tests/golden/<case>.npz holding, for
each dumped step, the SHA-256 of every array of the reference's state dump
(oracle/statedump.h layout) and the full particle / impactor / wall arrays.
Bit-exact agreement with the reference is then checked by hashing the
oracle's dump of the same step (tests/test_oracle_golden.py). The lattice
arrays themselves are too large to commit; their hashes pin them.
"""
from __future__ import annotations

import hashlib
import json
import os
import shutil
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(REPO, "lbm-dem_gb300"))
sys.path.insert(0, os.path.join(REPO, "tests"))

import casegen  # noqa: E402
from dumpio import read_dump  # noqa: E402

REF = os.path.join(REPO, "oracle", "_ref", "lbdem_ref")

# case name -> (steps, dump every, full arrays every); hashes are kept for
# every dumped step, the full particle / impactor / wall arrays (failure
# details and branch coverage) for every "full arrays every"-th of them
CASES = {
    "tiny_direct": (60, 1, 1),
    "small_cells": (60, 1, 1),
    "small_dup": (60, 1, 1),
    "c1": (100, 10, 1),
    "units_dyn": (60, 1, 1),
    "example": (20, 1, 10),
    "rheo_bingham": (40, 1, 1),
    "rheo_frictional": (40, 1, 1),
    "rheo_voellmy": (40, 1, 1),
    "rheo_turbulent": (40, 1, 1),
    "bodies": (40, 1, 1),
    "bodies_lj": (40, 1, 1),
    "slip_stat": (40, 1, 1),
    "slip_dyn": (40, 1, 1),
    "uncover_mid": (40, 1, 1),
    "uncover_wide": (40, 1, 1),
}

# The reference's own example input (example/input: unitLength 0.2,
# unitTime 1e-3, 123x200x123 lattice, 962 spheres of radius 1.0/1.2, one
# impactor), with two keys changed only to shorten the run: the DEM-only
# start (demInitialRepeat, 1000 steps) and the impactor wait (objWaitTime,
# 1000 steps) become 0 and 2 steps, so that lubrication and the impactor's
# motion start within the recorded steps.
EXAMPLE_OVERRIDES = {"demInitialRepeat": "0.0", "objWaitTime": "2"}


def write_example(cdir: str) -> None:
    src = os.environ.get("LBDEM_REFERENCE_SRC", "")
    ex = os.path.join(src, "..", "example", "input")
    if not src or not os.path.isfile(os.path.join(ex, "parameters.cfg")):
        sys.exit("set LBDEM_REFERENCE_SRC to the reference's src directory (its example/input "
                 "is read from there)")
    os.makedirs(os.path.join(cdir, "input"))
    with open(os.path.join(ex, "parameters.cfg")) as fh:
        lines = fh.read().split("\n")
    for i, line in enumerate(lines):
        key = line.split("=")[0].strip()
        if key in EXAMPLE_OVERRIDES:
            lines[i] = f"{key} = {EXAMPLE_OVERRIDES[key]}"
    with open(os.path.join(cdir, "parameters.cfg"), "w") as fh:
        fh.write("\n".join(lines))
    for f in ("particles.dat", "objects.dat", "body.dat"):
        shutil.copyfile(os.path.join(ex, f), os.path.join(cdir, "input", f))

SMALL_KEYS = ("p_", "o_", "w_", "b_", "step", "demTime", "demTimeStep")


def array_hash(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def make(name: str, steps: int, every: int, keep: int = 1) -> None:
    cdir = os.path.join(HERE, name)
    if os.path.isdir(cdir):
        shutil.rmtree(cdir)
    if name == "example":
        write_example(cdir)
    else:
        casegen.named_case(name).write(cdir)
    with tempfile.TemporaryDirectory() as tmp:
        dump = os.path.join(tmp, "dump")
        subprocess.run([REF, "-c", "parameters.cfg", "-steps", str(steps), "-dump", dump,
                        "-every", str(every)], cwd=cdir, check=True,
                       stdout=subprocess.DEVNULL)
        hashes = {}
        arrays = {}
        for s in [0] + list(range(every, steps + 1, every)):
            d = read_dump(os.path.join(dump, f"dump_{s:06d}.bin"))
            hashes[str(s)] = {k: array_hash(v) for k, v in d.items()}
            for k, v in d.items():
                if k.startswith(SMALL_KEYS) and (s // every) % keep == 0:
                    arrays[f"s{s}/{k}"] = v
            # a few lattice summaries, useful when a hash differs
            arrays[f"s{s}/type_counts"] = np.bincount(d["type"], minlength=13)
            arrays[f"s{s}/mass_sum"] = np.array([d["mass"].sum()])
    np.savez_compressed(os.path.join(HERE, f"{name}.npz"),
                        hashes=np.frombuffer(json.dumps(hashes).encode(), np.uint8),
                        **arrays)
    print(name, "steps", steps, "every", every, "arrays every", keep)


def main(names=None):
    if not os.path.exists(REF):
        sys.exit("oracle/_ref/lbdem_ref missing: run `make -C oracle ref REF=<reference>/src` first")
    for name in names or CASES:
        make(name, *CASES[name])


if __name__ == "__main__":
    main(sys.argv[1:] or None)
