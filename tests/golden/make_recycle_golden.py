"""Generate the golden fluid recycle files from the pinned reference build.

Run here (where the reference tree exists):
    make -C oracle ref REF=<reference>/src && python tests/golden/make_recycle_golden.py

For the tiny_direct case (tests/golden/tiny_direct/) it
1. runs the reference with its own IO code (oracle/_ref/lbdem_ref -io) for
   WRITE_STEP cycles with fluidRecycleExpTime = WRITE_STEP, and keeps the
   recycle file IO::exportRecycleFluid wrote after the last cycle as
   tests/golden/recycle/tiny_direct_step<WRITE_STEP>.dat.gz;
2. starts the reference again from that file (lbRestart = 1,
   lbRestartFile = the file: LB::restartInterface / restartVariables), runs
   RESTART_STEPS cycles with a state dump after each, and keeps the particle,
   impactor and wall arrays of every dump, the type counts and the mass sum
   in tests/golden/recycle/tiny_direct_restart.npz.
"""
from __future__ import annotations

import gzip
import os
import shutil
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(REPO, "tests"))

from dumpio import read_dump  # noqa: E402

REF = os.path.join(REPO, "oracle", "_ref", "lbdem_ref")
CASE = "tiny_direct"
WRITE_STEP = 8
RESTART_STEPS = 6
SMALL_KEYS = ("p_", "o_", "w_", "step", "demTime", "demTimeStep")


def main() -> None:
    if not os.path.exists(REF):
        sys.exit("oracle/_ref/lbdem_ref missing: run `make -C oracle ref REF=<reference>/src` first")
    out = os.path.join(HERE, "recycle")
    os.makedirs(out, exist_ok=True)
    with tempfile.TemporaryDirectory() as tmp:
        case = os.path.join(tmp, CASE)
        shutil.copytree(os.path.join(HERE, CASE), case)
        subprocess.run([REF, "-c", "parameters.cfg", "-steps", str(WRITE_STEP), "-io", "io",
                        "-fluidRecycleExpTime", str(WRITE_STEP)], cwd=case, check=True,
                       stdout=subprocess.DEVNULL)
        rec = os.path.join(case, "io", "fluidData", f"fluidRecycle{WRITE_STEP:010d}.dat")
        with open(rec, "rb") as src, open(
                os.path.join(out, f"{CASE}_step{WRITE_STEP}.dat.gz"), "wb") as raw, \
                gzip.GzipFile(fileobj=raw, mode="wb", mtime=0) as dst:
            shutil.copyfileobj(src, dst)
        dump = os.path.join(tmp, "dump")
        subprocess.run([REF, "-c", "parameters.cfg", "-steps", str(RESTART_STEPS), "-dump", dump,
                        "-every", "1", "-lbRestart", "1", "-lbRestartFile", rec], cwd=case,
                       check=True, stdout=subprocess.DEVNULL)
        arrays = {}
        for s in range(RESTART_STEPS + 1):
            d = read_dump(os.path.join(dump, f"dump_{s:06d}.bin"))
            for k, v in d.items():
                if k.startswith(SMALL_KEYS):
                    arrays[f"s{s}/{k}"] = v
            arrays[f"s{s}/type_counts"] = np.bincount(d["type"], minlength=13)
            arrays[f"s{s}/mass_sum"] = np.array([d["mass"].sum()])
    np.savez_compressed(os.path.join(out, f"{CASE}_restart.npz"), **arrays)
    print("wrote", out)


if __name__ == "__main__":
    main()
