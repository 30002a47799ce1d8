"""Generate the golden screen-phase output files from the pinned reference
build.

Run here (where the reference tree exists):
    make -C oracle ref REF=<reference>/src && python tests/golden/make_io_golden.py

For every case below it runs the reference's own IO code (oracle/_ref/lbdem_ref
with -io, which calls IO::initialize and IO::outputStep of src/IO.cpp) on the
committed inputs of tests/golden/<case>/ with the screenExpTime given here,
and partRecycleExpTime given here, and keeps the files it writes (export.dat,
objPosition.dat, objForce.dat, wallForce.dat, bodyPosition.dat, the three
stress files and the particle recycle files particleData/partRecycle*.dat) in
tests/golden/io/<case>/, with a cases.json of the steps and export times.
"""
from __future__ import annotations

import json
import os
import shutil
import subprocess
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
REF = os.path.join(REPO, "oracle", "_ref", "lbdem_ref")

# case -> (cycles, screenExpTime, partRecycleExpTime); unitTime is 1.0 in
# every case, so the reference writes at cycle 0 and whenever floor(t / T)
# advances
CASES = {
    "tiny_direct": (12, 3.5, 5.0),
    "small_cells": (24, 5.5, 10.0),
    "c1": (30, 7.5, 14.0),
    "bodies": (24, 5.5, 10.0),
}
FILES = ("export.dat", "objPosition.dat", "objForce.dat", "wallForce.dat", "bodyPosition.dat",
         "stressTensor.dat", "normalStressCont.dat", "shearStressCont.dat")


def make(name: str, steps: int, screen: float, part: float) -> None:
    out = os.path.join(HERE, "io", name)
    if os.path.isdir(out):
        shutil.rmtree(out)
    os.makedirs(out)
    with tempfile.TemporaryDirectory() as tmp:
        case = os.path.join(tmp, name)
        shutil.copytree(os.path.join(HERE, name), case)
        subprocess.run([REF, "-c", "parameters.cfg", "-steps", str(steps), "-io", "ioout",
                        "-screenExpTime", repr(screen), "-partRecycleExpTime", repr(part)],
                       cwd=case, check=True, stdout=subprocess.DEVNULL)
        for f in FILES:
            shutil.copy(os.path.join(case, "ioout", f), os.path.join(out, f))
        os.makedirs(os.path.join(out, "particleData"))
        pdir = os.path.join(case, "ioout", "particleData")
        for f in sorted(os.listdir(pdir)):
            if f.startswith("partRecycle"):
                shutil.copy(os.path.join(pdir, f), os.path.join(out, "particleData", f))


def main() -> None:
    for name, (steps, screen, part) in CASES.items():
        make(name, steps, screen, part)
        print("wrote", name)
    with open(os.path.join(HERE, "io", "cases.json"), "w") as fh:
        json.dump({k: {"steps": s, "screenExpTime": e, "partRecycleExpTime": p}
                   for k, (s, e, p) in CASES.items()}, fh, indent=1)


if __name__ == "__main__":
    main()
