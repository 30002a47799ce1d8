"""Pure-Python reader of a case in the reference's input format.

Test and baseline infrastructure: it fills the lbdem_config structure
(lbdem_types.Config, include/lbdem.h) from a GetPot ``parameters.cfg`` and
``input/{particles,objects,body}.dat`` without loading liblbdem.so, so that
the CPU restatement (oracle/) can be run and timed on its own, and so that
the library's own reader (csrc/config.cpp) can be checked against an
independent one.

It reads what the reference reads:
- the GetPot keys of LB::latticeBoltzmannGet (src/LB.cpp:128-338),
  DEM::discreteElementGet (src/DEM.cpp:17-78) and parseConfigFile
  (src/main.cpp:128-185), with the third argument of each
  PARSE_CLASS_MEMBER as its default, and "-key value" overrides that win
  over the file (src/macros.h:14-19);
- particles.dat (src/DEM.cpp:80-134: radius and position times ``scale``,
  positions less 0.05), objects.dat (src/DEM.cpp:137-166), body.dat
  (src/DEM.cpp:168-196: index, radius, position times ``scale``, velocity,
  spring stiffness and rest length).

Value conversion follows GetPot's stream rules: an integer key takes the
leading integer of its token, a real key the leading number, a failed
conversion keeps the default; a boolean is TRUE/FALSE anywhere in the token
(any case), else an unsigned number.
"""
from __future__ import annotations

import ctypes as C
import os
import re
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(os.path.dirname(HERE), "lbm-dem_gb300"))

from lbdem_types import BodyIn, Config, ObjectIn, ParticleIn  # noqa: E402

_INT = re.compile(r"\s*([+-]?\d+)")
_REAL = re.compile(r"\s*([+-]?(?:\d+\.?\d*|\.\d+)(?:[eE][+-]?\d+)?|[+-]?(?:inf|nan))",
                   re.IGNORECASE)


def tokenize(text: str) -> dict:
    """GetPot file -> {key: value} (last definition wins)."""
    tok: list[str] = []
    for line in text.splitlines():
        cur, quoted = "", False
        for ch in line:
            if quoted:
                if ch == '"':
                    quoted = False
                else:
                    cur += ch
                continue
            if ch == "#":
                break
            if ch == '"':
                quoted = True
                continue
            if ch == "=":
                if cur:
                    tok.append(cur)
                cur = ""
                tok.append("=")
                continue
            if ch.isspace():
                if cur:
                    tok.append(cur)
                cur = ""
                continue
            cur += ch
        if cur:
            tok.append(cur)
    out: dict[str, str] = {}
    k = 0
    while k + 1 < len(tok):
        if tok[k + 1] == "=" and tok[k] != "=":
            v = tok[k + 2] if k + 2 < len(tok) and tok[k + 2] != "=" else ""
            out[tok[k]] = v
            k += 2 if v == "" else 3
        else:
            k += 1
    return out


class _Keys:
    def __init__(self, file: dict, cli: dict):
        self.file, self.cli = file, cli

    def find(self, k):
        if k in self.cli:
            return self.cli[k]
        return self.file.get(k)

    def d(self, k, default):
        s = self.find(k)
        if s is None:
            return float(default)
        m = _REAL.match(s)
        return float(m.group(1)) if m else float(default)

    def i(self, k, default):
        s = self.find(k)
        if s is None:
            return int(default)
        m = _INT.match(s)
        if not m:
            return int(default)
        v = int(m.group(1))
        return v if -2**31 <= v < 2**31 else int(default)

    def b(self, k, default):
        s = self.find(k)
        if s is None:
            return bool(default)
        u = s.upper()
        if "TRUE" in u:
            return True
        if "FALSE" in u:
            return False
        m = _INT.match(s)
        return (int(m.group(1)) != 0) if m else bool(default)

    def s(self, k, default):
        v = self.find(k)
        return default if v is None else v


class CaseConfig:
    """A case read without the library: ``.cfg`` is the filled Config.

    Keeps the particle and impactor tables (and the restart file name) alive
    for as long as the object lives, as lbdem.LoadedConfig does.
    """

    def __init__(self, cfg_path: str, input_dir: str | None = None,
                 overrides: dict | None = None):
        with open(cfg_path) as fh:
            file = tokenize(fh.read())
        cli = {str(k): str(v) for k, v in (overrides or {}).items()}
        ks = _Keys(file, cli)
        c = Config()
        c.unitLength = c.unitTime = c.unitDensity = 1.0
        for a in range(3):
            c.lbRotCenter[a] = -1.0
        c.demInitialRepeat = ks.d("demInitialRepeat", 0.0)
        c.lbmInitialRepeat = ks.i("lbmInitialRepeat", 0)
        c.maxTime = ks.d("maxTime", 0.0)
        c.maximumTimeSteps = ks.i("maximumTimeSteps", 0)
        for k in ("screenExpTime", "fluidExpTime", "fluidLagrangianExpTime", "partExpTime",
                  "fluidRecycleExpTime", "partRecycleExpTime"):
            setattr(c, k, ks.d(k, 0.0))
        for k in ("demSolve", "lbSolve", "freeSurfaceSolve", "forceFieldSolve"):
            setattr(c, k, ks.i(k, 0))
        c.lbRestart = int(ks.b("lbRestart", False))
        restart = ks.s("lbRestartFile", "")
        self._restart = restart.encode() if restart else None
        c.lbRestartFile = self._restart
        c.lbTopography = int(ks.b("lbTopography", False))
        c.unitLength = ks.d("unitLength", 1.0)
        c.unitTime = ks.d("unitTime", 1.0)
        c.unitDensity = ks.d("unitDensity", 1.0)
        c.lbSizeX = ks.d("lbSizeX", 0.0)
        c.lbSizeY = ks.d("lbSizeY", 0.0)
        c.lbSizeZ = ks.d("lbSizeZ", 0.0)
        rheo = ks.s("rheologyModel", "none")
        model = {"BINGHAM": 1, "FRICTIONAL": 2, "VOELLMY": 3}.get(rheo, 0)
        c.rheologyModel = model
        c.rheologyNewtonian = 1 if model == 0 else 0
        c.initVisc = (1.0 - 0.5) / 3.0 if model == 1 else ks.d("initVisc", 1.0)
        if model == 1:
            c.plasticVisc = ks.d("plasticVisc", 0.0)
            c.yieldStress = ks.d("yieldStress", 0.0)
        if model in (2, 3):
            c.frictionCoefFluid = ks.d("frictionCoefFluid", 0.0)
        if model == 3:
            c.voellmyConstant = ks.d("voellmyConstant", 1.0)
        c.turbulenceSolve = ks.i("turbulenceSolve", 0)
        c.turbConst = ks.d("turbConst", 0.0)
        for a, ax in enumerate("XYZ"):
            c.initVelocity[a] = ks.d("initVelocity" + ax, 0.0)
            c.lbF[a] = ks.d("lbF" + ax, 0.0)
            c.lbRot[a] = ks.d("lbRot" + ax, 0.0)
            c.lbRotCenter[a] = ks.d("lbRotCenter" + ax, -1.0)
        for b in range(6):
            c.boundary[b] = ks.i(f"boundary{b}", 1)
        c.slipCoefficient = ks.d("slipCoefficient", 0.0)
        c.fluidHeight = ks.d("fluidHeight", 0.0)
        for k in ("density", "objectDensity", "bodyDensity", "linearStiff",
                  "frictionCoefPart", "lubNormal", "lubTangential", "lubRotation",
                  "lubCutoff", "kinVisc", "electroForce", "debyeLength", "springDamp",
                  "epsilon", "k13"):
            setattr(c, k, ks.d(k, 0.0))
        for k in ("objWaitTime", "intervalTime", "nonLinType"):
            setattr(c, k, ks.i(k, 0))
        c.scale = ks.d("scale", 1.0)
        self._read_inputs(c, input_dir or os.path.join(
            os.path.dirname(os.path.abspath(cfg_path)), "input"))
        self.cfg = c

    def _read_inputs(self, c: Config, d: str) -> None:
        scale = c.scale
        with open(os.path.join(d, "particles.dat")) as fh:
            tok = fh.read().split()
        tot = int(tok[0])
        parts = (ParticleIn * max(tot, 1))()
        pos = 1
        for n in range(tot):
            row = tok[pos:pos + 20]
            if len(row) < 20:
                raise ValueError("malformed particles.dat")
            pos += 20
            p = parts[n]
            p.index = int(row[0])
            p.size = int(row[1])
            p.r = float(row[2]) * scale
            for a in range(3):
                p.x[a] = float(row[3 + a]) * scale - 0.05
                p.v[a] = float(row[6 + a])
                p.w[a] = float(row[9 + a])
        with open(os.path.join(d, "objects.dat")) as fh:
            tok = fh.read().split()
        ot = int(tok[0])
        objs = (ObjectIn * max(ot, 1))()
        pos = 1
        for n in range(ot):
            row = tok[pos:pos + 8]
            if len(row) < 8:
                raise ValueError("malformed objects.dat")
            pos += 8
            o = objs[n]
            o.index = int(row[0])
            o.r = float(row[1]) * scale
            for a in range(3):
                o.x[a] = float(row[2 + a]) * scale
                o.v[a] = float(row[5 + a])
        with open(os.path.join(d, "body.dat")) as fh:
            tok = fh.read().split()
        bt = int(tok[0])
        bodies = (BodyIn * max(bt, 1))()
        pos = 1
        for n in range(bt):
            row = tok[pos:pos + 10]
            if len(row) < 10:
                raise ValueError("malformed body.dat")
            pos += 10
            b = bodies[n]
            b.index = int(row[0])
            b.r = float(row[1])
            for a in range(3):
                b.x[a] = float(row[2 + a]) * scale
                b.v[a] = float(row[5 + a])
            b.k = float(row[8])
            b.L0 = float(row[9])
        self._bodies = bodies
        c.n_bodies = bt
        c.bodies = C.cast(bodies, C.POINTER(BodyIn))
        self._parts, self._objs = parts, objs
        c.n_particles = tot
        c.particles = C.cast(parts, C.POINTER(ParticleIn))
        c.n_objects = ot
        c.objects = C.cast(objs, C.POINTER(ObjectIn))

    def close(self):
        self.cfg = None
