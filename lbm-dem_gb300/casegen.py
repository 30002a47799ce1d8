"""Seeded synthetic impact cases written in the reference's input format.

The reference reads a GetPot ``parameters.cfg`` (keys as parsed in
src/LB.cpp:128-338, src/DEM.cpp:17-78, src/main.cpp:128-185) and, relative to
the working directory, ``input/particles.dat`` (20 columns, src/DEM.cpp:85-134,
positions shifted by -0.05 on read at src/DEM.cpp:101), ``input/objects.dat``
(8 columns, src/DEM.cpp:142-166) and ``input/body.dat`` (src/DEM.cpp:173-196).
This module produces those files for seeded random-sequential-addition (RSA)
packings. The vertical axis is the reference's ``y``.

Everything here is host-side input preparation; nothing is timed.
"""
from __future__ import annotations

import math
import os
from dataclasses import dataclass, field

import numpy as np

# Keys in the order the reference parses them; values are strings written
# verbatim into parameters.cfg.
DEFAULT_PARAMS: dict[str, str] = {
    "demSolve": "1",
    "lbSolve": "1",
    "freeSurfaceSolve": "1",
    "forceFieldSolve": "1",
    "demInitialRepeat": "0.0",
    "lbmInitialRepeat": "0",
    "maximumTimeSteps": "0",
    "maxTime": "1.0e9",
    "screenExpTime": "0",
    "fluidExpTime": "0",
    "fluidLagrangianExpTime": "0",
    "partExpTime": "0",
    "partRecycleExpTime": "0",
    "fluidRecycleExpTime": "0",
    "unitLength": "1.0",
    "unitTime": "1.0",
    "unitDensity": "1.0",
    "lbSizeX": "64",
    "lbSizeY": "80",
    "lbSizeZ": "64",
    "lbRestart": "false",
    "lbRestartFile": '" "',
    "lbTopography": "false",
    "lbTopographyFile": "./",
    "initVelocityX": "0.0",
    "initVelocityY": "0.0",
    "initVelocityZ": "0.0",
    "lbFX": "0.0",
    "lbFY": "-1.0e-5",
    "lbFZ": "0.0",
    "lbRotX": "0.0",
    "lbRotY": "0.0",
    "lbRotZ": "0.0",
    "lbRotCenterX": "0.0",
    "lbRotCenterY": "0.0",
    "lbRotCenterZ": "0.0",
    "boundary0": "7",
    "boundary1": "7",
    "boundary2": "7",
    "boundary3": "7",
    "boundary4": "7",
    "boundary5": "7",
    "slipCoefficient": "0.0",
    "fluidHeight": "60",
    "rheologyModel": "NEWTONIAN",
    "initVisc": "0.1",
    "turbulenceSolve": "0",
    "turbConst": "0.0",
    "density": "1.0",
    "objectDensity": "5.0",
    "bodyDensity": "1.0",
    "linearStiff": "1.0e-2",
    "frictionCoefPart": "1.0",
    "lubNormal": "1.5",
    "lubTangential": "1.5",
    "lubRotation": "1.5",
    "lubCutoff": "1.0e-3",
    "kinVisc": "0.1",
    "debyeLength": "0.15",
    "electroForce": "1.0e-5",
    "objWaitTime": "1",
    "intervalTime": "0",
    "springDamp": "0.1",
    "epsilon": "1.0",
    "nonLinType": "0",
    "k13": "1.0",
    "scale": "1.0",
}


@dataclass
class Case:
    """One impact run: parameters plus particle and impactor tables.

    ``particles`` rows: r, x, y, z, vx, vy, vz, wx, wy, wz (physical units,
    positions as they should be *after* the reader's -0.05 shift).
    ``objects`` rows: r, x, y, z, vx, vy, vz.
    ``bodies`` rows: r, x, y, z, vx, vy, vz, k, L0 (body.dat,
    src/DEM.cpp:168-196).
    """

    params: dict[str, str] = field(default_factory=lambda: dict(DEFAULT_PARAMS))
    particles: np.ndarray = field(default_factory=lambda: np.zeros((0, 10)))
    objects: np.ndarray = field(default_factory=lambda: np.zeros((0, 7)))
    name: str = "case"
    bodies: np.ndarray = field(default_factory=lambda: np.zeros((0, 9)))

    @property
    def lattice(self) -> tuple[int, int, int]:
        L = float(self.params["unitLength"])
        return tuple(int(math.floor(float(self.params[k]) / L + 0.5))
                     for k in ("lbSizeX", "lbSizeY", "lbSizeZ"))

    def write(self, directory: str) -> str:
        """Write parameters.cfg and input/*.dat; returns the cfg path."""
        os.makedirs(os.path.join(directory, "input"), exist_ok=True)
        cfg = os.path.join(directory, "parameters.cfg")
        with open(cfg, "w") as fh:
            for k, v in self.params.items():
                fh.write(f"{k} = {v}\n")
        with open(os.path.join(directory, "input", "particles.dat"), "w") as fh:
            fh.write(f"{len(self.particles)}\n")
            for i, row in enumerate(self.particles):
                r, x, y, z, vx, vy, vz, wx, wy, wz = (float(a) for a in row)
                # the reader subtracts 0.05 from each coordinate
                vals = [r, x + 0.05, y + 0.05, z + 0.05, vx, vy, vz, wx, wy, wz]
                fh.write(f"{i} 1 " + " ".join(f"{a:.17g}" for a in vals)
                         + " 1 0 0 0 0 0 0 0\n")
        with open(os.path.join(directory, "input", "objects.dat"), "w") as fh:
            fh.write(f"{len(self.objects)}\n")
            for i, row in enumerate(self.objects):
                fh.write(f"{i} " + " ".join(f"{float(a):.17g}" for a in row) + "\n")
        with open(os.path.join(directory, "input", "body.dat"), "w") as fh:
            fh.write(f"{len(self.bodies)}\n")
            for i, row in enumerate(self.bodies):
                fh.write(f"{i} " + " ".join(f"{float(a):.17g}" for a in row) + "\n")
        return cfg


def rsa_pack(rng: np.random.Generator, lo, hi, radii: np.ndarray,
             gap: float = 0.05, max_tries: int = 2000) -> np.ndarray:
    """Random sequential addition of spheres (largest first) into [lo, hi].

    Returns an array (n_placed, 4) of r, x, y, z in insertion order of the
    input ``radii``. A sphere is placed at the first uniformly drawn centre
    whose surface stays ``gap`` away from every placed sphere and inside the
    box; spheres that find no place in ``max_tries`` draws are dropped.
    """
    lo = np.asarray(lo, float)
    hi = np.asarray(hi, float)
    rmax = float(np.max(radii)) if len(radii) else 1.0
    cell = 2.0 * rmax + gap
    dims = np.maximum(1, np.floor((hi - lo) / cell).astype(int))
    grid: dict[tuple[int, int, int], list[int]] = {}
    placed = np.zeros((len(radii), 4))
    n = 0
    for r in radii:
        a = lo + r
        b = hi - r
        if np.any(b <= a):
            continue
        for _ in range(max_tries):
            c = a + (b - a) * rng.random(3)
            key = tuple(np.minimum(dims - 1, ((c - lo) / cell).astype(int)))
            ok = True
            for dx in (-1, 0, 1):
                for dy in (-1, 0, 1):
                    for dz in (-1, 0, 1):
                        for j in grid.get((key[0] + dx, key[1] + dy, key[2] + dz), ()):
                            d = placed[j, 1:] - c
                            if d @ d < (placed[j, 0] + r + gap) ** 2:
                                ok = False
                                break
                        if not ok:
                            break
                    if not ok:
                        break
                if not ok:
                    break
            if ok:
                placed[n] = (r, *c)
                grid.setdefault(key, []).append(n)
                n += 1
                break
    return placed[:n]


def impact_case(lattice=(64, 80, 64), fill=60.0, n_particles=400,
                radii=(3.0, 4.2), impactor_r=8.0, impactor_y=70.0,
                impactor_vy=-0.01, impactor_density=5.0, tau=0.8,
                gravity=1.0e-5, seed=1, gap=0.05, overrides=None,
                name="case", bed_phi=None) -> Case:
    """Bidisperse suspension under a falling impactor (reference axes).

    Lattice sides are in lattice units (unitLength = unitTime = 1), the walls
    are the outermost node layers (wall planes at 0.5 and side-1.5, as set by
    src/LB.cpp:186-193). Half the spheres (by number) take each radius. They
    are RSA-placed below ``fill``, or, with ``bed_phi``, randomly inserted and
    compressed into a bed of that volume fraction on the floor
    (``compress_pack``; the bed must fit below ``fill``).
    """
    rng = np.random.default_rng(seed)
    p = dict(DEFAULT_PARAMS)
    nx, ny, nz = lattice
    p.update({
        "lbSizeX": str(nx), "lbSizeY": str(ny), "lbSizeZ": str(nz),
        "fluidHeight": repr(float(fill)),
        "initVisc": repr((tau - 0.5) / 3.0),
        "kinVisc": repr((tau - 0.5) / 3.0),
        "lbFY": repr(-float(gravity)),
        "objectDensity": repr(float(impactor_density)),
    })
    amean = 0.5 * (radii[0] + radii[1])
    p["lubNormal"] = p["lubTangential"] = p["lubRotation"] = repr(0.5 * amean)
    p["debyeLength"] = repr(0.05 * amean)
    # The reference integrates lubrication explicitly with coefficient
    # Xa ~ 6 pi nu a (a/h) dt (src/DEM.cpp:2354-2373); with dt = 1 lattice step
    # the minimum gap must keep Xa dt / m below 1, hence h_min = 0.1 a.
    p["lubCutoff"] = repr(0.1 * amean)
    if overrides:
        p.update({k: str(v) for k, v in overrides.items()})
    half = n_particles // 2
    rs = np.array([radii[1]] * (n_particles - half) + [radii[0]] * half)
    lo = (0.5, 0.5, 0.5)
    hi = (nx - 1.5, float(fill), nz - 1.5)
    if bed_phi is None:
        pk = rsa_pack(rng, lo, hi, rs, gap=gap)
    else:
        pk, _ = compress_pack(rng, lo, hi, rs, bed_phi)
    order = rng.permutation(len(pk))
    pk = pk[order]
    parts = np.zeros((len(pk), 10))
    parts[:, :4] = pk
    objs = np.zeros((1, 7))
    objs[0] = (impactor_r, 0.5 * (nx - 1), impactor_y, 0.5 * (nz - 1),
               0.0, impactor_vy, 0.0)
    return Case(params=p, particles=parts, objects=objs, name=name)


def _relax(x, r, lo, hi, gap, tol, max_iter, skin, state):
    """Remove overlaps (surfaces closer than ``gap``) by Jacobi position
    projection with heavy-ball momentum: every overlapping pair moves apart
    by half its overlap along the line of centres, the step keeps a fraction
    of the previous one (reset whenever the largest overlap grows), and every
    sphere is clipped into the box. Candidate pairs come from a Verlet list
    (centres within r_i + r_j + gap + skin) rebuilt whenever a sphere has
    moved more than skin / 2 since the last build; the pairs are sorted, so
    the sums (numpy bincount, in order) and the result are the same on every
    machine. Returns the largest remaining overlap."""
    from scipy.spatial import cKDTree
    n = len(r)
    rmax = float(r.max())
    worst = np.inf
    last = np.inf
    v = state.setdefault("v", np.zeros_like(x))
    lo_r = lo + r[:, None]
    hi_r = hi - r[:, None]
    for _ in range(max_iter):
        if state.get("pairs") is None or \
                np.max(np.abs(x - state["xref"])) > 0.5 * skin:
            p = cKDTree(x).query_pairs(2.0 * rmax + gap + skin, output_type="ndarray")
            p = p[np.lexsort((p[:, 1], p[:, 0]))] if len(p) else p.reshape(0, 2)
            i, j = p[:, 0], p[:, 1]
            contact = r[i] + r[j] + gap
            d = np.sqrt(np.sum((x[j] - x[i]) ** 2, axis=1))
            keep = d < contact + skin
            state["pairs"] = (i[keep].copy(), j[keep].copy(), contact[keep].copy())
            state["xref"] = x.copy()
        i, j, contact = state["pairs"]
        d = x[j] - x[i]
        dist = np.sqrt(np.einsum("ij,ij->i", d, d))
        ov = contact - dist
        m = ov > 0.0
        worst = float(ov[m].max()) if m.any() else 0.0
        if worst < tol:
            break
        if worst > last:
            v[:] = 0.0
        last = worst
        im, jm = i[m], j[m]
        s = 0.5 * ov[m] / np.maximum(dist[m], 1e-12)
        dm = d[m] * s[:, None]
        disp = np.empty_like(x)
        for a in range(3):
            disp[:, a] = np.bincount(jm, dm[:, a], n) - np.bincount(im, dm[:, a], n)
        v *= 0.5
        v += 0.6 * disp
        x += v
        np.clip(x, lo_r, hi_r, out=x)
    return worst


def compress_pack(rng: np.random.Generator, lo, hi, radii: np.ndarray, phi: float,
                  phi0: float = 0.30, gap: float = 0.02, step: float = 0.01,
                  tol: float = 1e-3) -> tuple[np.ndarray, float]:
    """Seeded random packing compressed into a bed of volume fraction ``phi``.

    The spheres are inserted at random (volume fraction ``phi0`` of a box as
    wide as [lo, hi] in x and z, as tall in y as that takes), their overlaps
    are relaxed away, and the box is then compressed along y towards the
    bed height H = V_spheres / (phi * width_x * width_z): every stage
    rescales the heights by (1 - ``step``) towards the floor lo[1] and relaxes
    the overlaps again (``_relax``), until the bed is H high. Surfaces end at
    least ``gap`` - ``tol`` apart and inside the box, so no two spheres and no
    sphere and wall touch.

    Returns (rows of r, x, y, z in the order of ``radii``, H).
    """
    lo = np.asarray(lo, float)
    hi = np.asarray(hi, float)
    r = np.asarray(radii, float)
    area = (hi[0] - lo[0]) * (hi[2] - lo[2])
    vol = float(np.sum(4.0 / 3.0 * math.pi * r ** 3))
    H = vol / (phi * area)
    if H > hi[1] - lo[1]:
        raise ValueError(f"a bed at volume fraction {phi} is {H:.1f} high, above the box")
    h = max(vol / (phi0 * area), H)
    top = lo.copy()
    top[0], top[2] = hi[0], hi[2]
    top[1] = lo[1] + h
    x = lo + r[:, None] + (top - lo - 2.0 * r[:, None]) * rng.random((len(r), 3))
    state: dict = {}
    skin = 0.6
    _relax(x, r, lo, top, gap, 0.05, 2000, skin, state)
    while top[1] > lo[1] + H:
        new = max(lo[1] + H, lo[1] + (top[1] - lo[1]) * (1.0 - step))
        x[:, 1] = lo[1] + (x[:, 1] - lo[1]) * ((new - lo[1]) / (top[1] - lo[1]))
        top[1] = new
        _relax(x, r, lo, top, gap, 0.05, 400, skin, state)
    worst = _relax(x, r, lo, top, gap, tol, 20000, skin, state)
    if worst >= tol:
        raise RuntimeError(f"packing did not relax: overlap {worst:.3g} left at phi {phi}")
    return np.column_stack([r, x]), float(H)


def grid_pack(rng: np.random.Generator, lo, hi, radii=(3.0, 4.2), phi=0.3,
              gap: float = 0.05) -> np.ndarray:
    """Spheres on a jittered cubic grid (vectorised, for many cases at once).

    Cells of side 2 r_max + 2 gap tile [lo, hi]; a cell holds a sphere with
    the probability that gives volume fraction ``phi`` (at most about 0.3
    for radii 3.0/4.2), half of them of each radius, each moved at random
    inside its cell by at most the slack its radius leaves, so no two
    spheres overlap. Returns (n, 4) rows of r, x, y, z.
    """
    lo = np.asarray(lo, float)
    hi = np.asarray(hi, float)
    a = 2.0 * max(radii) + 2.0 * gap
    n = np.maximum(np.floor((hi - lo) / a).astype(int), 0)
    if np.any(n == 0):
        return np.zeros((0, 4))
    centres = np.stack(np.meshgrid(*[lo[d] + a * (np.arange(n[d]) + 0.5) for d in range(3)],
                                   indexing="ij"), axis=-1).reshape(-1, 3)
    r = rng.choice(np.asarray(radii, float), size=len(centres))
    vol_box = float(np.prod(hi - lo))
    p = min(1.0, phi * vol_box / float(np.sum(4.0 / 3.0 * math.pi * r ** 3)))
    keep = rng.random(len(centres)) < p
    centres, r = centres[keep], r[keep]
    slack = (a - 2.0 * r - 2.0 * gap)[:, None] / 2.0
    pos = centres + slack * (2.0 * rng.random((len(r), 3)) - 1.0)
    return np.column_stack([r, pos])


def serving_case(rng: np.random.Generator, name: str = "job", bed: bool = True) -> Case:
    """One impact run of a varied job stream: lattice sides 48-128 (vertical
    up to 160), fluid to 60 % of the height, an impactor of radius 6-16 (at
    most what the gas layer holds) falling at 0.005-0.05 just above the
    surface, and a bidisperse suspension (radii 3.0 / 4.2, half each):
    with ``bed``, spheres compressed into a bed of volume fraction drawn from
    0.40-0.55 that fills 80 % of the fluid depth (``compress_pack``);
    otherwise a grid-packed suspension of volume fraction 0.25-0.30 through
    the whole fluid."""
    nx, nz = (int(v) for v in rng.integers(48, 129, size=2))
    ny = int(rng.integers(48, 161))
    fill = 0.6 * ny
    r_imp = float(min(rng.uniform(6.0, 16.0), (ny - 2.0 - fill) / 2.0 - 1.0, (nx - 4) / 2.0,
                      (nz - 4) / 2.0))
    vy = -float(rng.uniform(0.005, 0.05))
    p = dict(DEFAULT_PARAMS)
    tau = 0.6
    p.update({
        "lbSizeX": str(nx), "lbSizeY": str(ny), "lbSizeZ": str(nz),
        "fluidHeight": repr(float(fill)), "initVisc": repr((tau - 0.5) / 3.0),
        "kinVisc": repr((tau - 0.5) / 3.0), "lbFY": repr(-1.0e-5),
        "objectDensity": "5.0",
    })
    amean = 3.6
    p["lubNormal"] = p["lubTangential"] = p["lubRotation"] = repr(0.5 * amean)
    p["debyeLength"] = repr(0.05 * amean)
    p["lubCutoff"] = repr(0.1 * amean)
    if bed:
        phi = float(rng.uniform(0.40, 0.55))
        depth = 0.8 * (fill - 0.5)
        vmean = 0.5 * 4.0 / 3.0 * math.pi * (3.0 ** 3 + 4.2 ** 3)
        n = int(phi * (nx - 2) * (nz - 2) * depth / vmean)
        rs = np.array([4.2] * (n - n // 2) + [3.0] * (n // 2))
        pk, _ = compress_pack(rng, (0.5, 0.5, 0.5), (nx - 1.5, fill, nz - 1.5), rs, phi)
    else:
        pk = grid_pack(rng, (0.5, 0.5, 0.5), (nx - 1.5, fill, nz - 1.5),
                       phi=float(rng.uniform(0.25, 0.30)))
    parts = np.zeros((len(pk), 10))
    parts[:, :4] = pk[rng.permutation(len(pk))]
    objs = np.array([[r_imp, 0.5 * (nx - 1), fill + r_imp + 1.0, 0.5 * (nz - 1), 0.0, vy, 0.0]])
    return Case(params=p, particles=parts, objects=objs, name=name)


def to_physical(case: Case, length: float, time: float, density: float) -> Case:
    """The same run in physical units: unitLength/unitTime/unitDensity set to
    ``length``/``time``/``density`` and every dimensional input scaled so that
    the lattice run is unchanged (LB::latticeBoltzmannGet divides by the
    composite units, src/node.cpp:512-525, src/LB.cpp:153-326; the DEM works in
    physical units). The lubrication viscosity kinVisc is scaled with the
    density as well, so that its coefficient pi nu a dt (src/DEM.cpp:2354)
    keeps its ratio to the particle masses."""
    L, T, D = float(length), float(time), float(density)
    p = dict(case.params)
    scale = {
        "lbSizeX": L, "lbSizeY": L, "lbSizeZ": L, "fluidHeight": L,
        "initVisc": D * L * L / T,
        "lbFX": L / T / T, "lbFY": L / T / T, "lbFZ": L / T / T,
        "initVelocityX": L / T, "initVelocityY": L / T, "initVelocityZ": L / T,
        "density": D, "objectDensity": D, "bodyDensity": D,
        "linearStiff": D * L ** 3 / T / T,
        "kinVisc": D * L * L / T,
        "electroForce": D * L ** 4 / T / T,
        "debyeLength": L, "lubCutoff": L, "lubNormal": L, "lubTangential": L,
        "lubRotation": L,
    }
    for k, f in scale.items():
        p[k] = repr(float(p[k]) * f)
    p["unitLength"], p["unitTime"], p["unitDensity"] = repr(L), repr(T), repr(D)
    parts = case.particles.copy()
    parts[:, 0:4] *= L          # r, x, y, z
    parts[:, 4:7] *= L / T      # v
    parts[:, 7:10] /= T         # w
    objs = case.objects.copy()
    objs[:, 0:4] *= L
    objs[:, 4:7] *= L / T
    return Case(params=p, particles=parts, objects=objs, name=case.name)


def volume_fraction(case: Case) -> float:
    """Spheres' volume over the fluid column below fluidHeight."""
    nx, ny, nz = case.lattice
    fill = float(case.params["fluidHeight"])
    vol = (nx - 2) * (fill - 0.5) * (nz - 2)
    return float(np.sum(4.0 / 3.0 * math.pi * case.particles[:, 0] ** 3) / vol)


def bed_fraction(case: Case) -> float:
    """Spheres' volume over the bed they fill: the box floor (y = 0.5) up to
    the top of the highest sphere, across the inner width of the box."""
    nx, ny, nz = case.lattice
    p = case.particles
    top = float(np.max(p[:, 2] + p[:, 0]))
    return float(np.sum(4.0 / 3.0 * math.pi * p[:, 0] ** 3) / ((nx - 2) * (top - 0.5) * (nz - 2)))


# Named workloads. Sizes follow the benchmark configurations of this project
# (see the bench and the tests); "c1" is the CPU-runnable plain-FP64 case.
def named_case(name: str, seed: int = 1) -> Case:
    if name == "c1":
        return impact_case((64, 80, 64), 60.0, 400, (3.0, 4.2), 8.0, 70.0,
                           -0.01, 5.0, 0.8, 1.0e-5, seed, name=name)
    if name == "c2":
        # 25 000 spheres compressed into a bed of volume fraction 0.50 on the
        # floor (about 164 lattice units high), clear fluid above it to 240
        return impact_case((256, 320, 256), 240.0, 25000, (3.0, 4.2), 20.0,
                           262.0, -0.02, 5.0, 0.6, 1.0e-5, seed, name=name, bed_phi=0.50)
    if name == "c2s":  # config-2 physics on a 160x200x160 lattice (profiling size)
        return impact_case((160, 200, 160), 150.0, 6100, (3.0, 4.2), 14.0, 166.0,
                           -0.02, 5.0, 0.6, 1.0e-5, seed, name=name, bed_phi=0.50)
    if name == "c5":
        # 512x384x512, 200 000 spheres compressed into a bed of volume
        # fraction 0.55 (about 296 high, the fluid is filled to 300); impactor
        # of radius 32, density 8, falling at 0.03 from just above the surface
        return impact_case((512, 384, 512), 300.0, 200000, (3.0, 4.2), 32.0, 334.0,
                           -0.03, 8.0, 0.6, 1.0e-5, seed, name=name, bed_phi=0.55)
    if name == "small_cells":
        return impact_case((28, 40, 28), 27.0, 16, (3.0, 3.4), 5.0, 32.0,
                           -0.08, 5.0, 0.8, 1.0e-4, seed,
                           overrides={"objWaitTime": "3"}, name=name)
    if name == "small_dup":
        return impact_case((28, 40, 18), 27.0, 10, (3.0, 3.4), 4.0, 31.5,
                           -0.08, 5.0, 0.8, 1.0e-4, seed,
                           overrides={"objWaitTime": "3", "demInitialRepeat": "2.5"},
                           name=name)
    if name == "tiny_direct":
        return impact_case((18, 28, 18), 16.0, 5, (3.0, 3.4), 4.0, 20.5,
                           -0.05, 5.0, 0.8, 1.0e-4, seed,
                           overrides={"objWaitTime": "2"}, name=name)
    rheo = {
        # the rheology models of node::computeApparentViscosity
        # (src/node.cpp:113-168) on the small_cells geometry; lattice units
        "rheo_bingham": {"rheologyModel": "BINGHAM", "plasticVisc": "0.1",
                         "yieldStress": "2.0e-6"},
        "rheo_frictional": {"rheologyModel": "FRICTIONAL", "initVisc": "0.1",
                            "frictionCoefFluid": "0.4"},
        "rheo_voellmy": {"rheologyModel": "VOELLMY", "initVisc": "0.1",
                         "frictionCoefFluid": "0.4", "voellmyConstant": "2.0e-4"},
        "rheo_turbulent": {"rheologyModel": "NEWTONIAN", "initVisc": "0.1",
                           "turbulenceSolve": "1", "turbConst": "5.0"},
    }
    if name in rheo:
        ov = {"objWaitTime": "3"}
        ov.update(rheo[name])
        return impact_case((28, 40, 28), 27.0, 16, (3.0, 3.4), 5.0, 32.0,
                           -0.08, 5.0, 0.8, 1.0e-4, seed, overrides=ov, name=name)
    if name in ("slip_stat", "slip_dyn"):
        # slip walls (boundary0 5: static, 6: moving; DEM::initializeWalls
        # gives every wall the slip and moving flags of boundary0) with slip
        # coefficient 0.4, on the small_cells geometry
        ov = {"objWaitTime": "3", "boundary0": "5" if name == "slip_stat" else "6",
              "slipCoefficient": "0.4"}
        return impact_case((28, 40, 28), 27.0, 16, (3.0, 3.4), 5.0, 32.0,
                           -0.08, 5.0, 0.8, 1.0e-4, seed, overrides=ov, name=name)
    if name in ("bodies", "bodies_lj"):
        # two bodies above the impactor, each joined to it by a spring along y
        # (DEM::bodyObjectInteraction): spring-dashpot-cubic (nonLinType 2)
        # or spring-dashpot with the repulsive Lennard-Jones term (nonLinType 3)
        lj = name == "bodies_lj"
        ov = {"objWaitTime": "3", "bodyDensity": "5.0", "springDamp": "0.1",
              "nonLinType": "3" if lj else "2", "k13": "0.5", "epsilon": "1.0e-3"}
        c = impact_case((28, 40, 28), 27.0, 16, (3.0, 3.4), 5.0, 32.0,
                        -0.08, 5.0, 0.8, 1.0e-4, seed, overrides=ov, name=name)
        ox, oy, oz = c.objects[0, 1:4]
        L0 = 4.0 if lj else 9.0
        c.bodies = np.array([[2.0, ox, oy + 10.0, oz, 0.0, 0.0, 0.0, 2.0e-3, L0],
                             [1.5, ox + 1.0, oy + 12.0, oz, 0.0, 0.01, 0.0, 1.0e-3, L0 + 3.0]])
        return c
    if name in ("uncover_mid", "uncover_wide"):
        # a large, fast impactor entering the fluid: 36-80 (mid: radius 10 at
        # 0.2) or 200-350 (wide: radius 16 at 0.4) nodes uncovered behind it
        # in every step, for the resolution of many uncovered nodes at once
        # (LB::findNewActiveObject, src/LB.cpp:846)
        wide = name == "uncover_wide"
        lat, r, vy = ((44, 60, 44), 16.0, -0.4) if wide else ((40, 52, 40), 10.0, -0.2)
        return impact_case(lat, 30.0, 12, (3.0, 3.4), r, 30.0 + r + 1.5, vy, 5.0, 0.8,
                           1.0e-4, seed, overrides={"objWaitTime": "2"}, name=name)
    if name == "units_dyn":
        # a cell-list case in physical units (unitLength 0.5, unitTime 0.02,
        # unitDensity 1000), with boundary0 = 8: every wall is a moving
        # no-slip wall (type 8), as DEM::initializeWalls takes the moving flag
        # of boundary0 for all walls (src/DEM.cpp:430-447)
        lat = impact_case((30, 40, 30), 27.0, 18, (3.0, 3.4), 5.0, 32.0,
                          -0.08, 5.0, 0.8, 1.0e-4, seed,
                          overrides={"objWaitTime": "3", "boundary0": "8"}, name=name)
        return to_physical(lat, 0.5, 0.02, 1000.0)
    raise KeyError(name)
