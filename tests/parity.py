"""Comparison of a GPU state against the oracle's state dump (same keys).

Discrete state (node types, particle flags, solid indices, neighbour lists)
must be identical. Floating-point state is checked twice:
- against the field's own scale: max |a - b| <= rtol * max |b|;
- element by element: |a - b| <= rtol * |b| + ATOL_FRAC * max |b| for every
  element, so that a small entry (a low-density interface node, a small
  torque component) is held to rtol of its own value down to ATOL_FRAC of
  the field's scale.
The reductions over nodes and particles are summed in a different order than
in the reference (everything else rounds identically). A reordered sum of n
terms differs by up to about n * eps * sum |terms|, which for a component
that nearly cancels (a particle's total force: hydrodynamic, contact,
lubrication, gravity and repulsion) is far above eps times the result; the
absolute floor ATOL_FRAC (1e-11 of the field's scale, ten times below the
field-scale tolerance) covers that.
"""
from __future__ import annotations

import numpy as np

LATTICE_FLOAT = ("f", "mass", "visc")
PARTICLE_FLOAT = ("p_x0", "p_x1", "p_w1", "p_FHydro", "p_MHydro", "p_FContact", "p_MContact",
                  "p_FLub", "p_MLub", "p_FRep", "p_FTotal", "p_MTotal", "p_xiw", "p_xio",
                  "p_fluidVolume", "p_SHydro")
OBJECT_FLOAT = ("o_x0", "o_x1", "o_w1", "o_FHydro", "o_MHydro", "o_FContact", "o_FLub",
                "o_FTotal", "b_x0", "b_x1", "b_FSpring", "b_FTotal", "b_L")
TORQUE_FORCE = {"o_MHydro": "o_FHydro", "o_w1": "o_x1", "p_MHydro": "p_FHydro",
                "p_MContact": "p_FContact", "p_MLub": "p_FLub", "p_MTotal": "p_FTotal",
                "p_w1": "p_x1"}
LEVER = 10.0  # lattice units, of the order of the sphere radii
ATOL_FRAC = 1e-11  # element-wise absolute floor, as a fraction of the field's scale
# The per-node viscosity of a non-Newtonian run is a function of the
# non-equilibrium populations f - feq and of the shear rate in a denominator
# (node::computeApparentViscosity, src/node.cpp:113-168): the differences of
# about 1e-16 that reordered reductions leave in the inputs (interface masses,
# particle velocities) are amplified by |f| / |f - feq|, 1e4 to 1e6. It is
# therefore held to 1e-8, while the populations it produces stay at rtol.
FIELD_RTOL = {"visc": 1e-8}


def rel_err(a, b, scale=None):
    a = np.asarray(a, float)
    b = np.asarray(b, float)
    if a.size == 0:
        return 0.0
    s = scale if scale is not None else max(float(np.max(np.abs(b))), 1e-300)
    return float(np.max(np.abs(a - b))) / s


def elem_err(a, b, rtol, scale):
    """Largest |a - b| / (rtol |b| + ATOL_FRAC scale), element-wise; <= 1 passes."""
    a = np.asarray(a, float)
    b = np.asarray(b, float)
    if a.size == 0:
        return 0.0
    tol = rtol * np.abs(b) + ATOL_FRAC * max(scale, 1e-300)
    return float(np.max(np.abs(a - b) / tol))


def compare(gpu: dict, orc: dict, rtol: float = 1e-10, lattice: bool = True,
            fluid_mass: bool = True, elem: bool = True) -> list[str]:
    """fluid_mass=False skips the mass of fluid nodes: between the LB step
    and the free-surface step the GPU already holds updateMass's fluid rule
    (mass = density), which the reference applies in the free-surface step.
    elem=False keeps only the field-scale check (for the mixed form's
    looser tolerances)."""
    bad: list[str] = []
    if lattice:
        for k in ("type", "pflag"):
            if not np.array_equal(gpu[k], orc[k]):
                n = int(np.sum(gpu[k] != orc[k]))
                bad.append(f"{k}: {n} nodes differ")
        if not np.array_equal(gpu["solid"], orc["solid"]):
            bad.append(f"solid: {int(np.sum(gpu['solid'] != orc['solid']))} nodes differ")
        act = (orc["type"] == 0) | (orc["type"] == 3)
        for k in LATTICE_FLOAT:
            if k not in gpu or k not in orc:
                continue
            sel = act if (fluid_mass or k != "mass") else (orc["type"] == 3)
            g = gpu[k][..., sel]
            o = orc[k][..., sel]
            rk = max(rtol, FIELD_RTOL.get(k, 0.0))
            e = rel_err(g, o)
            if not e <= rk:
                bad.append(f"{k}: rel err {e:.3e}")
            if elem:
                q = elem_err(g, o, rk, max(float(np.max(np.abs(o))) if o.size else 0.0, 1e-300))
                if not q <= 1.0:
                    bad.append(f"{k}: element-wise error {q:.3e} of tolerance")
    for k in PARTICLE_FLOAT + OBJECT_FLOAT:
        if k in orc and k in gpu:
            scale = max(float(np.max(np.abs(orc[k]))) if orc[k].size else 0.0, 1e-300)
            # a torque that cancels to ~0 is judged against force x lever arm
            fk = TORQUE_FORCE.get(k)
            if fk and fk in orc and orc[fk].size:
                scale = max(scale, float(np.max(np.abs(orc[fk]))) * LEVER)
            e = rel_err(gpu[k], orc[k], scale)
            if not e <= rtol:
                bad.append(f"{k}: rel err {e:.3e}")
            if elem:
                q = elem_err(gpu[k], orc[k], rtol, scale)
                if not q <= 1.0:
                    bad.append(f"{k}: element-wise error {q:.3e} of tolerance")
    # neighbour lists: the valid slots only (slots past the count are stale)
    gl, ol = gpu["p_list"], orc["p_list"]
    if not np.array_equal(gl[:, 0], ol[:, 0]):
        bad.append("neighbour counts differ")
    else:
        for i in range(len(ol)):
            c = ol[i, 0]
            if not np.array_equal(gl[i, 1:c + 1], ol[i, 1:c + 1]):
                bad.append(f"neighbour list of particle {i} differs")
                break
    e = rel_err(gpu["p_xi"][:, :, 1:], orc["p_xi"][:, :, 1:],
                scale=max(float(np.max(np.abs(orc["p_xi"][:, :, 1:]))), 1e-12))
    if not e <= rtol:
        bad.append(f"p_xi: rel err {e:.3e}")
    return bad
