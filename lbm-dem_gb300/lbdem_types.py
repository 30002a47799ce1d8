"""ctypes layouts of the structures of the liblbdem.so C ABI (include/lbdem.h).

Plain data layouts only: importing this module loads no library. They are
shared by the ctypes binding (lbdem.py) and by host-side readers that fill
an lbdem_config without the library.
"""
from __future__ import annotations

import ctypes as C

PLAIN_FP64 = 0
MIXED = 1


class ParticleIn(C.Structure):
    _fields_ = [("r", C.c_double), ("x", C.c_double * 3), ("v", C.c_double * 3),
                ("w", C.c_double * 3), ("size", C.c_int32), ("index", C.c_int32)]


class ObjectIn(C.Structure):
    _fields_ = [("index", C.c_int32), ("r", C.c_double), ("x", C.c_double * 3),
                ("v", C.c_double * 3)]


class BodyIn(C.Structure):
    _fields_ = [("index", C.c_int32), ("r", C.c_double), ("x", C.c_double * 3),
                ("v", C.c_double * 3), ("k", C.c_double), ("L0", C.c_double)]


class Config(C.Structure):
    _fields_ = [
        ("demSolve", C.c_int32), ("lbSolve", C.c_int32),
        ("freeSurfaceSolve", C.c_int32), ("forceFieldSolve", C.c_int32),
        ("demInitialRepeat", C.c_double), ("lbmInitialRepeat", C.c_int32),
        ("maxTime", C.c_double), ("maximumTimeSteps", C.c_int32),
        ("screenExpTime", C.c_double), ("fluidExpTime", C.c_double),
        ("fluidLagrangianExpTime", C.c_double), ("partExpTime", C.c_double),
        ("partRecycleExpTime", C.c_double), ("fluidRecycleExpTime", C.c_double),
        ("unitLength", C.c_double), ("unitTime", C.c_double),
        ("unitDensity", C.c_double),
        ("lbSizeX", C.c_double), ("lbSizeY", C.c_double), ("lbSizeZ", C.c_double),
        ("lbRestart", C.c_int32), ("lbTopography", C.c_int32),
        ("initVelocity", C.c_double * 3), ("lbF", C.c_double * 3),
        ("lbRot", C.c_double * 3), ("lbRotCenter", C.c_double * 3),
        ("boundary", C.c_int32 * 6), ("slipCoefficient", C.c_double),
        ("fluidHeight", C.c_double), ("rheologyNewtonian", C.c_int32),
        ("initVisc", C.c_double), ("turbulenceSolve", C.c_int32),
        ("turbConst", C.c_double),
        ("density", C.c_double), ("objectDensity", C.c_double),
        ("bodyDensity", C.c_double), ("linearStiff", C.c_double),
        ("frictionCoefPart", C.c_double), ("lubNormal", C.c_double),
        ("lubTangential", C.c_double), ("lubRotation", C.c_double),
        ("lubCutoff", C.c_double), ("kinVisc", C.c_double),
        ("debyeLength", C.c_double), ("electroForce", C.c_double),
        ("objWaitTime", C.c_int32), ("intervalTime", C.c_int32),
        ("springDamp", C.c_double), ("epsilon", C.c_double),
        ("nonLinType", C.c_int32), ("k13", C.c_double), ("scale", C.c_double),
        ("n_particles", C.c_int32), ("particles", C.POINTER(ParticleIn)),
        ("n_objects", C.c_int32), ("objects", C.POINTER(ObjectIn)),
        ("n_bodies", C.c_int32), ("lbRestartFile", C.c_char_p),
        ("rheologyModel", C.c_int32), ("plasticVisc", C.c_double),
        ("yieldStress", C.c_double), ("frictionCoefFluid", C.c_double),
        ("voellmyConstant", C.c_double), ("bodies", C.POINTER(BodyIn)),
    ]


class Options(C.Structure):
    _fields_ = [("precision", C.c_int32), ("device", C.c_int32),
                ("check_every", C.c_int32), ("chunks_per_block", C.c_int32),
                ("async_init", C.c_int32), ("debug_flags", C.c_int32),
                ("reserved", C.c_int32 * 2)]


class Info(C.Structure):
    _fields_ = [("lb_size", C.c_int32 * 3), ("nodes", C.c_int64),
                ("n_particles", C.c_int32), ("n_objects", C.c_int32),
                ("n_walls", C.c_int32), ("precision", C.c_int32),
                ("time_step", C.c_int64), ("dem_step", C.c_int64),
                ("dem_time", C.c_double), ("unit_length", C.c_double),
                ("unit_time", C.c_double), ("unit_density", C.c_double),
                ("device_bytes", C.c_int64), ("neighbour_rebuilds", C.c_int32),
                ("reserved", C.c_int32 * 7)]


class Profile(C.Structure):
    _fields_ = [("lb_kernel_ms", C.c_double), ("lb_kernel_launches", C.c_int64),
                ("kernel_launches", C.c_int64), ("active_node_updates", C.c_int64),
                ("phase_ms", C.c_double * 4)]


class ServerOptions(C.Structure):
    _fields_ = [("device", C.c_int32), ("precision", C.c_int32), ("max_active", C.c_int32),
                ("slice_cycles", C.c_int32), ("device_budget_bytes", C.c_int64),
                ("batch_runs", C.c_int32), ("chunks_per_block", C.c_int32),
                ("reserved", C.c_int32 * 4)]


class JobResult(C.Structure):
    _fields_ = [("job_id", C.c_int64), ("status", C.c_int32), ("cycles", C.c_int32),
                ("submit_time", C.c_double), ("start_time", C.c_double),
                ("end_time", C.c_double), ("impactor_x0", C.c_double * 3),
                ("impactor_x1", C.c_double * 3), ("fluid_mass", C.c_double),
                ("active_node_updates", C.c_int64), ("device_bytes", C.c_int64),
                ("batched_cycles", C.c_int32), ("reserved", C.c_int32)]


_P = C.POINTER(C.c_double)
_PI = C.POINTER(C.c_int32)


class ParticleView(C.Structure):
    _fields_ = [(k, _P) for k in (
        "x0", "x1", "w1", "FHydro", "MHydro", "FContact", "MContact", "FLub",
        "MLub", "FRep", "FTotal", "MTotal", "fluidVolume", "SHydro")] + [
        ("list", _PI), ("xi", _P), ("xiw", _P), ("xio", _P)]


class ObjectView(C.Structure):
    _fields_ = [(k, _P) for k in (
        "x0", "x1", "w1", "FHydro", "MHydro", "FContact", "MContact", "FLub",
        "MLub", "FTotal")]
