"""Python binding of the liblbdem.so C ABI (include/lbdem.h), via ctypes.

This is the reference-facing host interface in Python: a ``Solver`` object
whose methods mirror the reference's step entry points
(``DEM::discreteElementStep``, ``LB::latticeBoltzmannCouplingStep``,
``LB::latticeBolzmannStep``, ``LB::latticeBoltzmannFreeSurfaceStep``,
goCycle). All compute happens in the CUDA library; if the library or a GPU
is missing, construction raises instead of falling back to anything else.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from lbdem_types import (  # noqa: F401
    Config, Info, JobResult, ObjectIn, ObjectView, Options, ParticleIn, ParticleView,
    Profile, ServerOptions, _P, _PI)

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liblbdem.so")

PLAIN_FP64 = 0
MIXED = 1
NOALLOC_MAX_NODES = 16384  # LBDEM_NOALLOC_MAX_NODES in include/lbdem.h
DEBUG_NO_LATTICE_COPIES = 1  # LBDEM_DEBUG_NO_LATTICE_COPIES

ERR_NONFINITE = 5      # LBDEM_ERR_NONFINITE
ERR_OVERFLOW = 6       # LBDEM_ERR_OVERFLOW
ERR_DEVICE_STATE = 7   # LBDEM_ERR_DEVICE_STATE
ERRORS = {
    0: "ok", 1: "invalid argument", 2: "CUDA error", 3: "out of device memory",
    4: "input error", 5: "non-finite state", 6: "list overflow",
    7: "device-side error", 8: "no CUDA device",
}


_lib = None


def load_library(path: str | None = None) -> C.CDLL:
    """Load liblbdem.so (built in-tree by __graft_entry__.build())."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise RuntimeError(f"liblbdem.so not built: {p} (run __graft_entry__.build())")
    lib = C.CDLL(p)
    c_ctx = C.c_void_p
    sig = {
        "lbdem_config_defaults": ([C.POINTER(Config)], C.c_int),
        "lbdem_config_load": ([C.c_char_p, C.c_char_p, C.c_int, C.POINTER(C.c_char_p),
                               C.POINTER(Config), C.c_char_p, C.c_size_t], C.c_int),
        "lbdem_config_release": ([C.POINTER(Config)], None),
        "lbdem_create": ([C.POINTER(Config), C.POINTER(Options), C.POINTER(c_ctx)], C.c_int),
        "lbdem_destroy": ([c_ctx], None),
        "lbdem_last_error": ([c_ctx], C.c_char_p),
        "lbdem_set_stream": ([c_ctx, C.c_void_p], C.c_int),
        "lbdem_dem_step": ([c_ctx], C.c_int),
        "lbdem_coupling_step": ([c_ctx], C.c_int),
        "lbdem_lb_step": ([c_ctx], C.c_int),
        "lbdem_free_surface_step": ([c_ctx], C.c_int),
        "lbdem_cycle": ([c_ctx, C.c_int32], C.c_int),
        "lbdem_sync": ([c_ctx], C.c_int),
        "lbdem_get_info": ([c_ctx, C.POINTER(Info)], C.c_int),
        "lbdem_download_lattice": ([c_ctx, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                    C.c_void_p, C.c_void_p, C.c_void_p], C.c_int),
        "lbdem_download_particles": ([c_ctx, C.POINTER(ParticleView)], C.c_int),
        "lbdem_download_viscosity": ([c_ctx, C.c_void_p], C.c_int),
        "lbdem_download_bodies": ([c_ctx, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                   C.c_void_p], C.c_int),
        "lbdem_download_objects": ([c_ctx, C.POINTER(ObjectView)], C.c_int),
        "lbdem_download_walls": ([c_ctx, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p],
                                 C.c_int),
        "lbdem_mass_summary": ([c_ctx, C.POINTER(C.c_double), C.POINTER(C.c_int64),
                                C.POINTER(C.c_int64)], C.c_int),
        "lbdem_mass_total": ([c_ctx, C.POINTER(C.c_double)], C.c_int),
        "lbdem_profile_enable": ([c_ctx, C.c_int], C.c_int),
        "lbdem_profile_read": ([c_ctx, C.POINTER(Profile), C.c_int], C.c_int),
        "lbdem_estimate_device_bytes": ([C.POINTER(Config), C.c_int32, C.POINTER(C.c_int64)],
                                        C.c_int),
        "lbdem_server_create": ([C.POINTER(ServerOptions), C.POINTER(C.c_void_p)], C.c_int),
        "lbdem_server_submit": ([C.c_void_p, C.POINTER(Config), C.c_int32,
                                 C.POINTER(C.c_int64)], C.c_int),
        "lbdem_server_poll": ([C.c_void_p, C.c_double, C.POINTER(JobResult), C.c_int32,
                               C.POINTER(C.c_int32)], C.c_int),
        "lbdem_server_status": ([C.c_void_p, C.POINTER(C.c_int32), C.POINTER(C.c_int32),
                                 C.POINTER(C.c_int32), C.POINTER(C.c_int64)], C.c_int),
        "lbdem_server_last_error": ([C.c_void_p], C.c_char_p),
        "lbdem_server_destroy": ([C.c_void_p], None),
        "lbdem_server_tune": ([C.POINTER(ServerOptions), C.POINTER(C.POINTER(Config)), C.c_int32,
                               C.c_int32, C.POINTER(C.c_double)], C.c_int),
        "lbdem_download_nodes_noalloc": ([c_ctx, C.c_int64, C.c_int64, C.c_void_p, C.c_void_p],
                                         C.c_int),
        "lbdem_device_allocations": ([], C.c_int64),
        "lbdem_checkpoint": ([c_ctx, C.c_char_p], C.c_int),
        "lbdem_export_recycle_fluid": ([c_ctx, C.c_char_p], C.c_int),
        "lbdem_output_open": ([c_ctx, C.c_char_p, C.c_double], C.c_int),
        "lbdem_output_close": ([c_ctx], C.c_int),
        "lbdem_output_recycle": ([c_ctx, C.c_double, C.c_double], C.c_int),
        "lbdem_restore": ([c_ctx, C.c_char_p], C.c_int),
    }
    for name, (args, res) in sig.items():
        fn = getattr(lib, name)  # a missing entry point is a build error
        fn.argtypes = args
        fn.restype = res
    if path is None:
        _lib = lib
    return lib


class LoadedConfig:
    """A parsed case: owns the Config and its arrays (released on close)."""

    def __init__(self, cfg_path: str, input_dir: str | None = None,
                 overrides: dict | None = None):
        self.lib = load_library()
        self.cfg = Config()
        argv = []
        for k, v in (overrides or {}).items():
            argv += [f"-{k}".encode(), str(v).encode()]
        arr = (C.c_char_p * max(1, len(argv)))(*argv)
        err = C.create_string_buffer(512)
        if input_dir is None:
            input_dir = os.path.join(os.path.dirname(os.path.abspath(cfg_path)), "input")
        rc = self.lib.lbdem_config_load(cfg_path.encode(), input_dir.encode(), len(argv),
                                        arr, C.byref(self.cfg), err, 512)
        if rc != 0:
            raise RuntimeError(f"lbdem_config_load: {ERRORS.get(rc, rc)}: {err.value.decode()}")

    def close(self):
        if self.cfg is not None:
            self.lib.lbdem_config_release(C.byref(self.cfg))
            self.cfg = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


class Solver:
    """One impact run on the GPU (wraps an lbdem_ctx)."""

    def __init__(self, config: LoadedConfig, precision: int = PLAIN_FP64,
                 device: int = 0, check_every: int = 0, async_init: bool = False,
                 debug_flags: int = 0):
        self.lib = load_library()
        self.ctx = C.c_void_p()
        opt = Options(precision=precision, device=device, check_every=check_every,
                      async_init=1 if async_init else 0, debug_flags=debug_flags)
        rc = self.lib.lbdem_create(C.byref(config.cfg), C.byref(opt), C.byref(self.ctx))
        if rc != 0:
            msg = self.lib.lbdem_last_error(self.ctx).decode() if self.ctx else ""
            if self.ctx:
                self.lib.lbdem_destroy(self.ctx)
                self.ctx = None
            raise RuntimeError(f"lbdem_create: {ERRORS.get(rc, rc)}: {msg}")
        self.info = self.get_info()
        self.n_bodies = int(config.cfg.n_bodies)

    def _check(self, rc: int, what: str):
        if rc != 0:
            raise RuntimeError(f"{what}: {ERRORS.get(rc, rc)}: "
                               f"{self.lib.lbdem_last_error(self.ctx).decode()}")

    def close(self):
        if self.ctx:
            self.lib.lbdem_destroy(self.ctx)
            self.ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # --- step entry points -------------------------------------------------
    def dem_step(self):
        self._check(self.lib.lbdem_dem_step(self.ctx), "dem_step")

    def coupling_step(self):
        self._check(self.lib.lbdem_coupling_step(self.ctx), "coupling_step")

    def lb_step(self):
        self._check(self.lib.lbdem_lb_step(self.ctx), "lb_step")

    def free_surface_step(self):
        self._check(self.lib.lbdem_free_surface_step(self.ctx), "free_surface_step")

    def cycle(self, n: int = 1):
        self._check(self.lib.lbdem_cycle(self.ctx, n), "cycle")

    def sync(self):
        self._check(self.lib.lbdem_sync(self.ctx), "sync")

    def set_stream(self, handle: int | None):
        self._check(self.lib.lbdem_set_stream(self.ctx, C.c_void_p(handle or 0)), "set_stream")

    # --- state ---------------------------------------------------------------
    def get_info(self) -> Info:
        info = Info()
        self._check(self.lib.lbdem_get_info(self.ctx, C.byref(info)), "get_info")
        return info

    def lattice(self) -> dict:
        N = int(self.info.nodes)
        out = {
            "type": np.zeros(N, np.uint8), "pflag": np.zeros(N, np.uint8),
            "solid": np.zeros(N, np.int32), "n": np.zeros(N), "u": np.zeros(3 * N),
            "mass": np.zeros(N), "f": np.zeros(19 * N),
        }
        self._check(self.lib.lbdem_download_lattice(
            self.ctx, _ptr(out["type"]), _ptr(out["pflag"]), _ptr(out["solid"]),
            _ptr(out["n"]), _ptr(out["u"]), _ptr(out["mass"]), _ptr(out["f"])),
            "download_lattice")
        u = out.pop("u").reshape(3, N)
        out["ux"], out["uy"], out["uz"] = u[0], u[1], u[2]
        out["f"] = out["f"].reshape(19, N)
        return out

    def bodies(self) -> dict:
        """Body state: b_x0, b_x1, b_FSpring, b_FTotal [B][3], b_L [B]."""
        B = self.n_bodies
        out = {k: np.zeros((B, 3)) for k in ("b_x0", "b_x1", "b_FSpring", "b_FTotal")}
        out["b_L"] = np.zeros(B)
        self._check(self.lib.lbdem_download_bodies(
            self.ctx, _ptr(out["b_x0"]), _ptr(out["b_x1"]), _ptr(out["b_FSpring"]),
            _ptr(out["b_FTotal"]), _ptr(out["b_L"])), "download_bodies")
        return out

    def viscosity(self) -> np.ndarray:
        """Per-node viscosity (lattice units), 0 at non-active nodes."""
        v = np.zeros(int(self.info.nodes))
        self._check(self.lib.lbdem_download_viscosity(self.ctx, _ptr(v)), "download_viscosity")
        return v

    def particles(self) -> dict:
        P = int(self.info.n_particles)
        names3 = ["x0", "x1", "w1", "FHydro", "MHydro", "FContact", "MContact", "FLub",
                  "MLub", "FRep", "FTotal", "MTotal", "xiw", "xio"]
        arr = {k: np.zeros((P, 3)) for k in names3}
        arr["fluidVolume"] = np.zeros(P)
        arr["SHydro"] = np.zeros((P, 9))
        arr["list"] = np.zeros((P, 50), np.int32)
        arr["xi"] = np.zeros((P, 3, 50))
        v = ParticleView()
        for k, a in arr.items():
            if k == "list":
                v.list = a.ctypes.data_as(_PI)
            else:
                setattr(v, k, a.ctypes.data_as(_P))
        self._check(self.lib.lbdem_download_particles(self.ctx, C.byref(v)),
                    "download_particles")
        return {"p_" + k: a for k, a in arr.items()}

    _OBJECT_FIELDS = ("x0", "x1", "w1", "FHydro", "MHydro", "FContact", "MContact", "FLub",
                      "MLub", "FTotal")

    def objects(self) -> dict:
        """lbdem_download_objects: the impactors' state, fresh arrays of shape
        (n_objects, 3) per field. The host buffer and its view are made once
        per solver (the call is cheap enough for a read-back every step)."""
        if getattr(self, "_obj_view", None) is None:
            O = int(self.info.n_objects)
            self._obj_buf = np.zeros((len(self._OBJECT_FIELDS), O, 3))
            self._obj_view = ObjectView(**{k: self._obj_buf[i].ctypes.data_as(_P)
                                           for i, k in enumerate(self._OBJECT_FIELDS)})
        self._check(self.lib.lbdem_download_objects(self.ctx, C.byref(self._obj_view)),
                    "download_objects")
        return {"o_" + k: self._obj_buf[i].copy() for i, k in enumerate(self._OBJECT_FIELDS)}

    def walls(self) -> dict:
        W = int(self.info.n_walls)
        arr = {k: np.zeros((W, 3)) for k in ("FHydro", "FContact", "FLub", "FTotal")}
        self._check(self.lib.lbdem_download_walls(
            self.ctx, *[_ptr(arr[k]) for k in ("FHydro", "FContact", "FLub", "FTotal")]),
            "download_walls")
        return {"w_" + k: a for k, a in arr.items()}

    def state(self) -> dict:
        """Everything, keyed like the oracle's state dumps."""
        d = {}
        d.update(self.lattice())
        d["visc"] = self.viscosity()
        d.update(self.particles())
        d.update(self.objects())
        d.update(self.walls())
        if self.n_bodies:
            d.update(self.bodies())
        info = self.get_info()
        d["step"] = np.array([info.time_step])
        d["demTime"] = np.array([info.dem_time])
        d["demTimeStep"] = np.array([info.dem_step])
        return d

    def profile_enable(self, on: bool = True):
        self._check(self.lib.lbdem_profile_enable(self.ctx, 1 if on else 0), "profile_enable")

    def profile_read(self, reset: bool = True) -> Profile:
        p = Profile()
        self._check(self.lib.lbdem_profile_read(self.ctx, C.byref(p), 1 if reset else 0),
                    "profile_read")
        return p

    def mass_summary(self):
        m = C.c_double()
        ni = C.c_int64()
        na = C.c_int64()
        self._check(self.lib.lbdem_mass_summary(self.ctx, C.byref(m), C.byref(ni), C.byref(na)),
                    "mass_summary")
        return m.value, ni.value, na.value

    def mass_total(self) -> float:
        """Mass of every active node, those inside particles included."""
        m = C.c_double()
        self._check(self.lib.lbdem_mass_total(self.ctx, C.byref(m)), "mass_total")
        return m.value

    def checkpoint(self, path) -> None:
        """Write a full-precision snapshot of the run (lbdem_checkpoint)."""
        self._check(self.lib.lbdem_checkpoint(self.ctx, os.fsencode(path)), "checkpoint")

    def restore(self, path) -> None:
        """Replace this run's state with a snapshot of a run of the same
        configuration and form (lbdem_restore)."""
        self._check(self.lib.lbdem_restore(self.ctx, os.fsencode(path)), "restore")

    def export_recycle_fluid(self, path) -> None:
        """Write the reference's fluid recycle file of the current state."""
        self._check(self.lib.lbdem_export_recycle_fluid(self.ctx, os.fsencode(path)),
                    "export_recycle_fluid")

    def output_open(self, directory, screen_exp_time: float) -> None:
        """Write the reference's screen-phase files into `directory` from now
        on (lbdem_output_open)."""
        self._check(self.lib.lbdem_output_open(self.ctx, os.fsencode(directory),
                                               float(screen_exp_time)), "output_open")

    def output_close(self) -> None:
        self._check(self.lib.lbdem_output_close(self.ctx), "output_close")

    def nodes_noalloc(self, first: int, count: int):
        """Populations [19, count] and masses [count] of nodes first ..
        first+count-1 through lbdem_download_nodes_noalloc (no device
        allocation; at most NOALLOC_MAX_NODES nodes per call)."""
        f = np.zeros((19, max(count, 0)))
        mass = np.zeros(max(count, 0))
        self._check(self.lib.lbdem_download_nodes_noalloc(
            self.ctx, int(first), int(count), f.ctypes.data_as(C.c_void_p),
            mass.ctypes.data_as(C.c_void_p)), "download_nodes_noalloc")
        return f, mass


def device_allocations() -> int:
    """Device allocations the library has made in this process so far
    (lbdem_device_allocations)."""
    return int(load_library().lbdem_device_allocations())


def estimate_device_bytes(cfg: "LoadedConfig", precision: int = PLAIN_FP64) -> int:
    """Device bytes a run of this configuration allocates (lbdem_create)."""
    lib = load_library()
    b = C.c_int64()
    rc = lib.lbdem_estimate_device_bytes(C.byref(cfg.cfg), precision, C.byref(b))
    if rc:
        raise RuntimeError(f"lbdem_estimate_device_bytes: {ERRORS.get(rc, rc)}")
    return b.value


class Server:
    """Many impact runs resident on one GPU (lbdem_server_*): jobs queue in
    submission order, are admitted while their device footprint fits the
    budget, and advance by slices of goCycles on their own streams; with
    batch_runs > 0 runs in their steady cycle share launches in groups."""

    def __init__(self, precision=PLAIN_FP64, device=0, max_active=16, slice_cycles=25,
                 device_budget_bytes=0, batch_runs=0, chunks_per_block=0):
        self.lib = load_library()
        o = ServerOptions(device=device, precision=precision, max_active=max_active,
                          slice_cycles=slice_cycles, device_budget_bytes=device_budget_bytes,
                          batch_runs=int(batch_runs),
                          chunks_per_block=int(chunks_per_block))
        h = C.c_void_p()
        rc = self.lib.lbdem_server_create(C.byref(o), C.byref(h))
        if rc:
            raise RuntimeError(f"lbdem_server_create: {ERRORS.get(rc, rc)}")
        self.h = h

    def submit(self, cfg: "LoadedConfig", cycles: int) -> int:
        jid = C.c_int64()
        rc = self.lib.lbdem_server_submit(self.h, C.byref(cfg.cfg), int(cycles), C.byref(jid))
        if rc:
            raise RuntimeError(f"lbdem_server_submit: {ERRORS.get(rc, rc)}: "
                               f"{self.lib.lbdem_server_last_error(self.h).decode()}")
        return jid.value

    def poll(self, wait_seconds: float = 0.0, max_out: int = 64) -> list:
        buf = (JobResult * max_out)()
        n = C.c_int32()
        rc = self.lib.lbdem_server_poll(self.h, float(wait_seconds), buf, max_out, C.byref(n))
        if rc:
            raise RuntimeError(f"lbdem_server_poll: {ERRORS.get(rc, rc)}")
        out = []
        for r in buf[:n.value]:
            out.append({"job_id": r.job_id, "status": r.status, "cycles": r.cycles,
                        "submit_time": r.submit_time, "start_time": r.start_time,
                        "end_time": r.end_time, "impactor_x0": list(r.impactor_x0),
                        "impactor_x1": list(r.impactor_x1), "fluid_mass": r.fluid_mass,
                        "active_node_updates": r.active_node_updates,
                        "device_bytes": r.device_bytes,
                        "batched_cycles": r.batched_cycles})
        return out

    def status(self) -> dict:
        q, r, u = C.c_int32(), C.c_int32(), C.c_int32()
        b = C.c_int64()
        self.lib.lbdem_server_status(self.h, C.byref(q), C.byref(r), C.byref(u), C.byref(b))
        return {"queued": q.value, "running": r.value, "unread": u.value,
                "device_bytes": b.value}

    def drain(self, timeout: float = 600.0) -> list:
        """Poll until every submitted job has finished."""
        import time
        res, t0 = [], time.perf_counter()
        while time.perf_counter() - t0 < timeout:
            res += self.poll(0.05)
            st = self.status()
            if st["queued"] == 0 and st["running"] == 0 and st["unread"] == 0:
                return res
        raise RuntimeError("server drain timed out")

    def last_error(self) -> str:
        """lbdem_server_last_error: the description of the last failed job or
        call of this server ("" if none failed)."""
        return self.lib.lbdem_server_last_error(self.h).decode() if self.h else ""

    def close(self):
        if self.h:
            self.lib.lbdem_server_destroy(self.h)
            self.h = None


def tune_server(cfgs, cycles=40, precision=MIXED, device=0, max_active=0, slice_cycles=24):
    """lbdem_server_tune: the fastest (batch_runs, chunks_per_block) for these
    sample runs; returns (batch_runs, chunks_per_block, seconds)."""
    lib = load_library()
    o = ServerOptions(device=device, precision=precision,
                      max_active=max_active or len(cfgs), slice_cycles=slice_cycles)
    arr = (C.POINTER(Config) * len(cfgs))(*[C.pointer(c.cfg) for c in cfgs])
    t = C.c_double()
    rc = lib.lbdem_server_tune(C.byref(o), arr, len(cfgs), int(cycles), C.byref(t))
    if rc:
        raise RuntimeError(f"lbdem_server_tune: {ERRORS.get(rc, rc)}: "
                           f"{lib.lbdem_server_last_error(None).decode()}")
    return o.batch_runs, o.chunks_per_block, t.value

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
