"""ctypes access to the CPU restatement (oracle/_build/liblbdem_oracle.so).

Test infrastructure: used only by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py, as the checker / baseline.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ORACLE_SO = os.path.join(REPO, "oracle", "_build", "liblbdem_oracle.so")

_lib = None


def build_oracle() -> str:
    subprocess.run(["make", "-s", "-C", os.path.join(REPO, "oracle"), "restate"], check=True)
    return ORACLE_SO


def load() -> C.CDLL:
    global _lib
    if _lib is None:
        if not os.path.exists(ORACLE_SO):
            build_oracle()
        lib = C.CDLL(ORACLE_SO)
        v = C.c_void_p
        lib.oracle_create.argtypes = [C.c_void_p, C.POINTER(v)]
        lib.oracle_destroy.argtypes = [v]
        lib.oracle_last_error.argtypes = [v]
        lib.oracle_last_error.restype = C.c_char_p
        for name in ("oracle_dem_step", "oracle_coupling_step", "oracle_lb_step",
                     "oracle_free_surface_step"):
            getattr(lib, name).argtypes = [v]
        lib.oracle_cycle.argtypes = [v, C.c_int32]
        lib.oracle_dump.argtypes = [v, C.c_char_p]
        lib.oracle_counters.argtypes = [v, C.POINTER(C.c_int64)]
        lib.oracle_dem_time.argtypes = [v]
        lib.oracle_dem_time.restype = C.c_double
        lib.oracle_object0.argtypes = [v, C.POINTER(C.c_double)]
        lib.oracle_set_threads.argtypes = [C.c_int32]
        lib.oracle_max_threads.argtypes = []
        _lib = lib
    return _lib


def set_threads(n: int) -> None:
    """OpenMP threads of the oracle's per-node loops (results do not change)."""
    load().oracle_set_threads(int(n))


def max_threads() -> int:
    return int(load().oracle_max_threads())


class Oracle:
    def __init__(self, config):
        """config: a parsed case with a ``cfg`` lbdem_config structure
        (caseio.CaseConfig, or lbdem.LoadedConfig)."""
        self.lib = load()
        self.ctx = C.c_void_p()
        rc = self.lib.oracle_create(C.byref(config.cfg), C.byref(self.ctx))
        if rc != 0:
            msg = self.lib.oracle_last_error(self.ctx).decode()
            self.close()
            raise RuntimeError(f"oracle_create failed ({rc}): {msg}")

    def _chk(self, rc, what):
        if rc != 0:
            raise RuntimeError(f"{what} failed ({rc}): "
                               f"{self.lib.oracle_last_error(self.ctx).decode()}")

    def cycle(self, n=1):
        self._chk(self.lib.oracle_cycle(self.ctx, n), "oracle_cycle")

    def dem_step(self):
        self._chk(self.lib.oracle_dem_step(self.ctx), "oracle_dem_step")

    def coupling_step(self):
        self._chk(self.lib.oracle_coupling_step(self.ctx), "oracle_coupling_step")

    def lb_step(self):
        self._chk(self.lib.oracle_lb_step(self.ctx), "oracle_lb_step")

    def free_surface_step(self):
        self._chk(self.lib.oracle_free_surface_step(self.ctx), "oracle_free_surface_step")

    def dump(self, path):
        self.lib.oracle_dump(self.ctx, path.encode())

    def state(self, tmpdir):
        from dumpio import read_dump
        p = os.path.join(tmpdir, "oracle_state.bin")
        self.dump(p)
        return read_dump(p)

    def counters(self):
        a = (C.c_int64 * 5)()
        self.lib.oracle_counters(self.ctx, a)
        return list(a)

    def object0(self):
        a = (C.c_double * 6)()
        self.lib.oracle_object0(self.ctx, a)
        return list(a)

    def close(self):
        if self.ctx:
            self.lib.oracle_destroy(self.ctx)
            self.ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
