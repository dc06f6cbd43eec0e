"""ctypes binding of the oracle (test infrastructure, never the product).

Only tests/, the smoke check and the CPU-baseline leg of bench.py use this.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

from geoflac_gb300.capi import GfClock, GfLayout, GfParams

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")

_lib = None


def build() -> str:
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB_PATH


def load():
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        build()
    lib = C.CDLL(LIB_PATH)
    P, K, L = C.POINTER(GfParams), C.POINTER(GfClock), C.POINTER(GfLayout)
    for name in ("fl_therm", "change_phase", "fl_rheol", "fl_node", "fl_move", "rmasses", "dt_mass",
                 "init_visc", "marker2elem", "finish_setflac", "flac", "bar2euler", "lpeuler2bar", "remesh",
                 "remesh_event", "restart_tail"):
        f = getattr(lib, "or_" + name)
        f.restype = C.c_int
        f.argtypes = [P, K, L]
    lib.or_step.restype = C.c_int
    lib.or_step.argtypes = [P, K, L, C.c_int]
    lib.or_itest_mesh.restype = C.c_int
    lib.or_itest_mesh.argtypes = [P, K, L, C.POINTER(C.c_double)]
    lib.or_read_params.restype = C.c_int
    lib.or_read_params.argtypes = [C.c_char_p, P]
    lib.or_setflac.restype = C.c_int
    lib.or_setflac.argtypes = [P, K, L]
    lib.or_set_threads.argtypes = [C.c_int]
    lib.or_set_threads.restype = None
    _lib = lib
    return lib


def read_params(path: str, markers_per_side: int = 3, eclogite_rule: int = 0,
                therm_sweeps: int = 0) -> GfParams:
    """The oracle's own read_params of an .inp file."""
    lib = load()
    p = GfParams()
    p.markers_per_side = markers_per_side
    p.eclogite_rule = eclogite_rule
    p.therm_sweeps = therm_sweeps
    rc = lib.or_read_params(path.encode(), C.byref(p))
    if rc:
        raise RuntimeError(f"oracle read_params({path}): status {rc}")
    return p


def new_state(path: str, markers_per_side: int = 3, eclogite_rule: int = 0, therm_sweeps: int = 0):
    """Start-up state (params, clock, host arrays) built by the oracle alone:
    its read_params and setflac chain (init_cord .. init_bc), without the
    product's library.  or_finish_setflac (Oracle.finish_setflac) completes
    it with rmasses, init_visc and dt_mass."""
    from geoflac_gb300.capi import HostState

    p = read_params(path, markers_per_side, eclogite_rule, therm_sweeps)
    s = HostState(p)
    c = GfClock()
    rc = load().or_setflac(C.byref(p), C.byref(c), C.byref(s.layout))
    if rc:
        raise RuntimeError(f"oracle setflac: status {rc}")
    return p, c, s


class Oracle:
    """Runs the oracle's routines on one host state (params, clock, arrays)."""

    def __init__(self, params: GfParams, clock: GfClock, state, threads: int = 1):
        self.lib = load()
        self.p = params
        self.c = clock
        self.s = state
        self.lib.or_set_threads(threads)

    def _call(self, name, *extra):
        rc = getattr(self.lib, "or_" + name)(C.byref(self.p), C.byref(self.c), C.byref(self.s.layout), *extra)
        if rc:
            raise RuntimeError(f"oracle {name}: status {rc}")
        return rc

    def __getattr__(self, name):
        if name in ("fl_therm", "change_phase", "fl_rheol", "fl_node", "fl_move", "rmasses", "dt_mass",
                    "init_visc", "marker2elem", "finish_setflac", "flac", "bar2euler", "lpeuler2bar", "remesh",
                    "remesh_event", "restart_tail"):
            return lambda: self._call(name)
        raise AttributeError(name)

    def step(self, n: int):
        return self._call("step", C.c_int(n))

    def itest_mesh(self) -> float:
        a = C.c_double()
        self._call("itest_mesh", C.byref(a))
        return a.value
