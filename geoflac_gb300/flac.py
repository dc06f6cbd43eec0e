"""Host-side driver of the GB300 FLAC step.

``Flac`` mirrors the reference's main program (src/par.f90) and time step
(src/flac.f90): its methods carry the names of the reference's per-step
subroutines (``fl_therm``, ``change_phase``, ``fl_rheol``, ``fl_node``,
``fl_move``, ``rmasses``, ``dt_mass``) and each one runs that routine's
CUDA kernels through the C-ABI, raising ``GfError`` with the reference's stop
code where the reference would stop.  The model state lives on the GPU; the
host arrays (``self.state``, reference layout) are refreshed by
``download()``.
"""
from __future__ import annotations

import ctypes as C
from typing import Optional

from . import capi
from .capi import GfClock, GfParams, HostState, check

MODES = {"fp64": capi.MODE_FP64, "mixed": capi.MODE_MIXED}


class Flac:
    def __init__(self, params: GfParams, clock: GfClock, state: HostState, mode: str = "fp64",
                 finish_setflac: bool = True):
        self.lib = capi.load_library()
        self.params = params
        self.clock = clock
        self.state = state
        self.mode = mode
        self.ctx = C.c_void_p()
        check(self.lib.gf_create(C.byref(self.ctx), C.byref(params), C.byref(state.layout), MODES[mode]),
              "gf_create")
        self.upload()
        if finish_setflac:
            check(self.lib.gf_finish_setflac(self.ctx), "gf_finish_setflac")
            self.download(0)

    # ---- construction -------------------------------------------------
    @classmethod
    def from_inp(cls, path: str, mode: str = "fp64", markers_per_side: int = 3, eclogite_rule: int = 0,
                 therm_sweeps: int = 0) -> "Flac":
        """read_params + setflac (src/par.f90:28-62) for a new start."""
        p = capi.read_params(path, markers_per_side, eclogite_rule, therm_sweeps)
        s = HostState(p)
        c = capi.setflac_host(p, s)
        return cls(p, c, s, mode)

    @classmethod
    def restart(cls, inp_path: str, directory: str = ".", mode: str = "fp64", markers_per_side: int = 3,
                eclogite_rule: int = 0, therm_sweeps: int = 0) -> "Flac":
        """read_params + rsflac (src/par.f90:28-45) for a restart from the
        `*.rs` files in `directory`."""
        p = capi.read_params(inp_path, markers_per_side, eclogite_rule, therm_sweeps)
        s = HostState(p)
        c = capi.setflac_host(p, s)
        g = cls(p, c, s, mode, finish_setflac=False)
        g.rsflac(directory)
        return g

    # ---- output and restart files (src/outflac.f90, outmarker.f90,
    # saveflac.f90, rsflac.f90) ------------------------------------------
    def outflac(self, directory: str = ".", fresh: bool = False):
        """Append one float32 frame (`<field>.0`, `_contents.0`)."""
        check(self.lib.gf_outflac(self.ctx, directory.encode(), 1 if fresh else 0), "outflac")

    def outmarker(self, directory: str = ".", fresh: bool = False):
        """Write marker1/marker2.NNNNNN.0 and list them in `_markers.0`."""
        check(self.lib.gf_outmarker(self.ctx, directory.encode(), 1 if fresh else 0), "outmarker")

    def saveflac(self, directory: str = "."):
        """Write the FP64 restart files (`*.rs`, `_contents.save`)."""
        check(self.lib.gf_saveflac(self.ctx, directory.encode()), "saveflac")
        self.download(0)

    def rsflac(self, directory: str = "."):
        """Restore the state from the restart files in `directory`."""
        check(self.lib.gf_rsflac(self.ctx, directory.encode()), "rsflac")
        check(self.lib.gf_get_params(self.ctx, C.byref(self.params)), "gf_get_params")
        self.download()

    # ---- sync points ----------------------------------------------------
    def upload(self, mask: int = capi.F_ALL):
        check(self.lib.gf_upload(self.ctx, mask), "gf_upload")
        check(self.lib.gf_set_clock(self.ctx, C.byref(self.clock)), "gf_set_clock")

    def download(self, mask: int = capi.F_ALL):
        if mask:
            check(self.lib.gf_download(self.ctx, mask), "gf_download")
        check(self.lib.gf_get_clock(self.ctx, C.byref(self.clock)), "gf_get_clock")
        return self.state

    # ---- the reference's per-step subroutines -------------------------
    def _call(self, name: str):
        check(getattr(self.lib, "gf_" + name)(self.ctx), name)

    def fl_therm(self):
        self._call("fl_therm")

    def change_phase(self):
        self._call("change_phase")

    def fl_rheol(self):
        self._call("fl_rheol")

    def fl_node(self):
        self._call("fl_node")

    def fl_move(self):
        self._call("fl_move")

    def rmasses(self):
        self._call("rmasses")

    def dt_mass(self):
        self._call("dt_mass")

    def init_visc(self):
        self._call("init_visc")

    def flac(self):
        """One call of the reference's `flac` plus nloop/time bookkeeping."""
        self._call("flac")

    def set_params(self):
        """Push edited parameters (e.g. remeshing settings) to the context."""
        check(self.lib.gf_set_params(self.ctx, C.byref(self.params)), "gf_set_params")

    def marker2elem(self):
        """Top up elements with fewer than 5 markers and recount phase ratios."""
        self._call("marker2elem")

    def remesh(self):
        """The remesh event of par.f90:94-108: bar2euler, remesh,
        lpeuler2bar, marker2elem, dhacc_correction reset."""
        self._call("remesh")

    def run(self, blocks: int) -> int:
        """par.f90:69-108 without output: `blocks` times, ntest_rem steps
        then the mesh-quality test and, if it fails, a remesh.  Returns the
        number of remesh events."""
        events = 0
        for _ in range(int(blocks)):
            self.step(self.params.ntest_rem)
            if self.params.ny_rem == 1 and self.params.itherm != 2:
                self.itest_mesh()
                check(self.lib.gf_get_clock(self.ctx, C.byref(self.clock)), "gf_get_clock")
                if self.clock.need_remeshing:
                    self.remesh()
                    events += 1
        return events

    def step(self, n: int):
        """n steps, each replayed from a captured CUDA graph."""
        check(self.lib.gf_step(self.ctx, int(n)), "gf_step")

    def itest_mesh(self) -> float:
        a = C.c_double()
        check(self.lib.gf_itest_mesh(self.ctx, C.byref(a)), "gf_itest_mesh")
        return a.value

    def set_sync(self, sync: bool):
        """sync=False: per-subroutine calls only enqueue (errors surface at
        the next status(), download() or step())."""
        check(self.lib.gf_set_sync(self.ctx, 1 if sync else 0), "gf_set_sync")

    def status(self):
        check(self.lib.gf_status(self.ctx), "gf_status")

    @property
    def stream(self) -> int:
        """The context's cudaStream_t (for recording events on it)."""
        return int(self.lib.gf_stream(self.ctx) or 0)

    @property
    def launches(self) -> int:
        return int(self.lib.gf_launch_count(self.ctx))

    def close(self):
        if self.ctx:
            self.lib.gf_destroy(self.ctx)
            self.ctx = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


def new_state(path: str, markers_per_side: int = 3, eclogite_rule: int = 0, therm_sweeps: int = 0):
    """Host-side start-up state (params, clock, arrays) without a device."""
    p = capi.read_params(path, markers_per_side, eclogite_rule, therm_sweeps)
    s = HostState(p)
    c = capi.setflac_host(p, s)
    return p, c, s


def clone(p: GfParams, c: GfClock, s: HostState, mp: Optional[int] = None):
    p2 = GfParams()
    C.memmove(C.byref(p2), C.byref(p), C.sizeof(GfParams))
    c2 = GfClock()
    C.memmove(C.byref(c2), C.byref(c), C.sizeof(GfClock))
    s2 = HostState(p2)
    s2.copy_from(s)
    return p2, c2, s2
