"""Ensembles: many independent models advanced by one persistent kernel per
step (gf_batch_* in include/geoflac_gb300.h)."""
from __future__ import annotations

import ctypes as C
import os
from typing import List, Optional, Sequence

from . import capi, inpgen
from .capi import GfBatchConfig, check
from .flac import Flac, new_state


class Batch:
    """A batch over existing mixed-precision models (they stay usable as
    single models and keep their own state arrays)."""

    def __init__(self, members: Sequence[Flac]):
        self.lib = capi.load_library()
        self.members = list(members)
        arr = (C.c_void_p * len(self.members))(*[m.ctx.value for m in self.members])
        self.handle = C.c_void_p()
        check(self.lib.gf_batch_create(C.byref(self.handle), arr, len(self.members)), "gf_batch_create")

    @property
    def elements(self) -> int:
        return int(self.lib.gf_batch_elements(self.handle))

    @property
    def grid(self) -> int:
        return int(self.lib.gf_batch_grid(self.handle))

    @property
    def stream(self) -> int:
        return self.lib.gf_batch_stream(self.handle) or 0

    def config(self) -> dict:
        c = GfBatchConfig()
        check(self.lib.gf_batch_get_config(self.handle, C.byref(c)), "gf_batch_get_config")
        return {f: getattr(c, f) for f, _ in GfBatchConfig._fields_}

    def set_config(self, threads=256, items_per_thread=2, ctas_per_sm=1, graph_steps=10):
        c = GfBatchConfig(threads, items_per_thread, ctas_per_sm, graph_steps)
        check(self.lib.gf_batch_set_config(self.handle, C.byref(c)), "gf_batch_set_config")

    def tune(self, trial_steps: int = 2) -> dict:
        """Autotune the CTA shape, tile depth and residency (the trial steps
        advance the members)."""
        c = GfBatchConfig()
        ms = C.c_double()
        check(self.lib.gf_batch_tune(self.handle, int(trial_steps), C.byref(c), C.byref(ms)), "gf_batch_tune")
        out = {f: getattr(c, f) for f, _ in GfBatchConfig._fields_}
        out["ms_per_step"] = ms.value
        return out

    def step(self, n: int):
        check(self.lib.gf_batch_step(self.handle, int(n)), "gf_batch_step")

    def sample(self, grid, H: int, W: int, phase_id: int = 2):
        """fields of every member on an H x W grid (device FP32 tensor
        [n, H, W, 9])"""
        check(self.lib.gf_batch_sample(self.handle, grid.data_ptr(), H, W, phase_id), "gf_batch_sample")

    def inject(self, grid, H: int, W: int):
        check(self.lib.gf_batch_inject(self.handle, grid.data_ptr(), H, W), "gf_batch_inject")

    def force_residual(self):
        import numpy as np
        out = np.zeros(len(self.members))
        check(self.lib.gf_batch_force_residual(self.handle, out.ctypes.data_as(C.POINTER(C.c_double))),
              "gf_batch_force_residual")
        return out

    def backup(self):
        """device copy of the fields an injection overwrites"""
        check(self.lib.gf_batch_backup(self.handle), "gf_batch_backup")

    def restore(self, members):
        arr = (C.c_int * len(members))(*[int(k) for k in members])
        check(self.lib.gf_batch_restore(self.handle, arr, len(members)), "gf_batch_restore")

    def close(self):
        if self.handle:
            self.lib.gf_batch_destroy(self.handle)
            self.handle = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def ensemble(n: int, workdir: str, seed: int = inpgen.ENSEMBLE_SEED, mode: str = "mixed",
             scale: Optional[tuple] = None) -> List[tuple]:
    """n sweep members as (Flac, sampled parameters), .inp files written to
    workdir (9 markers per element)."""
    from concurrent.futures import ThreadPoolExecutor

    def host(k):
        m, prm = inpgen.ensemble_member(k, seed, scale or (80, 25, 400, 120))
        path = m.write(os.path.join(workdir, f"member_{k:04d}.inp"))
        return new_state(path), prm

    # the host start-up (read_params + setflac) of the members runs in
    # parallel (the library calls release the interpreter lock); the
    # device contexts are then created in member order
    with ThreadPoolExecutor(max_workers=min(16, os.cpu_count() or 4)) as ex:
        states = list(ex.map(host, range(n)))
    return [(Flac(p, c, s, mode), prm) for (p, c, s), prm in states]
