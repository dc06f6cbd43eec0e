"""The bounded grid barrier of the persistent kernels (the ensemble step and
the FP64 thermal sweeps) gives up instead of hanging: a CTA that never
arrives makes the other wait out its poll limit and leave with the error
flag set, which the host reads as GF_ERR_TIMEOUT; the device stays usable
(a barrier and a model step run normally afterwards)."""
import ctypes as C
import time

import pytest

from geoflac_gb300 import inpgen, new_state
from geoflac_gb300.capi import load_library
from geoflac_gb300.flac import Flac

pytestmark = pytest.mark.gpu

GF_ERR_TIMEOUT = -6


def _selftest():
    f = load_library().gf_grid_barrier_selftest
    f.restype = C.c_int
    f.argtypes = [C.c_int, C.c_longlong, C.POINTER(C.c_int)]

    def run(absent, limit):
        passed = (C.c_int * 2)()
        rc = f(absent, limit, passed)
        return rc, list(passed)

    return run


def test_barrier_passes_when_every_cta_arrives():
    run = _selftest()
    assert run(-1, 1 << 16) == (0, [1, 1])


def test_barrier_times_out_when_a_cta_never_arrives(workdir):
    run = _selftest()
    t0 = time.perf_counter()
    rc, passed = run(1, 1 << 14)  # ~1 ms of polls
    assert rc == GF_ERR_TIMEOUT
    assert passed == [0, -1]
    assert time.perf_counter() - t0 < 10.0
    # the device is still usable
    assert run(-1, 1 << 16) == (0, [1, 1])
    p, c, s = new_state(inpgen.extension_60x20().write(str(workdir / "bar.inp")))
    g = Flac(p, c, s, "fp64")
    g.step(3)
    g.status()
    g.download(0)
    assert g.clock.nloop == 3
    g.close()
