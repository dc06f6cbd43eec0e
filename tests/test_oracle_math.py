"""The one piece of code the oracle shares with the library: the
deterministic FP64 exp / log / pow / sin / cos / tan of
geoflac_gb300/csrc/gf_math.h.  The reference calls the C library's
functions (src/matprops.f90:136-215 exp and **, src/rh_plastic.f90:33-46 sin
and tan), so these tests measure the shared implementation against the C
library (Python's math module calls it) over the argument ranges the step
uses, and how far the choice between the two moves an oracle run.

Bounds, in units in the last place of the C library's result:
  exp (|x| <= 80: Arrhenius factors, depth decays)         1 ulp
  log (1e-30 .. 1e30)                                      2 ulp
  sin, cos (angles 0 .. 90 degrees and |x| <= 100)         1 ulp
  tan (0 .. 1.5 rad: friction angles)                      3 ulp
  pow (x in 1e-20 .. 1e20, |y| <= 1.5)                     2 + 2 |y ln x| ulp
pow is exp(y log x): the rounding of y log x is carried into the result
scaled by |y ln x|.
"""
import ctypes as C
import math

import numpy as np
import pytest

from geoflac_gb300 import inpgen
from oracle import oracle as O

from ._util import rel_diff

N = 20000


def _gfm(fn, x, y=None):
    lib = O.load()
    lib.or_gfm.restype = None
    lib.or_gfm.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_longlong]
    x = np.ascontiguousarray(x, dtype=np.float64)
    y = np.ascontiguousarray(x if y is None else y, dtype=np.float64)
    out = np.empty_like(x)
    lib.or_gfm(fn, x.ctypes.data, y.ctypes.data, out.ctypes.data, x.size)
    return out


def _clib(f, *args):
    return np.array([f(*a) for a in zip(*args)], dtype=np.float64)


def _ulp(a, b):
    """Distance in representable doubles (both finite, same sign)."""
    ia, ib = a.view(np.int64).astype(object), b.view(np.int64).astype(object)
    return np.array([abs(p - q) for p, q in zip(ia, ib)], dtype=np.float64)


def test_exp_log_sin_cos_tan_against_c_library():
    rng = np.random.default_rng(0)
    x = rng.uniform(-80.0, 80.0, N)
    assert _ulp(_gfm(0, x), _clib(math.exp, x)).max() <= 1
    x = 10.0 ** rng.uniform(-30.0, 30.0, N)
    assert _ulp(_gfm(1, x), _clib(math.log, x)).max() <= 2
    for x in (rng.uniform(0.0, math.pi / 2, N), rng.uniform(-100.0, 100.0, N)):
        s, c = _gfm(3, x), _gfm(4, x)
        sl, cl = _clib(math.sin, x), _clib(math.cos, x)
        same = np.sign(s) == np.sign(sl)
        assert _ulp(s[same], sl[same]).max() <= 1 and np.abs(s - sl).max() <= 2.3e-16
        same = np.sign(c) == np.sign(cl)
        assert _ulp(c[same], cl[same]).max() <= 1 and np.abs(c - cl).max() <= 2.3e-16
    x = rng.uniform(0.0, 1.5, N)
    assert _ulp(_gfm(5, x), _clib(math.tan, x)).max() <= 3


def test_pow_against_c_library():
    rng = np.random.default_rng(1)
    x = 10.0 ** rng.uniform(-20.0, 20.0, N)
    y = rng.uniform(-1.5, 1.5, N)
    u = _ulp(_gfm(2, x, y), _clib(math.pow, x, y))
    bound = 2.0 + 2.0 * np.abs(y * np.log(x))
    assert (u <= bound).all(), float((u / bound).max())


@pytest.fixture
def libm_switch():
    lib = O.load()
    lib.or_set_libm.restype = None
    lib.or_set_libm.argtypes = [C.c_int]
    yield lib.or_set_libm
    lib.or_set_libm(0)


def test_oracle_drift_between_shared_and_c_library_functions(workdir, libm_switch):
    """The oracle with the C library's exp / pow / sin / tan against the
    oracle with gf_math.h's, on the 60x20 extension model: the two differ by
    ulps per call, and the step carries that into the fields slowly at
    first (velocity 4e-16 after 10 steps, 4e-10 after 100, 3e-9 after 300)
    and then fast (7e-2 after 1000 steps): on this model an oracle built on
    the C library agrees with this one to 1e-10 in velocity for fewer than
    100 steps."""
    path = inpgen.extension_60x20().write(str(workdir / "libm_drift.inp"))
    runs = []
    for libm in (0, 1):
        libm_switch(libm)
        p, c, s = O.new_state(path)
        o = O.Oracle(p, c, s)
        o.finish_setflac()
        runs.append((libm, o, s))
    bounds = {10: 1e-13, 100: 1e-8, 300: 1e-7}
    for n, tol in bounds.items():
        for libm, o, _ in runs:
            libm_switch(libm)
            o.step(n - o.c.nloop)
        d = rel_diff(runs[1][2]["vel"], runs[0][2]["vel"])
        assert d <= tol, (n, d)
        assert rel_diff(runs[1][2]["stress0"], runs[0][2]["stress0"]) <= tol
    # the two are not the same function: the runs do differ
    assert rel_diff(runs[1][2]["visn"], runs[0][2]["visn"]) > 0
