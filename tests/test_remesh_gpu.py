"""The remesh event on the GPU (bar2euler, remesh, lpeuler2bar, marker2elem,
src/par.f90:94-108) against the oracle, through the C-ABI.

Integer fields (marker element lists, triangle numbers, phases, marker
numbering of the top-up) must match exactly; floating-point fields are
compared at 1e-12 of each field's largest magnitude (the FP64 kernels repeat
the serial arithmetic, so the measured difference is 0), and the run goes on
for 50 steps after the event within the step parity tolerance 1e-10.
"""
import numpy as np
import pytest

from geoflac_gb300 import inpgen, new_state
from geoflac_gb300.flac import Flac
from oracle.oracle import Oracle

from ._util import FLOAT_FIELDS, INT_FIELDS, compare_states, oracle_state

pytestmark = pytest.mark.gpu

EVENT_TOL = 1e-12
STEP_TOL = 1e-10
EXTRA_FLOATS = ("temp0", "source", "mark_a1", "mark_a2", "mark_age")
EXTRA_INTS = ("jmoho",)


def _pair(workdir, name, mode="fp64", **kw):
    inp = inpgen.CONFIGS[name]().write(str(workdir / f"{name}_rm.inp"))
    p, c, s = new_state(inp, **kw)
    p2, c2, s2 = oracle_state(inp, **kw)
    orc = Oracle(p2, c2, s2)
    orc.finish_setflac()
    return Flac(p, c, s, mode), orc


def _compare(gpu, orc, tol, where):
    gpu.download()
    nm = orc.c.nmarkers
    assert gpu.clock.nmarkers == nm, f"{where}: nmarkers {gpu.clock.nmarkers} vs {nm}"
    diffs, bad = compare_states(gpu.state, orc.s, FLOAT_FIELDS + EXTRA_FLOATS, INT_FIELDS + EXTRA_INTS)
    assert not bad, f"{where}: integer fields differ: {bad}"
    worst = max(diffs, key=diffs.get)
    assert diffs[worst] <= tol, f"{where}: {worst} differs by {diffs[worst]:.3e} (all: {diffs})"
    for k in ("dt", "time", "dt_elastic", "dt_maxwell"):
        a, b = getattr(gpu.clock, k), getattr(orc.c, k)
        assert abs(a - b) <= tol * max(abs(b), 1e-300), f"{where}: clock {k} {a} vs {b}"
    return diffs


@pytest.mark.parametrize("name,mps,steps", [("convergence_60x15", 3, 400), ("convergence_60x15", 2, 600),
                                            ("extension_60x20", 3, 300)])
def test_remesh_event_matches_oracle(workdir, name, mps, steps):
    gpu, orc = _pair(workdir, name, markers_per_side=mps)
    gpu.step(steps)
    orc.step(steps)
    n0 = orc.c.nmarkers
    orc.remesh_event()
    gpu.remesh()
    _compare(gpu, orc, EVENT_TOL, "remesh")
    if mps == 2:
        assert orc.c.nmarkers > n0, "the 4-marker case must exercise the top-up"
    gpu.step(50)
    orc.step(50)
    _compare(gpu, orc, STEP_TOL, "after remesh")
    gpu.close()


def test_marker2elem_top_up_matches_oracle(workdir):
    """marker2elem alone on a state whose elements hold 4 markers each."""
    gpu, orc = _pair(workdir, "extension_60x20", markers_per_side=2)
    gpu.step(20)
    orc.step(20)
    gpu.download()  # the clock (nloop seeds the marker positions)
    assert gpu.clock.nloop == orc.c.nloop
    orc.s["nmark_elem"][...] = np.minimum(orc.s["nmark_elem"], 4)
    gpu.state.copy_from(orc.s)
    gpu.upload()
    orc.marker2elem()
    gpu.marker2elem()
    _compare(gpu, orc, EVENT_TOL, "marker2elem")
    gpu.close()


def test_run_loop_remeshes_like_the_oracle(workdir):
    """par.f90's loop: ntest_rem steps, itest_mesh, remesh when the smallest
    angle falls below angle_rem (raised here so that events happen)."""
    gpu, orc = _pair(workdir, "convergence_60x15")
    for pr in (gpu.params, orc.p):
        pr.ny_rem = 1
        pr.ntest_rem = 100
        pr.angle_rem = 44.2
    gpu.set_params()
    events = 0
    for _ in range(4):
        orc.step(orc.p.ntest_rem)
        angle = orc.itest_mesh()
        if angle <= orc.p.angle_rem:
            orc.remesh_event()
            events += 1
    assert gpu.run(4) == events
    assert events >= 1
    _compare(gpu, orc, STEP_TOL, "run")
    gpu.close()


def test_mixed_remesh_keeps_marker_bookkeeping(workdir):
    gpu, _ = _pair(workdir, "convergence_60x15", mode="mixed")
    gpu.step(400)
    gpu.remesh()
    gpu.step(50)
    s = gpu.download()
    nm = gpu.clock.nmarkers
    live = np.nonzero(s["mark_dead"][:nm])[0]
    assert s["nmark_elem"].sum() == len(live)
    assert np.allclose(s["phase_ratio"].sum(axis=0), 1.0, atol=1e-12)
    assert np.isfinite(s["stress0"]).all() and np.isfinite(s["vel"]).all()
    gpu.close()
