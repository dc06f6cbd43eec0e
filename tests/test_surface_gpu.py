"""Surface processes (diff_topo and resurface, src/fl_move.f90:138-472; the
topography test of src/rem_test.f90:45-66; the accumulators' remeshing,
src/remesh.f90:20-53) on the GPU against the oracle, through the C-ABI.

The 60x20 extension model gets a surface relief, a diffusivity and phase
erodibilities, and accumulated surface changes large enough that the first
resurface call (every ifreq_avgsr steps) erodes the topmost marker of some
surface elements and deposits sediment markers in others.  Integer fields
(marker lists, triangle numbers, phases, marker count) must match exactly;
floating-point fields, the accumulators included, to 1e-10 of each field's
largest magnitude (FP64 path, 60 steps).
"""
import numpy as np
import pytest

from geoflac_gb300 import capi, inpgen, new_state
from geoflac_gb300.flac import Flac
from oracle.oracle import Oracle

from ._util import FLOAT_FIELDS, INT_FIELDS, compare_states, oracle_state

pytestmark = pytest.mark.gpu

TOL = 1e-10
EXTRA_FLOATS = ("dhacc", "dtopo", "dhacc_correction", "mark_a1", "mark_a2", "mark_age", "temp0")


def _init_areas(s):
    """init_areas (src/init_areas.f90) for the relief-modified mesh."""
    c = s["cord"]
    x1, y1 = c[:-1, :-1, 0], c[:-1, :-1, 1]
    x2, y2 = c[1:, :-1, 0], c[1:, :-1, 1]
    x3, y3 = c[:-1, 1:, 0], c[:-1, 1:, 1]
    x4, y4 = c[1:, 1:, 0], c[1:, 1:, 1]
    a = s["area"]
    a[:, :, 0] = 1.0 / (((x2 * y3 - y2 * x3) - (x1 * y3 - y1 * x3)) + (x1 * y2 - y1 * x2))
    a[:, :, 1] = 1.0 / (((x2 * y4 - y2 * x4) - (x3 * y4 - y3 * x4)) + (x3 * y2 - y3 * x2))
    a[:, :, 2] = 1.0 / (((x2 * y4 - y2 * x4) - (x1 * y4 - y1 * x4)) + (x1 * y2 - y1 * x2))
    a[:, :, 3] = 1.0 / (((x4 * y3 - y4 * x3) - (x1 * y3 - y1 * x3)) + (x1 * y4 - y1 * x4))


def _surface_state(path, make):
    """The 60x20 model with a surface relief and accumulated surface
    changes; `make` builds the start-up state (the library's or the
    oracle's own)."""
    p, c, s = make(path)
    for k in range(p.nphase):
        p.erodibility[k] = 0.5 + 0.25 * k
    x = s["cord"][0, :, 0]
    s["cord"][0, :, 1] += 150.0 * np.sin(2 * np.pi * x / 60e3)
    _init_areas(s)
    # accumulated change of one element thickness (5 km) / markers per element
    # in alternating columns: erosion in some, deposition in others
    elz = s["cord"][0, :-1, 1] - s["cord"][1, :-1, 1]
    kinc = s["nmark_elem"][0, :]
    dh = np.zeros(p.nx)
    dh[3:-3:7] = -1.5 * elz[3:-3:7] / kinc[3:-3:7]
    dh[6:-3:7] = 1.5 * elz[6:-3:7] / kinc[6:-3:7]
    s["dhacc"][...] = dh
    return p, c, s


def _setup(workdir, tag, mode="fp64"):
    m = inpgen.extension_60x20()
    m.topo_kappa = 2e-5
    path = m.write(str(workdir / f"surf_{tag}.inp"))
    p, c, s = _surface_state(path, new_state)
    p2, c2, s2 = _surface_state(path, oracle_state)
    orc = Oracle(p2, c2, s2)
    orc.finish_setflac()
    return Flac(p, c, s, mode), orc


def _compare(gpu, orc, where, tol=TOL):
    gpu.download()
    assert gpu.clock.nmarkers == orc.c.nmarkers, f"{where}: nmarkers {gpu.clock.nmarkers} vs {orc.c.nmarkers}"
    diffs, bad = compare_states(gpu.state, orc.s, FLOAT_FIELDS + EXTRA_FLOATS, INT_FIELDS)
    assert not bad, f"{where}: integer fields differ: {bad}"
    worst = max(diffs, key=diffs.get)
    assert diffs[worst] <= tol, f"{where}: {worst} differs by {diffs[worst]:.3e}"


def test_diff_topo_and_resurface_match_oracle(workdir):
    gpu, orc = _setup(workdir, "a")
    n0 = orc.c.nmarkers
    live0 = int((orc.s["mark_dead"][:n0] != 0).sum())
    gpu.step(60)
    orc.step(60)
    _compare(gpu, orc, "60 steps")
    s = orc.s
    nm = orc.c.nmarkers
    live = int((s["mark_dead"][:nm] != 0).sum())
    # the first resurface call removed markers (erosion) and added sediment
    # markers (phase 1, deposition)
    assert nm > n0 and (s["mark_dead"][:n0] == 0).any() and live0 == n0
    assert (s["mark_phase"][n0:nm] == 1).all()
    assert np.abs(s["dtopo"]).max() > 0
    assert int(s["nmark_elem"].sum()) == live
    gpu.close()


def test_per_subroutine_calls_and_remesh_with_accumulators(workdir):
    gpu, orc = _setup(workdir, "b")
    for _ in range(12):  # per-subroutine drop-in calls, resurface at nloop 0 and 10
        gpu.flac()
        orc.flac()
    _compare(gpu, orc, "12 flac calls")
    # topography test: an accumulated change above 1/3 of the top element
    for st in (gpu.state, orc.s):
        st["dhacc"][5] = 0.5 * (st["cord"][0, 0, 1] - st["cord"][1, 0, 1])
    gpu.upload(capi.F_MARKERS)
    gpu.itest_mesh()
    orc.itest_mesh()
    gpu.download(0)
    assert gpu.clock.need_remeshing == orc.c.need_remeshing == 3
    orc.remesh_event()
    gpu.remesh()
    _compare(gpu, orc, "remesh", tol=1e-12)
    gpu.step(30)
    orc.step(30)
    _compare(gpu, orc, "after remesh")
    gpu.close()


def test_mixed_path_runs_surface_processes(workdir):
    gpu, orc = _setup(workdir, "m", mode="mixed")
    gpu.step(60)
    orc.step(60)
    s = gpu.download()
    nm = gpu.clock.nmarkers
    live = np.nonzero(s["mark_dead"][:nm])[0]
    assert nm == orc.c.nmarkers  # the same resurface events
    assert int(s["nmark_elem"].sum()) == len(live)
    top = s["cord"][0, :, 1]
    ref = orc.s["cord"][0, :, 1]
    assert np.abs(top - ref).max() <= 1e-6 * np.abs(ref).max() + 1e-3
    assert np.isfinite(s["vel"]).all() and np.isfinite(s["stress0"]).all()
    gpu.close()


def test_batch_rejects_surface_processes(workdir):
    from geoflac_gb300.batch import Batch
    gpu, _ = _setup(workdir, "r", mode="mixed")
    with pytest.raises(capi.GfError) as e:
        Batch([gpu])
    assert e.value.code == -5
    gpu.close()


def _flex_model(workdir, tag, mode="fp64", make=new_state):
    """The 60x20 model on a flexural bottom (nbc 200: 20 km elastic plate on
    a 3300 kg/m3 fluid) instead of the free-slip base, with a surface relief
    whose load the plate carries; `make` builds the start-up state."""
    m = inpgen.extension_60x20()
    m.bcs = [b for b in m.bcs if b.side != 2] + [inpgen.BC(2, 1, m.nex + 1, 200, 20e3, 3300.0)]
    p, c, s = make(m.write(str(workdir / f"flex_{tag}.inp")))
    x = s["cord"][0, :, 0]
    s["cord"][0, :, 1] += 300.0 * np.exp(-((x - 150e3) / 30e3) ** 2)
    _init_areas(s)
    return p, c, s


def test_flexure_matches_oracle(workdir):
    p, c, s = _flex_model(workdir, "a")
    assert p.nbc[[b for b in range(p.nofbc) if p.nofside[b] == 2][0]] == 200
    p2, c2, s2 = _flex_model(workdir, "a_o", make=oracle_state)
    orc = Oracle(p2, c2, s2)
    orc.finish_setflac()
    gpu = Flac(p, c, s, "fp64")
    gpu.step(60)
    orc.step(60)
    extra = ("q_init", "vel_flex_old", "orig")
    gpu.download()
    diffs, bad = compare_states(gpu.state, orc.s, FLOAT_FIELDS + EXTRA_FLOATS + extra, INT_FIELDS)
    assert not bad, f"integer fields differ: {bad}"
    worst = max(diffs, key=diffs.get)
    assert diffs[worst] <= TOL, f"{worst} differs by {diffs[worst]:.3e}"
    # the plate moved the bottom off its start-up depth
    bottom = orc.s["cord"][-1, :, 1]
    assert np.abs(bottom - orc.s["orig"][-1, :, 1]).max() > 0
    assert np.abs(orc.s["q_init"]).max() > 0
    gpu.close()


def test_flexure_rejected_in_mixed_contexts(workdir):
    p, c, s = _flex_model(workdir, "m")
    with pytest.raises(capi.GfError) as e:
        Flac(p, c, s, "mixed")
    assert e.value.code == -5
