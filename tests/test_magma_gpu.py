"""Magma sub-model (itype_melting = 1) on the GPU against the oracle, through
the C-ABI: melting after change_phase (src/change_phase.f90:264-483),
fl_therm's freezing, MOR melting zone, melt migration and dike release with
new markers (src/fl_therm.f90:56-391), the arc-extrusion and MOR-crust
blocks of diff_topo and the extrusion branch of resurface
(src/fl_move.f90:213-302, 403-416), and the remeshing of the magma pools
(src/remesh.f90:106-115).

The 60x15 arc model (all 19 special phase ids) gets a hot mantle column
(MOR melt), subducted basalt and sediment below the Moho (arc melt),
a serpentinite element under hot mantle (flux melting), dike and MOR
marker volumes just below the threshold of a new marker, and accumulated
extrusion above the threshold of resurface's arc markers.  Integer fields
(markers, phases, marker count) must match exactly; floating-point fields
to 1e-10 of each field's largest magnitude (FP64, 31 steps: melting at
steps 0, 10, 20, 30)."""
import numpy as np
import pytest

from geoflac_gb300 import capi, inpgen, new_state
from geoflac_gb300.flac import Flac
from oracle.oracle import Oracle

from ._util import FLOAT_FIELDS, INT_FIELDS, compare_states, oracle_state

pytestmark = pytest.mark.gpu

TOL = 1e-10
MAGMA_FIELDS = ("fmelt", "fmelt2", "fmagma", "fmagma2", "dike_backlog", "dike_marker_vol", "mor_marker_vol",
                "dike_released", "extrusion", "extr_acc", "dhacc", "dhacc_correction", "temp0", "mark_a1",
                "mark_a2", "mark_age")


def recount(s, nphase):
    """count_phase_ratio (marker_data.f90:140-172) of every element"""
    nm, ids, ph = s["nmark_elem"], s["mark_id_elem"], s["mark_phase"]
    for i in range(nm.shape[1]):
        for j in range(nm.shape[0]):
            k = nm[j, i]
            cnt = np.bincount(ph[ids[:k, j, i] - 1], minlength=nphase + 1)[1:nphase + 1]
            s["phase_ratio"][:, j, i] = cnt / k
            s["iphase"][j, i] = int(np.argmax(cnt)) + 1 if cnt.max() > 0 else 1


def _set_phase(s, j, i, ph):
    ids = s["mark_id_elem"][:s["nmark_elem"][j, i], j, i]
    s["mark_phase"][ids - 1] = ph


def magma_state(workdir, tag, make=new_state):
    """The seeded arc model; `make` builds the start-up state (the
    library's new_state, or the oracle's own for the oracle side)."""
    m = inpgen.magma_arc()
    p, c, s = make(m.write(str(workdir / f"magma_{tag}.inp")))
    T = s["temp"]
    T[2:5, 8:17] = 1500.0  # hot mantle: MOR melt (Katz solidus ~1300 C at 60 km)
    for i in range(34, 38):  # subducted basalt / sediment below the Moho
        for j in (3, 4):
            _set_phase(s, j, i, 3 if i % 2 else 11)
    T[3:6, 34:39] = 1100.0
    _set_phase(s, 6, 45, 9)  # serpentinite under hot mantle: flux melting
    T[3:7, 45:47] = 1000.0
    recount(s, p.nphase)
    area = s["area"]
    ea = 0.5 / area[:, :, 0] + 0.5 / area[:, :, 1]
    kinc = s["nmark_elem"]
    for i in range(33, 40):  # dike volumes just below a marker's share
        for j in (0, 1):
            s["dike_marker_vol"][j, i] = 0.99999 * ea[j, i] / kinc[j, i]
    for i in (10, 12):  # MOR marker volume above it
        s["mor_marker_vol"][0, i] = 1.01 * ea[0, i] / kinc[0, i]
    s["dike_backlog"][2, 35] = 1e5
    elz = s["cord"][0, :-1, 1] - s["cord"][1, :-1, 1]
    for i in (40, 41, 42):  # accumulated extrusion above resurface's threshold
        s["extr_acc"][i] = 1.3 * elz[i] / kinc[0, i]
    return p, c, s


def _pair(workdir, tag):
    p, c, s = magma_state(workdir, tag)
    p2, c2, s2 = magma_state(workdir, tag + "_o", make=oracle_state)
    orc = Oracle(p2, c2, s2)
    orc.finish_setflac()
    return Flac(p, c, s, "fp64"), orc


def _compare(gpu, orc, where, tol=TOL):
    gpu.download()
    assert gpu.clock.nmarkers == orc.c.nmarkers, f"{where}: nmarkers {gpu.clock.nmarkers} vs {orc.c.nmarkers}"
    diffs, bad = compare_states(gpu.state, orc.s, FLOAT_FIELDS + MAGMA_FIELDS, INT_FIELDS)
    assert not bad, f"{where}: integer fields differ: {bad}"
    worst = max(diffs, key=diffs.get)
    assert diffs[worst] <= tol, f"{where}: {worst} differs by {diffs[worst]:.3e}"


def test_magma_steps_match_oracle(workdir):
    gpu, orc = _pair(workdir, "a")
    n0 = orc.c.nmarkers
    gpu.step(31)
    orc.step(31)
    _compare(gpu, orc, "31 steps")
    s = orc.s
    nm = orc.c.nmarkers
    # every pathway ran: both melt fractions, both pools, dikes released,
    # arc (14) and oceanic-crust (3) markers added
    assert (s["fmelt"] > 0).any() or (s["fmagma"] > 0).any()
    assert (s["fmagma"] > 0).sum() > 10 and (s["fmagma2"] > 0).sum() > 5
    assert (s["dike_released"] > 0).any()
    new = s["mark_phase"][n0:nm]
    assert (new == 14).sum() > 0 and (new == 3).sum() > 0
    assert int(s["nmark_elem"].sum()) == int((s["mark_dead"][:nm] != 0).sum())
    gpu.close()


def test_magma_flac_calls_and_remesh(workdir):
    gpu, orc = _pair(workdir, "b")
    for _ in range(11):  # gf_flac calls (one step each), melting at nloop 0 and 10
        gpu.flac()
        orc.flac()
    _compare(gpu, orc, "11 flac calls")
    orc.remesh_event()
    gpu.remesh()
    _compare(gpu, orc, "remesh", tol=1e-12)
    gpu.step(10)
    orc.step(10)
    _compare(gpu, orc, "after remesh")
    gpu.close()


def test_magma_drop_in_subroutines(workdir):
    """The reference's flac.f90 order through the per-subroutine entry points
    (fl_therm with the magma part, change_phase with melting, fl_rheol,
    fl_node, fl_move with the magma blocks of diff_topo, rmasses, dt_mass),
    the caller advancing nloop and time as par.f90 does."""
    gpu, orc = _pair(workdir, "d")
    p = orc.p
    for _ in range(12):
        nl = orc.c.nloop
        calls = ["fl_therm"]
        if nl % p.ifreq_rmasses == 0:
            calls.append("change_phase")
        calls += ["fl_rheol", "fl_node", "fl_move"]
        if nl % p.ifreq_rmasses == 0:
            calls.append("rmasses")
        if nl % p.ifreq_imasses == 0:
            calls.append("dt_mass")
        for f in calls:
            getattr(orc, f)()
            getattr(gpu, f)()
        orc.c.nloop += 1
        orc.c.time += orc.c.dt
        gpu.download(0)
        gpu.clock.nloop += 1
        gpu.clock.time += gpu.clock.dt
        gpu.upload(0)
    _compare(gpu, orc, "12 drop-in steps")
    gpu.close()


def test_magma_restart_round_trip(workdir, tmp_path):
    gpu, orc = _pair(workdir, "c")
    gpu.step(12)
    gpu.saveflac(str(tmp_path))
    before = {k: gpu.state[k].copy() for k in ("dike_backlog", "dike_marker_vol", "mor_marker_vol", "fmagma2")}
    p, c, s = magma_state(workdir, "c2")
    gpu2 = Flac(p, c, s, "fp64")
    gpu2.rsflac(str(tmp_path))
    gpu2.download()
    for k, v in before.items():
        assert np.array_equal(gpu2.state[k], v), k
    assert not gpu2.state["fmelt"].any() and not gpu2.state["fmelt2"].any()  # rsflac.f90:239-240
    gpu.close()
    gpu2.close()


def test_magma_rejected_in_mixed_contexts(workdir):
    p, c, s = magma_state(workdir, "m")
    with pytest.raises(capi.GfError) as e:
        Flac(p, c, s, "mixed")
    assert e.value.code == -5
