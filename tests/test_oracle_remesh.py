"""CPU checks of the oracle's remesh event (bar2euler -> remesh ->
lpeuler2bar -> marker2elem, src/par.f90:89-108) on a deformed convergent
model: the regridded mesh, the marker bookkeeping and the phase ratios."""
import numpy as np

from geoflac_gb300 import inpgen
from oracle.oracle import Oracle, new_state


def test_remesh_event_invariants(workdir):
    inp = inpgen.CONFIGS["convergence_60x15"]().write(str(workdir / "c3s_rm.inp"))
    p, c, s = new_state(inp)
    assert p.incoming_left == 1
    o = Oracle(p, c, s, threads=2)
    o.finish_setflac()
    o.step(400)
    alive0 = int((s["mark_dead"][: c.nmarkers] != 0).sum())
    o.remesh_event()
    nm = c.nmarkers
    live = np.nonzero(s["mark_dead"][:nm])[0]
    assert 0.9 * alive0 <= len(live) <= nm
    # every live marker sits in the element of its triangle number with
    # barycentric coordinates of a point inside it
    a1, a2 = s["mark_a1"][live], s["mark_a2"][live]
    tol = 1e-9
    assert (a1 >= -tol).all() and (a2 >= -tol).all() and (a1 + a2 <= 1 + tol).all()
    nz = p.nz
    nt = s["mark_ntriag"][live]
    k = (nt - 1) % 2 + 1
    j = ((nt - k) // 2) % (nz - 1)
    i = (nt - k) // 2 // (nz - 1)
    counts = np.zeros((p.nx - 1, nz - 1), dtype=np.int64)
    np.add.at(counts, (i, j), 1)
    assert (counts.T == s["nmark_elem"]).all()
    # each element lists its own markers, in increasing index order
    ids = s["mark_id_elem"]
    for e_i in range(0, p.nx - 1, 7):
        for e_j in range(nz - 1):
            n = s["nmark_elem"][e_j, e_i]
            lst = ids[:n, e_j, e_i]
            assert (np.diff(lst) > 0).all()
    pr = s["phase_ratio"]
    assert np.allclose(pr.sum(axis=0), 1.0, atol=1e-12)
    # bottom row back at z0 + rzbo (mode_rem 1 without a flexural bottom)
    assert np.allclose(s["cord"][-1, :, 1], p.z0 + p.rzbo, atol=0, rtol=0)
    assert o.itest_mesh() > p.angle_rem
    o.step(50)
