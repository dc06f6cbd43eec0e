"""Pins the oracle's magma sub-model (src/change_phase.f90:264-483,
src/fl_therm.f90:56-391) to answers derived by hand from the reference's
formulas, on the 60x15 arc model (CPU only):

* an isolated basalt element above its solidus (Gutscher 2000 curve) melts
  by cp (T - T_s) / L, capped at 10 %, and its corners cool to the solidus;
* a magma pool freezes by dt lambda(T) per step and its latent heat
  L dM / cp / 4 warms each corner;
* the dike release is capped at 1e-4 Amin per step, the rest banked;
* a marker volume of k.x shares of the element adds ceil(k.x) markers of
  the pathway's phase (karc1 = 14, kocean1 = 3) at the element centre;
* without melt or magma the sub-model changes nothing.
"""
import math

import numpy as np
import pytest

from geoflac_gb300 import clone, inpgen
from oracle.oracle import Oracle, new_state

from .test_magma_gpu import _set_phase, recount


def _state(workdir, tag, **kw):
    m = inpgen.magma_arc()
    for k, v in kw.items():
        setattr(m, k, v)
    p, c, s = new_state(m.write(str(workdir / f"magma_or_{tag}.inp")))
    return p, c, s


def _node_xy(s, n, nz):
    """marker n's position from its barycentric coordinates (bar2euler.f90:73-117)"""
    nt = s["mark_ntriag"][n]
    k = (nt - 1) % 2 + 1
    jj = ((nt - k) // 2) % (nz - 1)
    ii = (nt - k) // 2 // (nz - 1)
    if k == 1:
        pts = [(jj, ii), (jj + 1, ii), (jj, ii + 1)]
    else:
        pts = [(jj, ii + 1), (jj + 1, ii), (jj + 1, ii + 1)]
    b = [s["mark_a1"][n], s["mark_a2"][n]]
    b.append(1.0 - b[0] - b[1])
    c = s["cord"]
    return (sum(b[q] * c[pts[q][0], pts[q][1], 0] for q in range(3)),
            sum(b[q] * c[pts[q][0], pts[q][1], 1] for q in range(3)))


def test_isolated_basalt_melts_to_its_solidus(workdir):
    p, c, s = _state(workdir, "melt")
    j, i = 4, 36
    _set_phase(s, j, i, 3)
    recount(s, p.nphase)
    T = s["temp"]
    T[j:j + 2, i:i + 2] = 900.0
    o = Oracle(p, c, s)
    o.change_phase()
    z = s["cord"][:, :, 1]
    yy = 0.25 * (z[j, i] + z[j, i + 1] + z[j + 1, i] + z[j + 1, i + 1])
    depth = 0.5 * (z[0, i] + z[0, i + 1]) - yy
    press = 3000 * 10 * depth / 1e9
    assert 1.0 <= press <= 2.7
    solidus = 630.0 + 13.0 * press ** 2  # Gutscher 2000, 1-2.7 GPa
    tpr = sum(s["phase_ratio"][k - 1, j, i] for k in (3, 7, 10, 13))
    assert tpr == pytest.approx(1.0)
    pmelt = min(p.cp[2] * (900.0 - solidus) / p.latent_heat_magma, 0.1)
    assert s["fmelt"][j, i] == pytest.approx(pmelt * tpr, rel=1e-12)
    assert 0 < s["fmelt"][j, i] <= 0.1
    tmpr = 0.25 * (T[j, i] + T[j, i + 1] + T[j + 1, i] + T[j + 1, i + 1])
    assert tmpr == pytest.approx(solidus, rel=1e-12)
    # nothing else melted
    assert np.count_nonzero(s["fmelt"]) == 1 and not s["fmelt2"].any()


def test_freezing_releases_latent_heat(workdir):
    p, c, s = _state(workdir, "freeze")
    for k in range(p.nphase):  # no diffusion: the latent heat alone changes temp
        p.conduct[k] = 0.0
    s["source"][...] = 0.0
    c.dt = 1e10
    j, i = 5, 20
    s["fmagma"][j, i] = 0.05
    s["fmagma2"][j, i] = 0.02
    T0 = s["temp"].copy()
    o = Oracle(p, c, s)
    o.fl_therm()
    tmpr = 0.25 * (T0[j, i] + T0[j + 1, i] + T0[j, i + 1] + T0[j + 1, i + 1])
    lam = p.lambda_freeze * math.exp(-p.lambda_freeze_tdep * (tmpr - p.t_top))
    d1, d2 = min(0.05, 0.05 * c.dt * lam), min(0.02, 0.02 * c.dt * lam)
    assert s["fmagma"][j, i] == pytest.approx(0.05 - d1, rel=1e-12)
    assert s["fmagma2"][j, i] == pytest.approx(0.02 - d2, rel=1e-12)
    cp = p.cp[s["iphase"][j, i] - 1]
    dT = (d1 + d2) * p.latent_heat_magma / cp / 4
    assert dT > 1e-4
    dTn = s["temp"] - T0
    np.testing.assert_allclose(dTn[j:j + 2, i:i + 2], dT, rtol=1e-9)
    dTn[j:j + 2, i:i + 2] = 0.0
    assert not dTn[1:-1, 1:-1].any()  # interior nodes other than the corners
    assert np.array_equal(s["temp0"], T0)


def test_dike_release_cap_and_new_markers(workdir):
    p, c, s = _state(workdir, "dike")
    c.dt = 1e10
    area = s["area"]
    ea = 0.5 / area[:, :, 0] + 0.5 / area[:, :, 1]
    kinc = s["nmark_elem"]
    s["dike_backlog"][1, 20] = 1e6
    unit_a = ea[0, 25] / kinc[0, 25]
    unit_r = ea[0, 26] / kinc[0, 26]
    s["dike_marker_vol"][0, 25] = 2.5 * unit_a
    s["mor_marker_vol"][0, 26] = 1.2 * unit_r
    k25, k26 = kinc[0, 25], kinc[0, 26]
    o = Oracle(p, c, s)
    n0 = o.c.nmarkers
    o.fl_therm()
    cap = 1e-4 * p.Amin
    assert s["dike_backlog"][1, 20] == pytest.approx(1e6 - cap, rel=1e-12)
    assert s["dike_released"][1, 20] == pytest.approx(cap / ea[1, 20], rel=1e-12)
    assert s["dike_marker_vol"][1, 20] == pytest.approx(cap, rel=1e-12)
    # 3 arc markers in (0, 25), then 2 oceanic-crust markers in (0, 26)
    assert o.c.nmarkers == n0 + 5
    assert list(s["mark_phase"][n0:n0 + 5]) == [14, 14, 14, 3, 3]
    assert s["nmark_elem"][0, 25] == k25 + 3 and s["nmark_elem"][0, 26] == k26 + 2
    assert s["dike_marker_vol"][0, 25] == 0.0 and s["mor_marker_vol"][0, 26] == 0.0
    cx = s["cord"][:, :, 0]
    cz = s["cord"][:, :, 1]
    for n, (jj, ii) in zip(range(n0, n0 + 5), [(0, 25)] * 3 + [(0, 26)] * 2):
        x, z = _node_xy(s, n, p.nz)
        assert x == pytest.approx(cx[jj:jj + 2, ii:ii + 2].mean(), rel=1e-12)
        assert z == pytest.approx(cz[jj:jj + 2, ii:ii + 2].mean(), abs=1e-6)
    # the recount sees the new phases
    assert s["phase_ratio"][13, 0, 25] == pytest.approx(3 / (k25 + 3))


def test_no_melt_no_magma_changes_nothing(workdir):
    p, c, s = _state(workdir, "quiet")
    c.dt = 1e10
    p0, c0, s0 = clone(p, c, s)
    p0.itype_melting = 0
    Oracle(p, c, s).fl_therm()
    Oracle(p0, c0, s0).fl_therm()
    for k in ("temp", "temp0", "fmagma", "fmagma2", "nmark_elem", "dike_released"):
        assert np.array_equal(s[k], s0[k]), k
    Oracle(p, c, s).change_phase()
    Oracle(p0, c0, s0).change_phase()
    assert np.array_equal(s["temp"], s0["temp"])
    assert not s["fmelt"].any() and not s["fmelt2"].any()
