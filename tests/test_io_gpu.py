"""Output frames and restart files through the C-ABI: outflac / outmarker
(src/outflac.f90, src/outmarker.f90) and saveflac / rsflac (src/saveflac.f90,
src/rsflac.f90).

The files are read here with numpy in the reference's record layout
(gfortran direct access: fixed-length records, no markers) and compared with
the context's state: float32 node fields that are plain conversions of FP64
values bit for bit, derived element fields within 1e-6 of each field's
largest value (FP64 arithmetic cast to float32; mixed-precision contexts
1e-5), integer records exactly.  The restart is compared with the oracle
given the same saved state and the same rsflac tail: 1e-12 right after the
restart, 1e-10 after 50 more steps.
"""
import os
import shutil

import numpy as np
import pytest

from geoflac_gb300 import capi, inpgen, new_state
from geoflac_gb300.capi import SEC_YEAR
from geoflac_gb300.flac import Flac, clone
from oracle.oracle import Oracle

from ._util import FLOAT_FIELDS, INT_FIELDS, compare_states

pytestmark = pytest.mark.gpu

MAXM = 32


def _records(path, dtype, count):
    a = np.fromfile(path, dtype=dtype)
    assert a.size % count == 0, f"{path}: {a.size} items is not a whole number of records of {count}"
    return a.reshape(-1, count)


def _field(d, name, dtype, shape, rec=1):
    n = int(np.prod(shape))
    return _records(os.path.join(d, name), dtype, n)[rec - 1].reshape(shape, order="F")


def _eff_dens(p, s):
    """Eff_dens (src/matprops.f90:3-83) over all elements, FP64."""
    z, t = s["cord"][:, :, 1], s["temp"]
    zc = 0.25 * (z[:-1, :-1] + z[1:, :-1] + z[:-1, 1:] + z[1:, 1:])
    t0 = 0.25 * (t[:-1, :-1] + t[1:, :-1] + t[:-1, 1:] + t[1:, 1:])
    zs = 0.50 * (z[0, :-1] + z[0, 1:])[None, :]
    tm = (zs - zc) * 1e-3 * 3e-1 + t0
    amp = np.ones_like(zc)
    d410 = -101.58 * (tm + 273.0) - 216828.0
    f = np.clip((d410 - zc) / (d410 - (d410 - 30e3)), 0.0, 1.0)
    amp = np.where(d410 > zc, 1.0 + 0.05 * f, amp)
    d660 = 66.55 * (tm + 273.0) - 788494.0
    f = np.clip((d660 - zc) / (d660 - (d660 - 30e3)), 0.0, 1.0)
    amp = np.where(d660 > zc, 1.05 + 0.085 * f, amp)
    st = s["stress0"]
    press = np.zeros_like(zc)
    for k in range(4):
        press = press - (st[:, :, 0, k] + st[:, :, 1, k] + st[:, :, 3, k])
    press = press / 12
    ed = np.zeros_like(zc)
    for k in range(p.nphase):
        r = s["phase_ratio"][k]
        use = r >= 0.01
        dens = p.den[k] * (1 - p.alfa[k] * tm + p.beta[k] * press)
        pk = dens * p.g * zc
        dens = p.den[k] * (1 - p.alfa[k] * tm + p.beta[k] * pk)
        press = np.where(use, pk, press)
        ed = ed + np.where(use, r * dens, 0.0)
    iph = s["iphase"]
    ed = np.where(np.isin(iph, (4, 8, 9, 16, 18)), ed * amp, ed)
    fma = np.minimum(s["fmagma"] + s["fmagma2"], p.fmagma_max)
    return ed - fma * (ed - p.rho_magma)


def _expected_elements(p, c, s):
    st = s["stress0"]
    sm = [0.25 * (st[:, :, q, 0] + st[:, :, q, 1] + st[:, :, q, 2] + st[:, :, q, 3]) for q in range(4)]
    sI = (sm[0] + sm[1] + sm[3]) / 3.0
    e = s["strain"]
    e2sr = s["e2sr"]
    t = s["temp"]
    iph = s["iphase"]
    den = np.array([p.den[k] for k in range(p.nphase)])
    with np.errstate(divide="ignore", invalid="ignore"):  # hs = 0 gives inf, as in the reference
        diss = s["shrheat"] / den[iph - 1] / p.hs if p.ishearh != 0 else np.zeros_like(sI)
    out = {
        "srII.0": np.where(e2sr != 0, np.log10(np.where(e2sr != 0, e2sr, 1.0)), 0.0),
        "srxx.0": s["se2sr"][:, :, 0] / c.dtavg,
        "srzz.0": s["se2sr"][:, :, 1] / c.dtavg,
        "srxz.0": s["se2sr"][:, :, 2] / c.dtavg,
        "eII.0": 0.5 * np.sqrt((e[:, :, 0] - e[:, :, 1]) ** 2 + 4 * e[:, :, 2] ** 2),
        "eI.0": 0.5 * (e[:, :, 0] + e[:, :, 1]),
        "exx.0": e[:, :, 0], "ezz.0": e[:, :, 1], "exz.0": e[:, :, 2],
        "density.0": _eff_dens(p, s),
        "area.0": 0.5 / s["area"][:, :, 0] + 0.5 / s["area"][:, :, 1],
        "aps.0": s["aps"],
        "sII.0": 0.5 * np.sqrt((sm[0] - sm[1]) ** 2 + 4 * sm[2] * sm[2]),
        "sxx.0": sm[0] - sI, "szz.0": sm[1] - sI, "sxz.0": sm[2], "syy.0": sm[3] - sI, "pres.0": sI,
        "temp.0": 0.25 * (t[:-1, :-1] + t[1:, :-1] + t[:-1, 1:] + t[1:, 1:]),
        "visc.0": np.log10(s["visn"]),
        "src.0": s["source"],
        "fmelt.0": np.zeros_like(sI), "fmelt2.0": np.zeros_like(sI),
        "fmagma.0": s["fmagma"], "fmagma2.0": s["fmagma2"],
        "diss.0": diss,
    }
    return out


def _model(workdir, name, mode, **kw):
    inp = inpgen.CONFIGS[name]().write(str(workdir / f"{name}_io_{mode}.inp"))
    p, c, s = new_state(inp, **kw)
    return inp, Flac(p, c, s, mode)


@pytest.mark.parametrize("mode,tol", [("fp64", 1e-6), ("mixed", 1e-5)])
def test_outflac_frame_matches_state(workdir, mode, tol):
    _, g = _model(workdir, "extension_60x20", mode)
    for k in range(19):
        g.params.io_flags[k] = 1
    g.set_params()
    cord0 = g.state["cord"].copy()
    g.step(60)
    d = str(workdir / f"frames_{mode}")
    os.makedirs(d, exist_ok=True)
    g.outflac(d, fresh=True)
    p, s = g.params, g.download()
    c = g.clock
    nx, nz = p.nx, p.nz
    lines = open(os.path.join(d, "_contents.0")).read().splitlines()
    assert len(lines) == 1
    nrec, nloop, tmy = lines[0].split()
    assert (int(nrec), int(nloop)) == (1, 60) and abs(float(tmy) - c.time / SEC_YEAR / 1e6) < 1e-6
    assert _records(os.path.join(d, "time.0"), np.float32, 1)[0, 0] == np.float32(c.time)
    f32 = np.float32
    exact = {
        "mesh.0": (s["cord"] / 1000).astype(f32),
        "vel.0": (s["vel"] * SEC_YEAR * 100).astype(f32),
        "temperature.0": s["temp"].astype(f32),
        "xoriginal.0": cord0[:, :, 0].astype(f32),
        "zoriginal.0": cord0[:, :, 1].astype(f32),
        "phase.0": s["iphase"],
        "topo.0": (s["cord"][0, :, 1] / 1000).astype(f32),
        "dtopo.0": np.zeros(nx, f32),
        "extrusion.0": np.zeros(nx - 1, f32),
    }
    for name, want in exact.items():
        got = _field(d, name, want.dtype, want.shape)
        assert np.array_equal(got, want), f"{name} differs"
    cool = (s["temp"] - s["temp0"]) / (c.dt / (SEC_YEAR * 1e6))
    got = _field(d, "coolingrate.0", f32, (nz, nx))
    assert np.allclose(got, cool, rtol=1e-6, atol=1e-6 * np.abs(cool).max() + 1e-30)
    ii = np.minimum(np.arange(nx), nx - 2)
    cond = np.array([p.conduct[k] for k in range(p.nphase)])[s["iphase"][0, ii] - 1]
    hfl = cond * (s["temp"][1] - s["temp"][0]) / (-(s["cord"][1, :, 1] - s["cord"][0, :, 1]) / 1000)
    got = _field(d, "hfl.0", f32, (nx,))
    assert np.allclose(got, hfl, rtol=1e-6, atol=1e-6 * np.abs(hfl).max())
    for name, want in _expected_elements(p, c, s).items():
        got = _field(d, name, f32, (nz - 1, nx - 1)).astype(np.float64)
        # the strain-rate averages are 0/0 right after an averaging reset
        # (dtavg = 0), in the reference as here
        fin = np.isfinite(want)
        assert np.array_equal(np.isfinite(got), fin), f"{name}: non-finite entries differ"
        if not fin.any():
            continue
        got, want = got[fin], want[fin]
        scale = max(float(np.abs(want).max()), 1e-300)
        err = float(np.abs(got - want).max()) / scale
        # log10 fields: absolute error in decades
        if name in ("srII.0", "visc.0"):
            err = float(np.abs(got - want).max())
        assert err <= tol, f"{name}: {err:.3e}"
    # a second frame is appended as record 2; record 1 stays
    first = {n: open(os.path.join(d, n), "rb").read() for n in ("mesh.0", "sII.0", "phase.0", "hfl.0")}
    g.step(10)
    g.outflac(d, fresh=False)
    lines = open(os.path.join(d, "_contents.0")).read().splitlines()
    assert [int(x.split()[0]) for x in lines] == [1, 2] and int(lines[1].split()[1]) == 70
    for n, b in first.items():
        now = open(os.path.join(d, n), "rb").read()
        assert len(now) == 2 * len(b) and now[: len(b)] == b, n
    s = g.download()
    got = _field(d, "mesh.0", f32, (nz, nx, 2), rec=2)
    assert np.array_equal(got, (s["cord"] / 1000).astype(f32))
    g.close()


def test_outmarker_matches_markers(workdir):
    _, g = _model(workdir, "convergence_60x15", "fp64")
    g.step(400)
    g.remesh()  # a remesh adds markers and kills some
    g.step(20)
    d = str(workdir / "markers")
    os.makedirs(d, exist_ok=True)
    g.outmarker(d, fresh=True)
    g.outmarker(d, fresh=False)
    s = g.download()
    c, nz = g.clock, g.params.nz
    nm = c.nmarkers
    lines = open(os.path.join(d, "_markers.0")).read().splitlines()
    assert [tuple(int(v) for v in x.split()[:3]) for x in lines] == [(1, c.nloop, nm), (2, c.nloop, nm)]
    for rec in (1, 2):
        m1 = _records(os.path.join(d, f"marker1.{rec:06d}.0"), np.float32, nm)
        m2 = _records(os.path.join(d, f"marker2.{rec:06d}.0"), np.int32, nm)
        assert m1.shape == (5, nm) and m2.shape == (3, nm)
        dead = s["mark_dead"][:nm]
        assert np.array_equal(m2[0], dead.astype(np.int32))
        assert np.array_equal(m2[1], s["mark_phase"][:nm].astype(np.int32))
        assert np.array_equal(m2[2], s["mark_ntriag"][:nm])
        a1, a2 = s["mark_a1"][:nm], s["mark_a2"][:nm]
        assert np.array_equal(m1[3], a1.astype(np.float32)) and np.array_equal(m1[4], a2.astype(np.float32))
        assert np.array_equal(m1[2], (s["mark_age"][:nm] / SEC_YEAR / 1e6).astype(np.float32))
        live = dead != 0
        n = s["mark_ntriag"][:nm][live].astype(np.int64)
        k = (n - 1) % 2 + 1
        jj = ((n - k) // 2) % (nz - 1)
        ii = (n - k) // 2 // (nz - 1)
        up = k == 1
        i1, i2, i3 = np.where(up, ii, ii + 1), ii, ii + 1
        j1, j2, j3 = jj, jj + 1, np.where(up, jj, jj + 1)
        b1, b2 = a1[live], a2[live]
        b3 = 1.0 - b1 - b2
        cd = s["cord"]
        x = cd[j1, i1, 0] * b1 + cd[j2, i2, 0] * b2 + cd[j3, i3, 0] * b3
        y = cd[j1, i1, 1] * b1 + cd[j2, i2, 1] * b2 + cd[j3, i3, 1] * b3
        assert np.allclose(m1[0][live], x * 1e-3, rtol=1e-6, atol=1e-4)
        assert np.allclose(m1[1][live], y * 1e-3, rtol=1e-6, atol=1e-4)
        assert (m1[0][~live] == 0).all() and (m1[1][~live] == 0).all()
    g.close()


def _read_restart(d, p, s):
    """The `*.rs` records read with numpy in the reference's layout."""
    nx, nz = p.nx, p.nz
    E, N = (nx - 1) * (nz - 1), nx * nz
    nrec, nloop, tmy, nm, _ = open(os.path.join(d, "_contents.rs")).read().split()
    nrec, nloop, nm = int(nrec), int(nloop), int(nm)
    t, dt = _records(os.path.join(d, "time.rs"), np.float64, 2)[nrec - 1]
    f8 = lambda n, k: _records(os.path.join(d, n), np.float64, k)[nrec - 1]
    s["cord"][...] = f8("cord.rs", 2 * N).reshape((nz, nx, 2), order="F")
    s["vel"][...] = f8("vel.rs", 2 * N).reshape((nz, nx, 2), order="F")
    s["strain"][...] = f8("strain.rs", 3 * E).reshape((nz - 1, nx - 1, 3), order="F")
    s["stress0"][...] = f8("stress.rs", 16 * E).reshape((nz - 1, nx - 1, 4, 4), order="F")
    s["temp"][...] = f8("temp.rs", N).reshape((nz, nx), order="F")
    ph = np.fromfile(os.path.join(d, "phase.rs"), dtype=np.int32).reshape(-1, 2 * E)[nrec - 1][:E]
    s["iphase"][...] = ph.reshape((nz - 1, nx - 1), order="F")
    for n, k in (("aps", "aps.rs"), ("fmagma", "fmagma.rs"), ("fmagma2", "fmagma2.rs"), ("source", "source.rs")):
        s[n][...] = f8(k, E).reshape((nz - 1, nx - 1), order="F")
    s["dhacc_correction"][...] = f8("dhacc_corr.rs", nx)
    m1 = _records(os.path.join(d, "marker1.rs"), np.float64, nm)
    m2 = _records(os.path.join(d, "marker2.rs"), np.int32, nm)
    s["mark_a1"][:nm], s["mark_a2"][:nm], s["mark_age"][:nm] = m1
    s["mark_dead"][:nm] = m2[0]
    s["mark_ntriag"][:nm] = m2[1]
    s["mark_phase"][:nm] = m2[2]
    amin = float(open(os.path.join(d, "Amin.rs")).read())
    # element marker lists (rsflac.f90:146-172)
    ids, cnt = s["mark_id_elem"], s["nmark_elem"]
    ids[...] = 0
    cnt[...] = 0
    for m in range(nm):
        if s["mark_dead"][m] == 0:
            continue
        n = int(s["mark_ntriag"][m])
        k = (n - 1) % 2 + 1
        j, i = ((n - k) // 2) % (nz - 1), (n - k) // 2 // (nz - 1)
        if cnt[j, i] == MAXM:
            continue
        ids[cnt[j, i], j, i] = m + 1
        cnt[j, i] += 1
    return nloop, t, dt, nm, amin


def test_saveflac_rsflac_round_trip_matches_oracle(workdir):
    inp, g1 = _model(workdir, "convergence_60x15", "fp64")
    g1.step(400)
    g1.remesh()
    g1.step(30)
    d = str(workdir / "restart")
    os.makedirs(d, exist_ok=True)
    g1.saveflac(d)
    shutil.copy(os.path.join(d, "_contents.save"), os.path.join(d, "_contents.rs"))
    s1 = g1.download()
    c1 = g1.clock
    # the files hold the saved state exactly
    p0, c0, s0 = new_state(inp)
    nloop, t, dt, nm, amin = _read_restart(d, p0, s0)
    assert (nloop, t, dt, nm) == (c1.nloop, c1.time, c1.dt, c1.nmarkers)
    assert amin == g1.params.Amin
    for f in ("cord", "vel", "strain", "stress0", "temp", "aps", "iphase", "source", "fmagma"):
        assert np.array_equal(s0[f], s1[f]), f
    for f in ("mark_a1", "mark_a2", "mark_age", "mark_dead", "mark_phase", "mark_ntriag"):
        assert np.array_equal(s0[f][:nm], s1[f][:nm]), f
    g2 = Flac.restart(inp, d, "fp64")
    assert g2.clock.nloop == c1.nloop and g2.clock.time == c1.time
    # the oracle: same files, marker2elem, the library's init_bc result
    # (host set-up code), then the rsflac tail
    c0.nloop, c0.time, c0.dt, c0.nmarkers = nloop, t, dt, nm
    p0.Amin = amin
    orc = Oracle(p0, c0, s0)
    orc.marker2elem()
    s2 = g2.download()
    assert np.array_equal(s0["iphase"], s2["iphase"]) and np.array_equal(s0["jmoho"], s2["jmoho"])
    s0["bc"][...] = s2["bc"]
    s0["ncod"][...] = s2["ncod"]
    for k in ("ivis_present", "vbc", "incoming_left", "incoming_right", "nopbmax", "dxmin", "dzmin"):
        setattr(p0, k, getattr(g2.params, k))
    orc.restart_tail()
    extra_f = ("temp0", "amass", "rmass", "visn", "e2sr", "se2sr", "area", "dvol", "mark_a1", "mark_a2")
    diffs, bad = compare_states(s2, s0, FLOAT_FIELDS + extra_f, INT_FIELDS)
    assert not bad, f"integer fields differ after the restart: {bad}"
    worst = max(diffs, key=diffs.get)
    assert diffs[worst] <= 1e-12, f"restart: {worst} differs by {diffs[worst]:.3e}"
    assert g2.clock.nmarkers == c0.nmarkers
    for k in ("dt", "dt_elastic", "dt_maxwell"):
        a, b = getattr(g2.clock, k), getattr(c0, k)
        assert abs(a - b) <= 1e-12 * abs(b), k
    g2.step(50)
    orc.step(50)
    s2 = g2.download()
    diffs, bad = compare_states(s2, s0, FLOAT_FIELDS, INT_FIELDS)
    assert not bad, f"integer fields differ 50 steps after the restart: {bad}"
    worst = max(diffs, key=diffs.get)
    assert diffs[worst] <= 1e-10, f"after restart: {worst} differs by {diffs[worst]:.3e}"
    g1.close()
    g2.close()


def test_rsflac_mixed_and_bad_files(workdir):
    inp, g1 = _model(workdir, "extension_60x20", "mixed")
    g1.step(100)
    d = str(workdir / "restart_mixed")
    os.makedirs(d, exist_ok=True)
    g1.saveflac(d)  # no _contents.rs: rsflac falls back to _contents.save
    s1 = {k: np.array(g1.download()[k]) for k in ("cord", "temp", "stress0")}
    g2 = Flac.restart(inp, d, "mixed")
    s2 = g2.download()
    assert np.array_equal(s2["cord"], s1["cord"]) and np.array_equal(s2["temp"], s1["temp"])
    sc = np.abs(s1["stress0"]).max()
    assert np.abs(s2["stress0"] - s1["stress0"]).max() <= 1e-6 * sc
    g2.step(20)
    s2 = g2.download()
    assert np.isfinite(s2["vel"]).all() and np.isfinite(s2["stress0"]).all()
    # a triangle number outside the mesh stops with 999, as the reference does
    m2 = os.path.join(d, "marker2.rs")
    raw = np.fromfile(m2, dtype=np.int32)
    nm = raw.size // 3
    live = np.nonzero(raw[:nm])[0][0]
    raw[nm + live] = 2 * (g1.params.nx - 1) * (g1.params.nz - 1) + 1
    raw.tofile(m2)
    p, c, s = new_state(inp)
    g3 = Flac(p, c, s, "mixed", finish_setflac=False)
    with pytest.raises(capi.GfError) as e:
        g3.rsflac(d)
    assert e.value.code == 999
    os.remove(os.path.join(d, "_contents.save"))
    with pytest.raises(capi.GfError) as e:
        g3.rsflac(d)
    assert e.value.code == -3
    for g in (g1, g2, g3):
        g.close()
