"""Host side, no GPU: the .inp reader (read_params.f90 semantics) and the
start-up state (setflac chain) the kernels begin from."""
import glob
import os

import numpy as np
import pytest

from geoflac_gb300 import capi, inpgen, new_state

REF = "/root/reference"


def test_generated_configs_round_trip(workdir):
    for name, make in inpgen.CONFIGS.items():
        m = make()
        p = capi.read_params(m.write(str(workdir / f"{name}.inp")))
        assert (p.nx, p.nz) == (m.nex + 1, m.nez + 1)
        assert p.nphase == len(m.phases)
        assert p.nofbc == len(m.bcs)
        assert p.rxbo == m.rxbo and p.rzbo == m.rzbo
        for k, ph in enumerate(m.phases):
            assert p.irheol[k] == ph.irheol and p.den[k] == ph.den and p.cohesion1[k] == ph.coh1
        assert p.time_max == pytest.approx(m.time_max_kyr * 1000 * capi.SEC_YEAR)


def test_list_directed_forms(workdir):
    """Repeat counts, D exponents, trailing remarks and values continued on
    the next line, as Fortran list-directed input allows."""
    txt = inpgen.extension_60x20().text().splitlines()
    # the viscosity line "v_min, v_max, 2, 500.0" -> D exponent, split across lines
    i = next(k for k, s in enumerate(txt) if s.startswith("1e+20") or s.startswith("100000000000000000000"))
    txt[i] = "1.0D20,"
    txt.insert(i + 1, "  3.0d27  2 500.0 ; remark")
    # the four process frequencies written as a repeat count on one line
    j = next(k for k, s in enumerate(txt) if s.startswith("; ---- process control"))
    path = workdir / "forms.inp"
    path.write_text("\n".join(txt) + "\n")
    p = capi.read_params(str(path))
    assert p.v_min == 1e20 and p.v_max == 3e27 and p.ivis_shape == 2 and p.efoldc == 500.0
    assert j > 0


def test_parse_error_is_reported(workdir):
    path = workdir / "bad.inp"
    path.write_text("; only a comment\n60,20\n")
    with pytest.raises(capi.GfError) as e:
        capi.read_params(str(path))
    assert e.value.code == -4


@pytest.mark.skipif(not os.path.isdir(REF), reason="reference inputs not mounted")
def test_reference_inputs_parse():
    files = sorted(glob.glob(f"{REF}/benchmark/*.inp") + glob.glob(f"{REF}/examples/**/*.inp", recursive=True))
    assert files
    for f in files:
        p = capi.read_params(f)
        assert p.nx > 1 and p.nz > 1 and 1 <= p.nphase <= 20, f


def test_setflac_host_state(workdir):
    m = inpgen.extension_60x20()
    p, c, s = new_state(m.write(str(workdir / "c1.inp")))
    nex, nez = m.nex, m.nez
    # uniform mesh
    x = s["cord"][0, :, 0]
    assert np.allclose(np.diff(x), m.rxbo / nex)
    assert np.allclose(s["cord"][:, 0, 1], np.linspace(0, m.rzbo, nez + 1))
    # 9 markers per element, each inside its element's triangle
    assert c.nmarkers == 9 * nex * nez
    assert (s["nmark_elem"] == 9).all()
    n = c.nmarkers
    a1, a2 = s["mark_a1"][:n], s["mark_a2"][:n]
    assert (a1 >= 0).all() and (a2 >= 0).all() and (a1 + a2 <= 1).all()
    ntr = s["mark_ntriag"][:n]
    e_of_marker = (ntr - 1) // 2
    ids = s["mark_id_elem"].reshape(32, -1, order="F")
    for e in (0, 17, nex * nez - 1):
        mine = ids[:9, e] - 1
        assert (e_of_marker[mine] == e).all()
    # crust (phase 2) above 30 km, mantle (phase 4) below
    zc = 0.25 * (s["cord"][:-1, :-1, 1] + s["cord"][1:, :-1, 1] + s["cord"][:-1, 1:, 1] + s["cord"][1:, 1:, 1])
    ip = s["iphase"]
    assert (ip[zc > -29e3] == 2).all() and (ip[zc < -31e3] == 4).all()
    # linear geotherm 0 -> 1330 C at 100 km depth
    assert np.allclose(s["temp"][:, 0], -s["cord"][:, 0, 1] * 1e-3 * 13.3)
    # lithostatic prestress grows with depth; weak seed through aps = 0.1
    sxx = s["stress0"][:, 0, 0, 0]
    assert (np.diff(sxx) < 0).all()
    assert np.isclose(s["aps"].max(), 0.1) and (s["aps"] > 0).sum() == 9
    # side walls pulled apart at 1 cm/yr, free-slip base
    v = inpgen.CM_PER_YR
    assert (s["ncod"][:, 0, 0] == 1).all() and np.allclose(s["bc"][:, 0, 0], -v)
    assert (s["ncod"][:, -1, 0] == 1).all() and np.allclose(s["bc"][:, -1, 0], v)
    assert (s["ncod"][-1, :, 1] == 1).all() and (s["bc"][-1, :, 1] == 0).all()
    assert p.vbc == pytest.approx(v)
    # inverse double areas of the four triangles of a 5 km x 5 km quad
    assert np.allclose(s["area"], 1.0 / (5e3 * 5e3))


def _myrandom(seed):
    """myrandom_mod.f90:9-19: iseed = mod(8121*mod(iseed,134456) + 28411, 134456), r = iseed/134456."""
    seed = seed % 134456
    seed = (8121 * seed + 28411) % 134456
    return seed, seed / 134456


def _marker_xy(s, ids):
    """marker2xy (bar2euler.f90:73-117) in numpy: positions of markers `ids`
    (1-based) from their triangle and barycentric coordinates."""
    cord = s["cord"]
    nz1 = cord.shape[0] - 1
    n = s["mark_ntriag"][ids - 1].astype(np.int64)
    k = (n - 1) % 2 + 1
    jj = ((n - k) // 2) % nz1
    ii = (n - k) // 2 // nz1
    a1, a2 = s["mark_a1"][ids - 1], s["mark_a2"][ids - 1]
    a3 = 1.0 - a1 - a2
    i1 = np.where(k == 1, ii, ii + 1)
    j2, i2 = jj + 1, ii
    j3 = np.where(k == 1, jj, jj + 1)
    i3 = ii + 1
    x = cord[jj, i1, 0] * a1 + cord[j2, i2, 0] * a2 + cord[j3, i3, 0] * a3
    y = cord[jj, i1, 1] * a1 + cord[j2, i2, 1] * a2 + cord[j3, i3, 1] * a3
    return x, y


@pytest.mark.parametrize("ms", [3, 5])
def test_marker_positions_follow_the_lcg_chain(workdir, ms):
    """init_marker.f90:30-128 restated in numpy for the first mesh column:
    the serial LCG chain (seed += i + j per element, two draws per point),
    the point pattern (the reference's 1/6-1/2-5/6 weights for 3 x 3; the
    same construction at (2m+1)/(2 ms) for ms x ms) and a jitter of one point
    spacing; the product's start-up markers sit at these positions, in this
    order, with the layer phase of their depth."""
    m = inpgen.extension_60x20()
    p, c, s = new_state(m.write(str(workdir / f"lcg{ms}.inp")), markers_per_side=ms)
    cord = s["cord"]
    if ms == 3:
        w1 = np.array([0.1666666666666666666666, 0.5, 0.8333333333333333333333])
        w0 = np.array([0.8333333333333333333333, 0.5, 0.1666666666666666666666])
    else:
        w1 = (2.0 * np.arange(ms) + 1.0) / (2.0 * ms)
        w0 = 1.0 - w1
    seed = 0
    i = 0
    for j in range(p.nz - 1):
        ax = cord[j, i, 0] * w0 + cord[j + 1, i, 0] * w1
        ay = cord[j, i, 1] * w0 + cord[j + 1, i, 1] * w1
        bx = cord[j, i + 1, 0] * w0 + cord[j + 1, i + 1, 0] * w1
        by = cord[j, i + 1, 1] * w0 + cord[j + 1, i + 1, 1] * w1
        px = (ax[:, None] * w0[None, :] + bx[:, None] * w1[None, :]).ravel()
        py = (ay[:, None] * w0[None, :] + by[:, None] * w1[None, :]).ravel()
        dx = cord[j, i + 1, 0] - cord[j, i, 0]
        dy = cord[j + 1, i, 1] - cord[j, i, 1]
        seed = seed + (i + 1) + (j + 1)
        xs, ys = [], []
        for q in range(ms * ms):
            seed, rx = _myrandom(seed)
            seed, ry = _myrandom(seed)
            xs.append(px[q] + dx * (0.5 - rx) / ms)
            ys.append(py[q] + dy * (0.5 - ry) / ms)
        ids = s["mark_id_elem"][:ms * ms, j, i]
        assert s["nmark_elem"][j, i] == ms * ms
        x, y = _marker_xy(s, ids)
        assert np.allclose(x, xs, rtol=0, atol=1e-6) and np.allclose(y, ys, rtol=0, atol=1e-6), (j, i)
        # crust above 30 km depth, mantle below (the age zone's layer)
        expect_ph = np.where(np.array(ys) * -1e-3 < 30.0, 2, 4)
        assert np.array_equal(s["mark_phase"][ids - 1], expect_ph)
    # the draws are the recurrence's: the first is 8121 * 2 + 28411
    assert _myrandom(2) == ((8121 * 2 + 28411) % 134456, ((8121 * 2 + 28411) % 134456) / 134456)


def test_hydrostatic_prestress_and_winkler_pisos(workdir):
    """init_stress.f90:16-51 restated in numpy from the start-up mesh,
    phases and temperatures: every column's pressure at each element centre
    (oceanic columns under 8 km of water) is the element's -sxx = -szz = -syy,
    and with nyhydro = 2 pisos is the pressure at the base of the last column."""
    p, c, s = new_state(inpgen.convergence_60x15().write(str(workdir / "c3.inp")))
    assert p.nyhydro == 2
    cord, temp, iph = s["cord"], s["temp"], s["iphase"]
    den = np.array([p.den[k] for k in range(p.nphase)])
    alfa = np.array([p.alfa[k] for k in range(p.nphase)])
    beta = np.array([p.beta[k] for k in range(p.nphase)])
    st = s["stress0"]
    pisos = 0.0
    for i in range(p.nx - 1):
        rogh = -1030.0 * p.g * 8.0e3 if iph[0, i] in (3, 7) else 0.0
        for j in range(p.nz - 1):
            ph = iph[j, i] - 1
            tmpr = 0.25 * (temp[j, i] + temp[j + 1, i] + temp[j, i + 1] + temp[j + 1, i + 1])
            densT = den[ph] * (1 - alfa[ph] * tmpr)
            dh = 0.5 * ((cord[j, i, 1] - cord[j + 1, i, 1]) + (cord[j, i + 1, 1] - cord[j + 1, i + 1, 1]))
            dPT = densT * p.g * dh
            dP = dPT * (1 - beta[ph] * rogh) / (1 + beta[ph] / 2 * dPT)
            press = rogh + 0.5 * dP
            for k in range(4):
                assert st[j, i, 0, k] == pytest.approx(-press, rel=1e-13)
                assert st[j, i, 1, k] == pytest.approx(-press, rel=1e-13)
                assert st[j, i, 2, k] == 0.0
                assert st[j, i, 3, k] == pytest.approx(-press, rel=1e-13)
            rogh = rogh + dP
        if i == p.nx - 2:
            pisos = rogh + p.extra_pres
    assert pisos > 0
    assert p.pisos == pytest.approx(pisos, rel=1e-13)


def _struct_diff(a, b):
    """Fields of two ctypes structures whose bytes differ."""
    import ctypes as C

    out = []
    for name, _ in a._fields_:
        f = getattr(type(a), name)
        if C.string_at(C.addressof(a) + f.offset, f.size) != C.string_at(C.addressof(b) + f.offset, f.size):
            out.append(name)
    return out


@pytest.mark.parametrize("name", sorted(inpgen.CONFIGS))
@pytest.mark.parametrize("ms", [3, 5])
def test_oracle_startup_equals_library_startup(workdir, name, ms):
    """The oracle builds its initial state on its own (read_params and the
    setflac chain restated from the Fortran: init_cord, init_phase,
    init_marker with its serial LCG chain, check_visc_rheol, init_areas,
    init_temp, init_stress, init_bc, vbcal); the library's host start-up
    gives the same parameters, clock and arrays bit for bit."""
    from oracle.oracle import new_state as oracle_new_state

    path = inpgen.CONFIGS[name]().write(str(workdir / f"st_{name}_{ms}.inp"))
    p1, c1, s1 = new_state(path, markers_per_side=ms)
    p2, c2, s2 = oracle_new_state(path, markers_per_side=ms)
    assert _struct_diff(p1, p2) == []
    assert _struct_diff(c1, c2) == []
    bad = [k for k in s1.arrays if not np.array_equal(s1.arrays[k], s2.arrays[k])]
    assert bad == []
    assert c2.nmarkers == ms * ms * (p2.nx - 1) * (p2.nz - 1)


@pytest.mark.skipif(not os.path.isdir(REF), reason="reference inputs not mounted")
def test_oracle_reads_reference_inputs_like_the_library():
    from oracle.oracle import read_params as oracle_read_params

    files = sorted(glob.glob(f"{REF}/benchmark/*.inp") + glob.glob(f"{REF}/examples/**/*.inp", recursive=True))
    assert files
    for f in files:
        assert _struct_diff(capi.read_params(f), oracle_read_params(f)) == [], f
