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


def test_marker_lcg_matches_published_recurrence():
    """myrandom_mod.f90: iseed = mod(8121*iseed + 28411, 134456)."""
    seeds = []
    k = 0
    for _ in range(5):
        k = (8121 * (k % 134456) + 28411) % 134456
        seeds.append(k / 134456)
    assert seeds[0] == 28411 / 134456
    assert all(0 <= v < 1 for v in seeds)


def test_winkler_pisos(workdir):
    """nyhydro = 2: pisos is the lithostatic pressure at the base of the last
    column (init_stress.f90:400-403)."""
    p, c, s = new_state(inpgen.convergence_60x15().write(str(workdir / "c3.inp")))
    rho_g_h = 0.0
    assert p.pisos > 0
    col = s["stress0"][:, -1, 1, 0]
    # pisos exceeds the pressure at the centre of the deepest element
    assert p.pisos > -col[-1]
    assert rho_g_h == 0.0
