"""FP64 parity of the CUDA step against the oracle (serial FP64 restatement
of the reference's Fortran), through the C-ABI.

Tolerances: floating-point fields within 1e-10 relative to the field's
largest magnitude (the normalisation of benchmark/compare.py); integer
fields (iphase, marker element/triangle indices, phase counts) bit-exact.
"""
import numpy as np
import pytest

from geoflac_gb300 import capi, inpgen, new_state
from geoflac_gb300.flac import Flac
from oracle.oracle import Oracle

from ._util import compare_states, oracle_state, rel_diff

pytestmark = pytest.mark.gpu

TOL = 1e-10
ROUTINES = ("fl_therm", "change_phase", "fl_rheol", "fl_node", "fl_move", "rmasses", "dt_mass", "init_visc")


def _pair(workdir, name, mode="fp64", **kw):
    inp = inpgen.CONFIGS[name]().write(str(workdir / f"{name}.inp"))
    p, c, s = new_state(inp, **kw)
    p2, c2, s2 = oracle_state(inp, **kw)
    orc = Oracle(p2, c2, s2)
    orc.finish_setflac()
    gpu = Flac(p, c, s, mode)
    return gpu, orc


def _assert_close(gpu, orc, tol=TOL, where=""):
    gpu.download()
    diffs, bad = compare_states(gpu.state, orc.s)
    worst = max(diffs, key=diffs.get)
    assert not bad, f"{where}: integer fields differ: {bad}"
    assert diffs[worst] <= tol, f"{where}: {worst} differs by {diffs[worst]:.3e} (all: {diffs})"
    for k in ("dt", "time", "dtavg", "dt_elastic", "dt_maxwell"):
        a, b = getattr(gpu.clock, k), getattr(orc.c, k)
        assert abs(a - b) <= tol * max(abs(b), 1e-300), f"{where}: clock {k} {a} vs {b}"
    assert gpu.clock.nloop == orc.c.nloop and gpu.clock.nsrate == orc.c.nsrate
    return diffs


@pytest.mark.parametrize("name", ["extension_60x20", "convergence_60x15"])
def test_setflac_parity(workdir, name):
    """The library's start-up state finished on the device (rmasses,
    init_visc, dt_mass) against the oracle's own read_params, setflac chain
    and finish."""
    gpu, orc = _pair(workdir, name)
    _assert_close(gpu, orc, where="setflac")
    gpu.close()


@pytest.mark.parametrize("routine", ROUTINES)
def test_each_routine_matches_oracle(workdir, routine):
    """Advance 37 steps with the oracle, give both the same state, then run
    one reference subroutine on each side and compare every field."""
    gpu, orc = _pair(workdir, "convergence_60x15")
    orc.step(37)
    gpu.state.copy_from(orc.s)
    C = gpu.clock
    for k, _ in capi.GfClock._fields_:
        setattr(C, k, getattr(orc.c, k))
    gpu.upload()
    getattr(orc, routine)()
    getattr(gpu, routine)()
    diffs = _assert_close(gpu, orc, where=routine)
    # the FP64 kernels round exactly as the serial reference: bit-exact
    assert max(diffs.values()) == 0.0, diffs
    gpu.close()


@pytest.mark.parametrize("name,steps", [("extension_60x20", 1000), ("convergence_60x15", 600)])
def test_steps_match_oracle(workdir, name, steps):
    """The full step (flac.f90) over many steps: captured-graph driver vs
    the serial oracle, checked every 100 steps."""
    gpu, orc = _pair(workdir, name)
    done = 0
    while done < steps:
        n = min(100, steps - done)
        orc.step(n)
        gpu.step(n)
        done += n
        _assert_close(gpu, orc, where=f"{name} step {done}")
    gpu.close()


def test_plastic_strain_branches_match_oracle(workdir):
    """pre_plast + the plastic constants of single-phase elements come from a
    per-phase table for plastic strain before softening, exactly at its
    start and after it; other elements compute them.  On the 60x20
    extension model with softening between plastic strain 0.02 and 0.2,
    elements get strains in every branch (0, 0.02 exactly, inside the
    interval, 0.2 and beyond; crust, mantle and the mixed rows at the
    Moho), and fl_rheol then matches the oracle bit for bit, as do 50 steps."""
    m = inpgen.extension_60x20()
    for ph in m.phases:
        ph.pls1, ph.pls2 = 0.02, 0.2
    inp = m.write(str(workdir / "pls_branches.inp"))
    p, c, s = new_state(inp)
    p2, c2, s2 = oracle_state(inp)
    orc = Oracle(p2, c2, s2)
    orc.finish_setflac()
    orc.step(20)
    aps = orc.s["aps"]
    levels = np.array([0.0, 0.02, 0.05, 0.2, 0.7])
    jj, ii = np.indices(aps.shape)
    aps[...] = levels[(jj + 3 * ii) % levels.size]
    # phase mixtures: columns 10-14 with 60 % of their own phase and 40 % of
    # another, columns 20-24 with a 0.005 trace of another phase (below the
    # 0.01 cut-off of pre_plast) beside a ratio of exactly 1
    pr, iph = orc.s["phase_ratio"], orc.s["iphase"]
    for i in range(10, 15):
        for j in range(pr.shape[1]):
            own = iph[j, i] - 1
            pr[:, j, i] = 0.0
            pr[own, j, i] = 0.6
            pr[(own + 2) % p.nphase, j, i] = 0.4
    for i in range(20, 25):
        for j in range(pr.shape[1]):
            pr[(iph[j, i] - 1 + 1) % p.nphase, j, i] = 0.005
    gpu = Flac(p, c, s, "fp64")
    gpu.state.copy_from(orc.s)
    for k, _ in capi.GfClock._fields_:
        setattr(gpu.clock, k, getattr(orc.c, k))
    gpu.upload()
    orc.fl_rheol()
    gpu.fl_rheol()
    diffs = _assert_close(gpu, orc, where="fl_rheol")
    assert max(diffs.values()) == 0.0, diffs
    orc.step(50)
    gpu.step(50)
    _assert_close(gpu, orc, where="50 steps")
    gpu.close()


def test_graph_step_equals_flac_calls(workdir):
    """gf_step(n) (graph replay) and n gf_flac calls give identical bits."""
    a, _ = _pair(workdir, "extension_60x20")
    b, _ = _pair(workdir, "extension_60x20")
    a.step(25)
    for _ in range(25):
        b.flac()
    a.download()
    b.download()
    for f in ("cord", "vel", "temp", "stress0", "aps", "amass"):
        assert np.array_equal(a.state[f], b.state[f]), f
    a.close()
    b.close()


def test_thermal_fixed_point_is_exact(workdir):
    """The in-place (Gauss-Seidel) thermal update of fl_therm.f90 is
    reproduced bit for bit: the sweeps reach their fixed point well below
    the cap, and the temperatures equal the serial oracle's exactly."""
    gpu, orc = _pair(workdir, "extension_60x20")
    for _ in range(30):
        orc.fl_therm()
        gpu.fl_therm()
    gpu.download()
    assert gpu.clock.therm_unconverged == 0
    assert 1 <= gpu.clock.therm_sweeps < 24
    assert np.array_equal(gpu.state["temp"], orc.s["temp"])
    gpu.close()


def test_thermal_sweep_cap_reports_unconverged(workdir):
    """A cap below the number of sweeps needed is reported, not hidden."""
    inp = inpgen.extension_60x20().write(str(workdir / "c1cap.inp"))
    p, c, s = new_state(inp, therm_sweeps=1)
    g = Flac(p, c, s, "fp64")
    g.fl_therm()
    g.download(0)
    assert g.clock.therm_unconverged == 1
    g.close()


def test_maxwell_stop_code(workdir):
    """A viscosity far below the Maxwell limit makes the reference stop with
    code 22 (rh_maxwell.f90:24-30); the GPU path returns the same code."""
    gpu, orc = _pair(workdir, "extension_60x20")
    gpu.download()
    gpu.state["visn"][...] = 1e10
    gpu.upload(capi.F_VISN)
    orc.s["visn"][...] = 1e10
    orc.c.nloop = 1
    with pytest.raises(RuntimeError, match="status 22"):
        orc.fl_rheol()
    with pytest.raises(capi.GfError) as e:
        # no Eff_visc refresh on this step (nloop % ifreq_visc != 0)
        gpu.clock.nloop = 1
        gpu.upload(0)
        gpu.fl_rheol()
    assert e.value.code == 22
    gpu.close()


def test_negative_area_stop_code(workdir):
    """Velocities that fold an element make fl_move stop with code 40
    (fl_move.f90:110-126) on both sides."""
    gpu, orc = _pair(workdir, "extension_60x20")
    gpu.download()
    v = gpu.state["vel"]
    v[...] = 0.0
    v[5, 10, 0] = 1e6  # one node crosses its neighbours in one step
    orc.s["vel"][...] = v
    gpu.upload(capi.F_VEL)
    with pytest.raises(RuntimeError, match="status 40"):
        orc.fl_move()
    with pytest.raises(capi.GfError) as e:
        gpu.fl_move()
    assert e.value.code == 40
    gpu.close()
