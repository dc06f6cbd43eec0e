"""FP64 parity on the workload configurations themselves, through the C-ABI:

* the 1000x300 extension model with 25 markers per element (5 x 5 points),
  50 steps, a forced remesh event, 20 more steps: the multi-block reductions,
  tiles that span many columns, a thermal update that needs several sweeps and
  a remesh at scale, against the serial oracle;
* the basalt -> eclogite rule of the convergence model (change_phase.f90:159-170
  and the 600 C / 1.5 GPa option) on basalt seeded below the Moho.

Tolerances as in test_parity_gpu: floats within 1e-10 of each field's
largest magnitude, integer fields (marker elements, triangles, phases,
counts) bit-exact.
"""
import numpy as np
import pytest

from geoflac_gb300 import inpgen, new_state
from geoflac_gb300.flac import Flac
from oracle.oracle import Oracle

from ._util import FLOAT_FIELDS, INT_FIELDS, compare_states, oracle_state

pytestmark = pytest.mark.gpu

TOL = 1e-10
EXTRA_FLOATS = ("temp0", "source", "mark_a1", "mark_a2", "mark_age")
EXTRA_INTS = ("jmoho",)
KOCEAN1, KECLG = 3, 13


def _compare(gpu, orc, where, tol=TOL):
    gpu.download()
    assert gpu.clock.nmarkers == orc.c.nmarkers, f"{where}: nmarkers {gpu.clock.nmarkers} vs {orc.c.nmarkers}"
    diffs, bad = compare_states(gpu.state, orc.s, FLOAT_FIELDS + EXTRA_FLOATS, INT_FIELDS + EXTRA_INTS)
    assert not bad, f"{where}: integer fields differ: {bad}"
    worst = max(diffs, key=diffs.get)
    assert diffs[worst] <= tol, f"{where}: {worst} differs by {diffs[worst]:.3e} (all: {diffs})"
    for k in ("dt", "time", "dt_elastic", "dt_maxwell"):
        a, b = getattr(gpu.clock, k), getattr(orc.c, k)
        assert abs(a - b) <= tol * max(abs(b), 1e-300), f"{where}: clock {k} {a} vs {b}"
    assert gpu.clock.nloop == orc.c.nloop
    return diffs


def test_extension_1000x300_25_markers_with_remesh(workdir):
    inp = inpgen.extension_1000x300().write(str(workdir / "extension_1000x300_25.inp"))
    p, c, s = new_state(inp, markers_per_side=5)
    E = (p.nx - 1) * (p.nz - 1)
    assert (p.nx, p.nz) == (1001, 301)
    # 25 markers in every element, each inside its own element at start-up
    assert c.nmarkers == 25 * E
    assert np.all(s["nmark_elem"] == 25)
    p2, c2, s2 = oracle_state(inp, markers_per_side=5)
    orc = Oracle(p2, c2, s2)
    orc.finish_setflac()
    gpu = Flac(p, c, s, "fp64")
    _compare(gpu, orc, "setflac")
    for _ in range(2):
        gpu.step(25)
        orc.step(25)
        _compare(gpu, orc, f"step {orc.c.nloop}")
    # several thermal sweeps per step on this mesh, none at the cap
    assert 2 <= gpu.clock.therm_sweeps < 24 and gpu.clock.therm_unconverged == 0
    orc.remesh_event()
    gpu.remesh()
    _compare(gpu, orc, "remesh")
    gpu.step(20)
    orc.step(20)
    _compare(gpu, orc, "20 steps after remesh")
    gpu.close()


def _seed_basalt(p, s):
    """Basalt (kocean1) markers in a block of elements below the Moho of the
    convergence model, under temperatures that rise along x from 450 to
    1050 C, so that the two eclogite rules select different elements."""
    nz1, nx1 = p.nz - 1, p.nx - 1
    ids, nm, ph = s["mark_id_elem"], s["nmark_elem"], s["mark_phase"]
    j0, j1 = 2, min(nz1, 8)
    i0, i1 = nx1 // 3, 2 * nx1 // 3
    for i in range(i0, i1):
        for j in range(j0, j1):
            ph[ids[:nm[j, i], j, i] - 1] = KOCEAN1
            cnt = np.bincount(ph[ids[:nm[j, i], j, i] - 1], minlength=p.nphase + 1)[1:p.nphase + 1]
            s["phase_ratio"][:, j, i] = cnt / nm[j, i]
            s["iphase"][j, i] = int(np.argmax(cnt)) + 1
    T = s["temp"]
    for i in range(i0, i1 + 1):
        T[j0:j1 + 1, i] = 450.0 + 600.0 * (i - i0) / (i1 - i0)


@pytest.mark.parametrize("rule", [0, 1])
def test_eclogite_rule_matches_oracle(workdir, rule):
    inp = inpgen.convergence_60x15().write(str(workdir / f"convergence_60x15_ecl{rule}.inp"))
    p, c, s = new_state(inp, eclogite_rule=rule)
    assert p.eclogite_rule == rule
    _seed_basalt(p, s)
    p2, c2, s2 = oracle_state(inp, eclogite_rule=rule)
    _seed_basalt(p2, s2)
    orc = Oracle(p2, c2, s2)
    orc.finish_setflac()
    gpu = Flac(p, c, s, "fp64")
    for _ in range(3):
        gpu.step(10)
        orc.step(10)
        _compare(gpu, orc, f"rule {rule} step {orc.c.nloop}")
    nm = orc.c.nmarkers
    ecl = int(np.count_nonzero(orc.s["mark_phase"][:nm] == KECLG))
    # the seeded basalt turns into eclogite under both rules, on different markers
    assert ecl > 0
    test_eclogite_rule_matches_oracle.counts[rule] = ecl
    if len(test_eclogite_rule_matches_oracle.counts) == 2:
        a, b = test_eclogite_rule_matches_oracle.counts[0], test_eclogite_rule_matches_oracle.counts[1]
        assert a != b, "the 600 C / 1.5 GPa rule and Hacker's lines select the same markers"
    gpu.close()


test_eclogite_rule_matches_oracle.counts = {}
