"""Ensemble driver (one persistent kernel per step over many models) against
the same models stepped one by one, through the C-ABI.

The batch runs the single-model device code per element and node.  Within
one compiled batch kernel the result of a member does not depend on the
company it keeps or on the tile depth: those are compared to the last bit.
Between differently compiled kernels (the single-model kernels, or batch
kernels built for another CTA width or register cap) the FP32 fields can
differ by FMA contraction; those are compared after 25 steps at rounding
level: coordinates and temperatures 1e-10, stresses and velocities 1e-5 of
the field's largest value, plastic strain 1e-6, integer fields exact.
"""
import numpy as np
import pytest

from geoflac_gb300 import capi, inpgen
from geoflac_gb300.batch import Batch
from geoflac_gb300.flac import Flac, new_state

from ._util import FLOAT_FIELDS, INT_FIELDS

pytestmark = pytest.mark.gpu

SMALL = (20, 8, 60, 20)  # mesh range of the test sweep


def _members(workdir, n, mode="mixed", tag="a"):
    out = []
    for k in range(n):
        m, _ = inpgen.ensemble_member(k, scale=SMALL)
        path = m.write(str(workdir / f"bm_{tag}_{k}.inp"))
        p, c, s = new_state(path)
        out.append(Flac(p, c, s, mode))
    return out


TOL = {"cord": 1e-10, "temp": 1e-10, "temp0": 1e-10, "vel": 1e-5, "stress0": 1e-5, "aps": 1e-6}


def _assert_close(a, b, where):
    a.download()
    b.download()
    for f in FLOAT_FIELDS + ("temp0",):
        x, y = np.asarray(a.state[f], dtype=np.float64), np.asarray(b.state[f], dtype=np.float64)
        scale = max(float(np.abs(y).max()), 1e-300)
        d = float(np.abs(x - y).max()) / scale
        assert d <= TOL.get(f, 1e-5), f"{where}: {f} differs by {d:.3e} of its largest value"
    for f in INT_FIELDS:
        assert np.array_equal(a.state[f], b.state[f]), f"{where}: {f} differs"
    assert a.clock.nloop == b.clock.nloop and a.clock.nsrate == b.clock.nsrate


def _assert_same(a, b, where):
    a.download()
    b.download()
    for f in FLOAT_FIELDS + ("temp0", "mark_a1", "mark_a2"):
        x, y = np.asarray(a.state[f]), np.asarray(b.state[f])
        assert np.array_equal(x, y), f"{where}: {f} differs by {np.abs(x - y).max():.3e}"
    for f in INT_FIELDS:
        assert np.array_equal(a.state[f], b.state[f]), f"{where}: {f} differs"
    for k in ("dt", "time", "dtavg", "dt_elastic", "dt_maxwell", "frac"):
        assert getattr(a.clock, k) == getattr(b.clock, k), f"{where}: clock {k}"
    assert a.clock.nloop == b.clock.nloop and a.clock.nsrate == b.clock.nsrate


@pytest.mark.parametrize("graph_steps", [0, 10])
def test_batch_matches_single_models(workdir, graph_steps):
    n = 6
    alone = _members(workdir, n, tag="s")
    batched = _members(workdir, n, tag="b")
    b = Batch(batched)
    b.set_config(threads=256, items_per_thread=2, ctas_per_sm=1, graph_steps=graph_steps)
    assert b.elements == sum((g.params.nx - 1) * (g.params.nz - 1) for g in batched)
    for g in alone:
        g.step(25)
    b.step(25)
    for k in range(n):
        _assert_close(batched[k], alone[k], f"member {k}")
    b.close()


def test_batch_member_independent_of_company(workdir):
    """A member in a batch of six evolves exactly as in a batch of one."""
    six = _members(workdir, 6, tag="six")
    one = _members(workdir, 6, tag="one")[3]
    b6, b1 = Batch(six), Batch([one])
    for b in (b6, b1):
        b.set_config(threads=256, items_per_thread=2, ctas_per_sm=1, graph_steps=10)
        b.step(25)
    _assert_same(six[3], one, "member 3")
    b6.close()
    b1.close()


def test_batch_shapes_agree(workdir):
    """Tile depth leaves the states unchanged to the bit; other CTA widths
    and residencies (separately compiled kernels: the residency selects a
    register-capped build) agree at rounding level."""
    ref = _members(workdir, 4, tag="r")
    rb = Batch(ref)
    rb.set_config(threads=256, items_per_thread=1, ctas_per_sm=1, graph_steps=0)
    rb.step(12)
    for threads, ipt, cps in ((256, 8, 1), (256, 2, 2), (128, 1, 2), (512, 4, 1)):
        ms = _members(workdir, 4, tag=f"{threads}_{ipt}_{cps}")
        b = Batch(ms)
        b.set_config(threads=threads, items_per_thread=ipt, ctas_per_sm=cps, graph_steps=0)
        b.step(12)
        for k in range(4):
            if threads == 256 and cps == 1:
                _assert_same(ms[k], ref[k], f"shape {threads}x{ipt}x{cps} member {k}")
            else:
                _assert_close(ms[k], ref[k], f"shape {threads}x{ipt}x{cps} member {k}")
        b.close()
    rb.close()


def test_batch_autotuner_picks_a_valid_shape(workdir):
    ms = _members(workdir, 8, tag="t")
    b = Batch(ms)
    best = b.tune(trial_steps=1)
    assert best["threads"] in (128, 256, 512)
    assert best["items_per_thread"] in (1, 2, 4, 8)
    assert best["ctas_per_sm"] >= 1 and best["ms_per_step"] > 0
    cfg = b.config()
    assert cfg["threads"] == best["threads"] and cfg["items_per_thread"] == best["items_per_thread"]
    b.step(5)
    for g in ms:
        g.download()
        assert np.isfinite(g.state["vel"]).all()
    b.close()


def test_batch_rejects_fp64_and_mismatched_schedules(workdir):
    ms = _members(workdir, 1, mode="fp64", tag="f")
    with pytest.raises(capi.GfError) as e:
        Batch(ms)
    assert e.value.code == -5
    a, c = _members(workdir, 2, tag="m")
    c.step(1)  # nloop differs
    with pytest.raises(capi.GfError) as e:
        Batch([a, c])
    assert e.value.code == -2


# members of the workload's own sweep (mesh 80x25 .. 400x120 quads): the
# smallest and largest of the first 40 draws, an extension and a convergence
SWEEP_MEMBERS = (4, 37, 1, 24)


def test_batch_sweep_members_against_single_models_and_oracle(workdir):
    """Members at the sweep's real sizes (84x26 .. 397x119 quads) advanced
    10 steps by the ensemble kernel: against the same members stepped alone
    by the single-model mixed kernels (rounding level, as above), and against
    the FP64 oracle from its own start-up state: coordinates 1e-8 and
    temperature 1e-9 of each field's largest value; stress 1e-6 and velocity
    2e-4 (the 60x20 / 60x15 10-step bounds) or, where the member itself is
    that sensitive, 3x the change a relative 1e-7 perturbation of its
    initial stresses makes in the oracle's FP64 run (the damping of
    fl_node.f90 switches with the sign of each nodal velocity); integer
    fields exact."""
    from oracle.oracle import Oracle

    from ._util import oracle_state, rel_diff

    batched, alone, orcs, perts = [], [], [], []
    for k in SWEEP_MEMBERS:
        m, _ = inpgen.ensemble_member(k)
        path = m.write(str(workdir / f"sweep_{k}.inp"))
        batched.append(Flac(*new_state(path), "mixed"))
        alone.append(Flac(*new_state(path), "mixed"))
        for perturb, lst in ((False, orcs), (True, perts)):
            p, c, st = oracle_state(path)
            if perturb:
                rng = np.random.default_rng(k)
                st["stress0"][...] *= 1 + 1e-7 * rng.choice([-1.0, 1.0], size=st["stress0"].shape)
            o = Oracle(p, c, st)
            o.finish_setflac()
            lst.append(o)
    sizes = [(g.params.nx - 1) * (g.params.nz - 1) for g in batched]
    assert min(sizes) < 2500 and max(sizes) > 45000
    b = Batch(batched)
    b.set_config(threads=256, items_per_thread=2, ctas_per_sm=2, graph_steps=10)
    b.step(10)
    for g in alone:
        g.step(10)
    for o in orcs + perts:
        o.step(10)
    fields = ("vel", "cord", "temp", "stress0", "aps")
    for k, (g, h, o, q) in enumerate(zip(batched, alone, orcs, perts)):
        who = SWEEP_MEMBERS[k]
        _assert_close(g, h, f"member {who} vs alone")
        err = {f: rel_diff(g.state[f], o.s[f]) for f in fields}
        sens = {f: rel_diff(q.s[f], o.s[f]) for f in fields}
        assert err["cord"] <= 1e-8 and err["temp"] <= 1e-9, (who, err)
        assert err["stress0"] <= max(1e-6, 3.0 * sens["stress0"]), (who, err, sens)
        assert err["vel"] <= max(2e-4, 3.0 * sens["vel"]), (who, err, sens)
        for f in ("iphase", "nmark_elem", "mark_ntriag"):
            assert np.array_equal(g.state[f], o.s[f]), (who, f)
        assert g.clock.nloop == o.c.nloop
    b.close()
    for g in batched + alone:
        g.close()
