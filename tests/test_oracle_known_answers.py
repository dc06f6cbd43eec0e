"""Pins the oracle to the reference's analytic known answers
(examples/tutorial01-03 of the reference): the oracle must reproduce the
physics those tutorials verify before it can check the CUDA kernels.

* elastic bar in plane strain: E_eff = 4 mu (lambda+mu)/(lambda+2 mu) = 80 GPa
* Maxwell column under constant strain rate: sigma_xx(t) =
  4 eta edot (1 - exp(-t/tau)), tau = eta (lambda+2mu)/(mu (lambda+mu))
* Mohr-Coulomb bar: peak mean vertical stress = UCS = 2 c cos(phi)/(1 - sin(phi))
"""
import math

import numpy as np
import pytest

from geoflac_gb300 import capi, inpgen
from oracle.oracle import Oracle, new_state

SEC_YEAR = capi.SEC_YEAR


def _run(workdir, model, name, **kw):
    inp = model.write(str(workdir / f"{name}.inp"))
    p, c, s = new_state(inp, **kw)
    o = Oracle(p, c, s)
    o.finish_setflac()
    return o


def test_elastic_bar_modulus(workdir):
    o = _run(workdir, inpgen.elastic_bar(), "bar")
    s = o.s
    z0 = s["cord"][:, :, 1].copy()
    o.step(300)  # ~0.5% strain: small-strain regime
    uz = (s["cord"][:, :, 1] - z0).mean(axis=1)
    strain = np.polyfit(z0.mean(axis=1), uz, 1)[0]  # d(uz)/dz over the column
    szz = s["stress0"][:, :, 1, :].mean()
    e_eff = szz / strain
    lam = mu = 3e10
    expect = 4 * mu * (lam + mu) / (lam + 2 * mu)
    assert expect == pytest.approx(80e9)
    assert e_eff == pytest.approx(expect, rel=0.01)


def test_maxwell_relaxation_time(workdir):
    eta = 1e21
    model = inpgen.maxwell_column(eta)
    model.strain_inert = 1e-5  # quasi-static loading: no inertial overshoot
    o = _run(workdir, model, "maxwell")
    s, c = o.s, o.c
    L = s["cord"][0, -1, 0] - s["cord"][0, 0, 0]
    edot = -(0.1 * inpgen.CM_PER_YR) / L
    lam = mu = 3e10
    tau = eta * (lam + 2 * mu) / (mu * (lam + mu))
    assert tau == pytest.approx(5e10)
    sig_ss = 4 * eta * edot
    for _ in range(3):
        o.step(1000)
        t = c.time
        sxx = s["stress0"][:, :, 0, :].mean()
        expect = sig_ss * (1 - math.exp(-t / tau))
        assert sxx == pytest.approx(expect, rel=0.03)


def test_plastic_bar_ucs(workdir):
    model = inpgen.plastic_bar()
    model.strain_inert = 2e-5  # quasi-static loading (smaller steps)
    o = _run(workdir, model, "plastic")
    s = o.s
    peak = 0.0
    for _ in range(60):
        o.step(100)
        peak = min(peak, s["stress0"][:, :, 1, :].mean())
    c, phi = 2e7, math.radians(30.0)
    ucs = 2 * c * math.cos(phi) / (1 - math.sin(phi))
    assert ucs == pytest.approx(69.282e6, rel=1e-4)
    assert -peak == pytest.approx(ucs, rel=0.01)
