"""Writers of GeoFLAC ``.inp`` parameter files for the workloads of this
package.

The file layout is the reference's positional format read by
``src/read_params.f90:3-348`` (one READ per non-comment line, ``;`` starts a
comment line).  The workloads are seeded synthetic models:

* ``extension_60x20``  -- two-phase extension, 60x20 quads, 300 km x 100 km (CPU-sized)
* ``extension_1000x300``  -- the same physics at 1000x300 quads, 1000 km x 300 km,
                  remeshing when a triangle angle falls below 10 degrees
* ``convergence``  -- ocean-continent convergence, 600x150 quads, 1200 km x 300 km,
                  Winkler foundation, basalt -> eclogite
* ``elastic_bar``, ``maxwell_column``, ``plastic_bar`` -- the analytic
  known-answer set-ups described by the reference's tutorials 01-03
  (examples/tutorial0{1,2,3}-*/tutorial.md)

Phase ids follow the reference's special ids (src/phases.f90): continental
crust is phase 2 (kcont1), mantle is phase 4 (kmant1), oceanic basalt is
phase 3 (kocean1), sediment phase 11 (ksed2), eclogite phase 13 (keclg), so
that change_phase applies its rules to the right materials.
"""
from __future__ import annotations

from dataclasses import dataclass, field
from typing import List, Sequence

CM_PER_YR = 0.01 / 3.1558e7  # m/s


@dataclass
class Phase:
    irheol: int = 12
    den: float = 2800.0
    alfa: float = 3e-5
    beta: float = 0.0
    n: float = 3.0
    A: float = 5e2
    E: float = 1.9e5
    V: float = 0.0
    rl: float = 3e10
    rm: float = 3e10
    pls1: float = 0.0
    pls2: float = 0.1
    fric1: float = 30.0
    fric2: float = 30.0
    coh1: float = 4e7
    coh2: float = 4e6
    dil1: float = 0.0
    dil2: float = 0.0
    cond: float = 3.0
    cp: float = 1000.0

    def line(self) -> str:
        v = [self.irheol, 1, self.den, self.alfa, self.beta, self.n, self.A, self.E, self.V,
             self.rl, self.rm, self.pls1, self.pls2, self.fric1, self.fric2, self.coh1,
             self.coh2, self.dil1, self.dil2, self.cond, self.cp, 13000, 16000, 16000, 1]
        return ", ".join(_fmt(x) for x in v)


@dataclass
class BC:
    side: int  # 1 left, 2 bottom, 3 right, 4 top
    n1: int
    n2: int
    nbc: int  # 10 vx, 1 vz, 200 flexural bottom
    a: float
    b: float = 0.0  # second coefficient (nbc 200: the fluid's density)


@dataclass
class AgeZone:
    ictherm: int
    age: float
    tp1: float
    tp2: float
    ix1: int
    ix2: int
    hc: Sequence[float]  # layer depths (km), len = nlayers - 1
    phases: Sequence[int]


@dataclass
class Inhom:
    ix1: int
    ix2: int
    iy1: int
    iy2: int
    phase: int
    geom: int
    aps: float


@dataclass
class Model:
    nex: int
    nez: int
    x0: float = 0.0
    z0: float = 0.0
    rxbo: float = 300e3
    rzbo: float = -100e3
    bcs: List[BC] = field(default_factory=list)
    nyhydro: int = 0
    pisos: float = 0.0
    iphsub: int = 4
    drosub: float = 0.0
    g: float = 10.0
    itherm: int = 1
    istress_therm: int = 0
    ishearh: int = 1
    t_top: float = 0.0
    t_bot: float = 1330.0
    hs: float = 0.0
    hr: float = 10.0
    itemp_bc: int = 1
    bot_bc: float = 1330.0
    zones: List[AgeZone] = field(default_factory=list)
    phases: List[Phase] = field(default_factory=list)
    inhoms: List[Inhom] = field(default_factory=list)
    ten_off: float = 1e9
    tau_heal: float = 0.0
    v_min: float = 1e20
    v_max: float = 3e27
    ny_rem: int = 0
    mode_rem: int = 1
    ntest_rem: int = 100
    angle_rem: float = 10.0
    idt_scale: int = 2
    dt_scale: float = 1.0
    strain_inert: float = 5e-4
    i_rey: int = 1
    xReyn: float = 5.0
    ifreq: int = 10
    topo_kappa: float = 0.0  # surface diffusion (diff_topo); 0 = off
    # magma sub-model (read_params.f90:243-255); itype_melting 0 = off
    itype_melting: int = 0
    nelem_dike: int = 1
    prod_magma: float = 2e-15
    prod_magma2: float = 0.0
    rho_magma: float = 2700.0
    angle_mzone: float = 30.0
    fmagma_max: float = 0.1
    ratio_mantle_mzone: float = 0.1
    ratio_crust_mzone: float = 0.1
    latent_heat_magma: float = 420000.0
    lambda_freeze: float = 1e-13
    lambda_freeze_tdep: float = 0.002
    weaken_ratio_plastic: float = 1.0
    weaken_ratio_viscous: float = 1.0
    frac: float = 0.45
    fracm: float = 0.5
    demf: float = 0.8
    mix_strain: int = 1
    mix_stress: int = 1
    time_max_kyr: float = 1e6

    def text(self) -> str:
        L: List[str] = []
        c = L.append
        c("; GeoFLAC parameter file written by geoflac_gb300.inpgen")
        c("; ---- mesh: elements in x and z, origin, extent")
        c(f"{self.nex},{self.nez}")
        c(f"{_fmt(self.x0)},{_fmt(self.z0)}")
        c(f"{_fmt(self.rxbo)},{_fmt(self.rzbo)}")
        c("; ircoord, coordinate file")
        c("0, points.xy")
        c("; x zones (0 = uniform)")
        c("0")
        c("; z zones (0 = uniform)")
        c("0")
        c("; ---- mechanical conditions: nystressbc, nydrsides")
        c("0  0")
        c("; number of boundary conditions")
        c(f"{len(self.bcs)}")
        c("; side  nbc1 nbc2 nbc  a b c d e f g h i")
        for b in self.bcs:
            nbc = "01" if b.nbc == 1 else str(b.nbc)
            c(f"{b.side} {b.n1} {b.n2} {nbc} {_fmt(b.a)} {_fmt(b.b)} 0 0 0 0 0 0 0")
        c("; hydrostatic pressure: nyhydro, pisos, iphsub, drosub, damp_vis")
        c(f"{self.nyhydro} {_fmt(self.pisos)} {self.iphsub} {_fmt(self.drosub)} 0.0")
        c("; gravity")
        c(_fmt(self.g))
        c("; ---- thermal: i_prestress, extra_pres, itherm, istress_therm, ishearh, t_top, t_bot")
        c("0")
        c("0.0")
        c(f"{self.itherm}")
        c(f"{self.istress_therm}")
        c(f"{self.ishearh}")
        c(_fmt(self.t_top))
        c(_fmt(self.t_bot))
        c("; radiogenic heating hs, hr")
        c(f"{_fmt(self.hs)}, {_fmt(self.hr)}")
        c("; bottom temperature bc: type, value")
        c(f"{self.itemp_bc} {_fmt(self.bot_bc)}")
        c("; irtemp, temperature file")
        c("0")
        c("proftemp.dat")
        c("; number of age zones; per zone: ictherm, age, tp1, tp2, ix1, ix2 / layers / phases")
        c(f"{len(self.zones)}")
        for z in self.zones:
            c(f" {z.ictherm}, {_fmt(z.age)}, {_fmt(z.tp1)}, {_fmt(z.tp2)}, {z.ix1}, {z.ix2}")
            hc = " ".join(_fmt(h) for h in z.hc)
            c(f"    {len(z.phases)}, {hc}".rstrip(", "))
            c("    " + " ".join(str(p) for p in z.phases))
        c("; ---- rheology: number of phases, then one line per phase")
        c(f"{len(self.phases)}")
        for ph in self.phases:
            c(ph.line())
        c("; irphase, phase file")
        c("0")
        c("phasedat.inp")
        c("; inhomogeneities: ix1 ix2 iy1 iy2 phase geometry aps")
        c(f"{len(self.inhoms)}")
        for h in self.inhoms:
            c(f"{h.ix1} {h.ix2} {h.iy1} {h.iy2} {h.phase} {h.geom} {_fmt(h.aps)}")
        c("; tension cut-off")
        c(_fmt(self.ten_off))
        c("; healing time")
        c(_fmt(self.tau_heal))
        c("; viscosity limits: v_min, v_max, ivis_shape, efoldc")
        c(f"{_fmt(self.v_min)}, {_fmt(self.v_max)}, 2, 500.0")
        c("; magma: itype_melting, nelem_serp, nelem_dike, prod_magma, prod_magma2, rho_magma")
        c(f"{self.itype_melting}, 2, {self.nelem_dike}, {_fmt(self.prod_magma)}, {_fmt(self.prod_magma2)}, "
          f"{_fmt(self.rho_magma)}")
        c("; angle_mzone, fmagma_max, ratio_mantle_mzone, ratio_crust_mzone")
        c(f"{_fmt(self.angle_mzone)}, {_fmt(self.fmagma_max)}, {_fmt(self.ratio_mantle_mzone)}, "
          f"{_fmt(self.ratio_crust_mzone)}")
        c("; latent_heat_magma, lambda_freeze, lambda_freeze_tdep")
        c(f"{_fmt(self.latent_heat_magma)}, {_fmt(self.lambda_freeze)}, {_fmt(self.lambda_freeze_tdep)}")
        c("; weaken_ratio_plastic, weaken_ratio_viscous")
        c(f"{_fmt(self.weaken_ratio_plastic)}, {_fmt(self.weaken_ratio_viscous)}")
        c("; ---- remeshing: ny_rem, mode_rem, ntest_rem, angle_rem")
        c(f"{self.ny_rem}  {self.mode_rem}  {self.ntest_rem}  {_fmt(self.angle_rem)}")
        c("; dx_rem")
        c("1.3")
        c("; topography diffusion: topo_kappa, fac_kappa")
        c(f"{_fmt(self.topo_kappa)}  0.0")
        c("; ---- process control")
        c(f"{self.idt_scale}")
        c(f"{_fmt(self.dt_scale)},{_fmt(self.strain_inert)}")
        c(f"{self.i_rey},{_fmt(self.xReyn)}")
        for _ in range(4):
            c(f"{self.ifreq}")
        c(f"{_fmt(self.frac)},{_fmt(self.fracm)}")
        c("1,2")
        c(f"{_fmt(self.demf)},{self.mix_strain},{self.mix_stress}")
        c("; ---- output: time_max (kyr), screen, file intervals (kyr), flags, lastout, save")
        c(_fmt(self.time_max_kyr))
        c("1000.0")
        c("1000.0")
        c("  " + "   ".join(["1"] * 19))
        c("0")
        c("1000.0")
        c("1")
        return "\n".join(L) + "\n"

    def write(self, path: str) -> str:
        with open(path, "w") as f:
            f.write(self.text())
        return path


def _fmt(x) -> str:
    if isinstance(x, int):
        return str(x)
    return repr(float(x))


def crust(**kw) -> Phase:
    base = dict(irheol=12, den=2800.0, n=3.0, A=5e2, E=1.9e5, fric1=30.0, fric2=30.0,
                coh1=4e7, coh2=4e6)
    base.update(kw)
    return Phase(**base)


def mantle(**kw) -> Phase:
    base = dict(irheol=12, den=3300.0, n=3.5, A=7e4, E=5.2e5, fric1=30.0, fric2=30.0,
                coh1=4e7, coh2=4e6)
    base.update(kw)
    return Phase(**base)


def two_phase_extension(nex: int, nez: int, width: float, depth: float,
                        crust_km: float = 30.0, half_rate_cm_yr: float = 1.0,
                        ny_rem: int = 0, seed_size: int = 3) -> Model:
    """Crust over mantle pulled apart at both walls; linear geotherm
    0 C -> 1330 C at 100 km (ictherm 21); a seed_size^2-element weak seed at
    the centre of the crust starts fully softened (cohesion 4 MPa) through its
    initial plastic strain (igeom 0, phase -1 keeps the crust phase)."""
    v = half_rate_cm_yr * CM_PER_YR
    ph = [crust(), crust(), crust(), mantle()]  # ids 1..4; 1 and 3 unused
    nzn = nez + 1
    nxn = nex + 1
    rows_crust = max(1, round(crust_km * 1e3 / (depth / nez)))
    cx = nex // 2
    cy = max(1, rows_crust // 2)
    h = seed_size // 2
    m = Model(nex=nex, nez=nez, rxbo=width, rzbo=-depth,
              bcs=[BC(1, 1, nzn, 10, -v), BC(3, 1, nzn, 10, v), BC(2, 1, nxn, 1, 0.0)],
              zones=[AgeZone(21, 100.0, 0.0, 0.0, 1, nxn, [crust_km], [2, 4])],
              phases=ph,
              inhoms=[Inhom(cx - h + 1, cx - h + seed_size, cy - h + 1, cy - h + seed_size,
                            -1, 0, 0.1)],
              ny_rem=ny_rem, ntest_rem=100)
    return m


def extension_60x20() -> Model:
    return two_phase_extension(60, 20, 300e3, 100e3)


def extension_1000x300() -> Model:
    return two_phase_extension(1000, 300, 1000e3, 300e3, ny_rem=1)


def convergence(nex: int = 600, nez: int = 150) -> Model:
    """Ocean-continent convergence: 60-Myr half-space cooling oceanic plate
    (7 km basalt, 1 km weak sediment) on the left, 35 km continental crust on
    the right, left wall pushing at 5 cm/yr, Winkler foundation."""
    nxn, nzn = nex + 1, nez + 1
    v = 5.0 * CM_PER_YR
    ph = [crust() for _ in range(13)]
    ph[1] = crust()  # 2: continental crust
    ph[2] = crust(den=3000.0, n=3.05, A=0.125, E=3.76e5)  # 3: basalt
    ph[3] = mantle()  # 4: mantle
    ph[10] = crust(fric1=5.0, fric2=5.0, coh1=4e6, coh2=4e6)  # 11: sediment
    ph[12] = crust(den=3400.0, n=3.05, A=0.125, E=4.5e5)  # 13: eclogite
    half = nxn // 2
    zones = [AgeZone(1, 60.0, 0.0, 0.0, 1, half, [1.0, 8.0], [11, 3, 4]),
             AgeZone(21, 100.0, 0.0, 0.0, half + 1, nxn, [35.0], [2, 4])]
    return Model(nex=nex, nez=nez, rxbo=1200e3, rzbo=-300e3,
                 bcs=[BC(1, 1, nzn, 10, v), BC(3, 1, nzn, 10, 0.0)],
                 nyhydro=2, iphsub=4, zones=zones, phases=ph, ntest_rem=100)


def elastic_bar() -> Model:
    """Tutorial 01: 3x10 elements, 1000 m x 3000 m, elastic (irheol 1),
    lambda = mu = 3e10 Pa, no gravity, bottom vz = 0, top vz = -1e-9 m/s.
    Analytic plane-strain modulus E_eff = 4 mu (lambda+mu)/(lambda+2mu) = 80 GPa."""
    # phase id 2 (kcont1) has no change_phase rule; id 1 would turn into sediment
    ph = [Phase(irheol=1, den=2700.0, alfa=0.0)] * 2
    return Model(nex=3, nez=10, rxbo=1000.0, rzbo=-3000.0,
                 bcs=[BC(2, 1, 4, 1, 0.0), BC(4, 1, 4, 1, -1e-9)],
                 g=0.0, ishearh=0, t_bot=0.0, bot_bc=0.0,
                 zones=[AgeZone(21, 100.0, 0.0, 0.0, 1, 4, [], [2])],
                 phases=ph, v_min=1e19, ntest_rem=100, mix_strain=0, mix_stress=0)


def maxwell_column(eta: float = 1e21) -> Model:
    """Tutorial 02: 40x10 elements, 20 km x 5 km, Maxwell (irheol 3) with a
    constant viscosity eta (v_min = v_max = eta), left wall pushing at
    0.1 cm/yr, right wall fixed, free top, free-slip base, no gravity.
    Analytic tau_eff = eta (lambda+2mu)/(mu (lambda+mu)) = 5e10 s."""
    ph = [Phase(irheol=3, den=2700.0, alfa=0.0, n=1.0, A=1.0, E=0.0)] * 2
    return Model(nex=40, nez=10, rxbo=20e3, rzbo=-5e3,
                 bcs=[BC(1, 1, 11, 10, 0.1 * CM_PER_YR), BC(3, 1, 11, 10, 0.0),
                      BC(2, 1, 41, 1, 0.0)],
                 g=0.0, ishearh=0, t_bot=0.0, bot_bc=0.0,
                 zones=[AgeZone(21, 100.0, 0.0, 0.0, 1, 41, [], [2])],
                 phases=ph, v_min=eta, v_max=eta, ntest_rem=100)


def plastic_bar() -> Model:
    """Tutorial 03: 10x30 elements, 1000 m x 3000 m, Mohr-Coulomb (irheol 6),
    cohesion 20 MPa, friction 30 deg, no dilation, no gravity; bottom vz = 0,
    top vz = -1e-9 m/s and vx = 0.  Analytic UCS = 2 c cos(phi)/(1-sin(phi))
    = 69.282 MPa."""
    ph = [Phase(irheol=6, den=2700.0, alfa=0.0, coh1=2e7, coh2=2e6, fric1=30.0, fric2=30.0)] * 2
    return Model(nex=10, nez=30, rxbo=1000.0, rzbo=-3000.0,
                 bcs=[BC(2, 1, 11, 1, 0.0), BC(4, 1, 11, 1, -1e-9), BC(4, 1, 11, 10, 0.0)],
                 g=0.0, ishearh=0, t_bot=0.0, bot_bc=0.0,
                 zones=[AgeZone(21, 100.0, 0.0, 0.0, 1, 11, [], [2])],
                 phases=ph, v_min=1e19, ntest_rem=100)


def convergence_60x15() -> Model:
    """The ocean-continent convergence model on a 60x15 mesh (CPU-sized
    parity case)."""
    return convergence(60, 15)


def magma_arc(nex: int = 60, nez: int = 15) -> Model:
    """The convergence model with all 19 phase ids of the reference's
    special rules, the magma sub-model on (itype_melting 1: melting, dikes, mantle percolation,
    the MOR pool with eruption) and surface diffusion (which carries the
    arc-extrusion and MOR-crust blocks).  The melting itself is set up by
    the caller (temperatures, subducted phases)."""
    m = convergence(nex, nez)
    m.phases = m.phases + [crust() for _ in range(19 - len(m.phases))]
    m.phases[13] = crust(den=2800.0)  # 14: arc crust
    m.phases[15] = mantle()  # 16: hydrated mantle
    m.phases[17] = mantle()  # 18: dry mantle
    m.itype_melting = 1
    m.nelem_dike = 3
    m.prod_magma = 2e-13
    m.prod_magma2 = 1e-11
    m.topo_kappa = 1e-6
    return m


CONFIGS = {"extension_60x20": extension_60x20, "extension_1000x300": extension_1000x300, "convergence_600x150": convergence, "convergence_60x15": convergence_60x15,
           "elastic_bar": elastic_bar, "maxwell_column": maxwell_column,
           "plastic_bar": plastic_bar, "magma_arc": magma_arc}


# ---------------------------------------------------------------- ensembles
ENSEMBLE_SEED = 20261203
ELEMENT_KM = 2.5  # element edge of the ensemble meshes (aspect-matched domains)


def ensemble_member(k: int, seed: int = ENSEMBLE_SEED, scale: tuple = (80, 25, 400, 120)):
    """Member k of the parameter sweep: mesh drawn between 80x25 and
    400x120 quads (both sides from one draw, so the domain keeps its aspect,
    2.5 km elements), crust friction 10-35 deg, crust thickness 25-45 km,
    Moho temperature 400-800 C (piecewise-linear geotherm, ictherm 22, 1330 C
    at 100 km or the base), wall velocity 0.5-5 cm/yr, extension or
    convergence.  Returns (Model, the 4 sampled parameters)."""
    import numpy as np
    rng = np.random.default_rng([seed, k])
    s = rng.uniform()
    nex = int(round(scale[0] + s * (scale[2] - scale[0])))
    nez = int(round(scale[1] + s * (scale[3] - scale[1])))
    fric = float(rng.uniform(10.0, 35.0))
    crust_km = float(rng.uniform(25.0, 45.0))
    moho_t = float(rng.uniform(400.0, 800.0))
    v_cm = float(rng.uniform(0.5, 5.0)) * (1.0 if rng.uniform() < 0.5 else -1.0)
    width, depth = nex * ELEMENT_KM * 1e3, nez * ELEMENT_KM * 1e3
    m = two_phase_extension(nex, nez, width, depth, crust_km=crust_km, half_rate_cm_yr=v_cm)
    m.phases[1] = crust(fric1=fric, fric2=fric)
    base_km = min(100.0, depth / 1e3)
    m.zones = [AgeZone(22, moho_t, crust_km, base_km, 1, nex + 1, [crust_km], [2, 4])]
    return m, {"friction": fric, "crust_km": crust_km, "moho_t": moho_t, "v_cm_yr": v_cm}
