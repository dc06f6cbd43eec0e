// ORACLE -- test infrastructure only, never part of the product path.
//
// Serial FP64 restatement of GeoFLAC's explicit time step, written from the
// reference's Fortran (tan2/geoflac, src/*.f90) loop by loop, in the same
// evaluation order (left-to-right sums, no FMA contraction: build with
// -ffp-contract=off).  With one thread it is the parity oracle for the CUDA
// kernels; with OpenMP threads (loops parallelised where the reference has
// `!$OMP do`) it is the timed host baseline.
//
// It builds its own initial state from the .inp file (read_params and the
// setflac chain, restated below) and works on the reference's column-major
// array layout through the interface structures of include/geoflac_gb300.h
// (gf_params / gf_clock / gf_layout), so that a test can start the library
// and the oracle from the same file, advance both and compare every field.
// The one piece of code it shares with the library is the deterministic
// FP64 exp/log/pow/sin/tan of geoflac_gb300/csrc/gf_math.h, which the tests
// check against the C library (and or_set_libm switches the oracle's
// transcendentals to the C library's, to measure how far that moves a run).
//
// Parity pinning: the reference cannot be compiled in this environment (no
// Fortran compiler), and it commits no golden outputs.  The oracle is pinned
// by the reference's known-answer tutorials (elastic bar E_eff = 80 GPa,
// Maxwell relaxation time 1.584 kyr, Mohr-Coulomb UCS 69.282 MPa) and by
// hand-derived identities; see tests/test_oracle_known_answers.py.

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <string>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "../include/geoflac_gb300.h"
#include "../geoflac_gb300/csrc/gf_math.h"

namespace {

// Index helpers of the reference's column-major layout (src/arrays.f90),
// 0-based: node (j,i) is cord(j+1,i+1,:), element (j,i) is
// stress0(j+1,i+1,:,:); the depth index j runs fastest.
struct ODims {
    int nx, nz, nphase;
    long long N; // nodes
    long long E; // elements
};
inline long long o_node(const ODims &d, int j, int i) { return (long long)i * d.nz + j; }
inline long long o_elem(const ODims &d, int j, int i) { return (long long)i * (d.nz - 1) + j; }
// cord(j,i,k), vel, bc, ncod: plane k (0 x, 1 z) of nz*nx values
inline long long o_n2(const ODims &d, int j, int i, int k) { return k * d.N + o_node(d, j, i); }
// stress0(j,i,c,k): component c (sxx, szz, sxz, syy) of triangle k
inline long long o_s(const ODims &d, long long e, int c, int k) { return (long long)(c + 4 * k) * d.E + e; }
// area(j,i,k), dvol, strain, se2sr: plane k of E values
inline long long o_ek(const ODims &d, long long e, int k) { return (long long)k * d.E + e; }
// phase_ratio(ph,j,i): the phase index runs fastest
inline long long o_pr(const ODims &d, long long e, int ph) { return e * d.nphase + ph; }

// myrandom (src/myrandom_mod.f90:9-19): r in [0,1), the seed updated
inline double o_myrandom(int &iseed) {
    iseed = iseed % 134456;
    iseed = (8121 * iseed + 28411) % 134456;
    return (iseed * 1.0) / 134456;
}

// Transcendentals of the step: the deterministic FP64 implementation the
// library's kernels use (gf_math.h, so that both sides round alike), or,
// after or_set_libm(1), the C library's (to measure how far the choice
// moves a run; the library's kernels always use gf_math.h).
bool g_libm = false;
inline double o_exp(double x) { return g_libm ? std::exp(x) : gfm::exp(x); }
inline double o_pow(double x, double y) { return g_libm ? std::pow(x, y) : gfm::pow(x, y); }
inline double o_sin(double x) { return g_libm ? std::sin(x) : gfm::sin(x); }
inline double o_tan(double x) { return g_libm ? std::tan(x) : gfm::tan(x); }

int g_threads = 1;

struct Stop {
    int code;
};

struct St {
    gf_params *p;
    gf_clock *c;
    gf_layout *L;
    ODims d;
    double cord(int j, int i, int k) const { return L->cord[o_n2(d, j, i, k)]; }
    double &cordr(int j, int i, int k) { return L->cord[o_n2(d, j, i, k)]; }
    double vel(int j, int i, int k) const { return L->vel[o_n2(d, j, i, k)]; }
    double &temp(int j, int i) { return L->temp[o_node(d, j, i)]; }
    long long e(int j, int i) const { return o_elem(d, j, i); }
    double area(long long e, int k) const { return L->area[o_ek(d, e, k)]; }
    double &st(long long e, int c, int k) { return L->stress0[o_s(d, e, c, k)]; }
    // phase_ratio(iph, e) with the reference's flat-memory semantics for a
    // phase id above nphase (read the neighbouring entries, 0 past the end)
    double pr(long long e, int iph1) const {
        long long off = (long long)(iph1 - 1) + (long long)p->nphase * e;
        long long total = (long long)p->nphase * d.E;
        if (off < 0 || off >= total) return 0.0;
        return L->phase_ratio[off];
    }
};

St make(gf_params *p, gf_clock *c, gf_layout *L) {
    return St{p, c, L, ODims{p->nx, p->nz, p->nphase, (long long)p->nx * p->nz, (long long)(p->nx - 1) * (p->nz - 1)}};
}

// --------------------------------------------------------------------------
// Material functions (src/matprops.f90)

// Eff_dens (matprops.f90:3-83).  Writes the global `frac` exactly where the
// reference does (matprops.f90:37-39, 48-50); the caller passes the slot.
double eff_dens(St &s, int j, int i, double *frac_slot) {
    const gf_params &p = *s.p;
    double adi_grad = 3e-1, den_ramp_dist = 30e3, amp410 = 0.05, amp660 = 0.085;
    long long e = s.e(j, i);
    double zcord = 0.25 * (s.cord(j, i, 1) + s.cord(j + 1, i, 1) + s.cord(j, i + 1, 1) + s.cord(j + 1, i + 1, 1));
    double tmpr0 = 0.25 * (s.L->temp[o_node(s.d, j, i)] + s.L->temp[o_node(s.d, j + 1, i)] +
                           s.L->temp[o_node(s.d, j, i + 1)] + s.L->temp[o_node(s.d, j + 1, i + 1)]);
    double zsurf = 0.50 * (s.cord(0, i, 1) + s.cord(0, i + 1, 1));
    double tmpr = (zsurf - zcord) * 1e-3 * adi_grad + tmpr0;
    int iph = s.L->iphase[e];
    double deptmpr410 = -101.58 * (tmpr + 273.0) - 216828.0;
    double deptmpr420 = deptmpr410 - den_ramp_dist;
    double den_amp = 1.0;
    if (deptmpr410 > zcord) {
        double f = (deptmpr410 - zcord) / (deptmpr410 - deptmpr420);
        if (f < 0.0) f = 0.0;
        if (f > 1.0) f = 1.0;
        *frac_slot = f;
        den_amp = 1.0 + amp410 * f;
    }
    double deptmpr660 = 66.55 * (tmpr + 273.0) - 788494.0;
    double deptmpr670 = deptmpr660 - den_ramp_dist;
    if (deptmpr660 > zcord) {
        double f = (deptmpr660 - zcord) / (deptmpr660 - deptmpr670);
        if (f < 0.0) f = 0.0;
        if (f > 1.0) f = 1.0;
        *frac_slot = f;
        den_amp = 1.05 + amp660 * f;
    }
    double press = 0;
    for (int k = 0; k < 4; ++k)
        press = press - (s.L->stress0[o_s(s.d, e, 0, k)] + s.L->stress0[o_s(s.d, e, 1, k)] + s.L->stress0[o_s(s.d, e, 3, k)]);
    press = press / 12;
    double ed = 0.0;
    for (int k = 0; k < p.nphase; ++k) {
        double ratio = s.L->phase_ratio[o_pr(s.d, e, k)];
        if (ratio < 0.01) continue;
        double dens = p.den[k] * (1 - p.alfa[k] * tmpr + p.beta[k] * press);
        press = dens * p.g * zcord;
        dens = p.den[k] * (1 - p.alfa[k] * tmpr + p.beta[k] * press);
        ed = ed + ratio * dens;
    }
    if (iph == 4 || iph == 8 || iph == 9 || iph == 16 || iph == 18) ed = ed * den_amp;
    double fm = (s.L->fmagma ? s.L->fmagma[e] : 0.0) + (s.L->fmagma2 ? s.L->fmagma2[e] : 0.0);
    double fma = std::min(fm, p.fmagma_max);
    ed = ed - fma * (ed - p.rho_magma);
    return ed;
}

// Eff_visc (matprops.f90:136-215); i, j are 0-based.
double eff_visc(St &s, int j, int i) {
    const gf_params &p = *s.p;
    for (int k = 0; k < p.inhom; ++k)
        if (p.igeom[k] == 100 && i + 1 >= p.ix1[k] && i + 1 <= p.ix2[k] && j + 1 >= p.iy1[k] && j + 1 <= p.iy2[k])
            return p.v_min;
    long long e = s.e(j, i);
    double adi_grad = 3e-1, r = 8.31448;
    double zcord = 0.25 * (s.cord(j, i, 1) + s.cord(j + 1, i, 1) + s.cord(j, i + 1, 1) + s.cord(j + 1, i + 1, 1));
    double tmpr0 = 0.25 * (s.L->temp[o_node(s.d, j, i)] + s.L->temp[o_node(s.d, j + 1, i)] +
                           s.L->temp[o_node(s.d, j, i + 1)] + s.L->temp[o_node(s.d, j + 1, i + 1)]);
    double zsurf = 0.50 * (s.cord(0, i, 1) + s.cord(0, i + 1, 1));
    double tmpr = (zsurf - zcord) * 1e-3 * adi_grad + tmpr0;
    double s11 = 0.25 * (s.st(e, 0, 0) + s.st(e, 0, 1) + s.st(e, 0, 2) + s.st(e, 0, 3));
    double s22 = 0.25 * (s.st(e, 1, 0) + s.st(e, 1, 1) + s.st(e, 1, 2) + s.st(e, 1, 3));
    double s33 = 0.25 * (s.st(e, 3, 0) + s.st(e, 3, 1) + s.st(e, 3, 2) + s.st(e, 3, 3));
    double pres = -1 * (s11 + s22 + s33) / 3.0;
    double deptmpr410 = -101.58 * (tmpr + 273.0) - 216828.0;
    double deptmpr660 = 66.55 * (tmpr + 273.0) - 788494.0;
    double ev;
    if (zcord < deptmpr660) {
        ev = 1e22 * o_exp(-0.0115 * (tmpr - p.t_bot));
        return std::min(p.v_max, std::max(p.v_min, ev));
    } else if (zcord < deptmpr410) {
        ev = 1e21 * o_exp(-0.0115 * (tmpr - p.t_bot));
        return std::min(p.v_max, std::max(p.v_min, ev));
    }
    double srat = s.L->e2sr[e];
    if (srat == 0) srat = p.vbc / p.rxbo;
    ev = 0.0;
    for (int k = 0; k < p.nphase; ++k) {
        double ratio = s.L->phase_ratio[o_pr(s.d, e, k)];
        if (ratio < 0.01) continue;
        double pw = 1.0 / p.pln[k] - 1.0;
        double pw1 = -1.0 / p.pln[k];
        double vis = 0.25 * o_pow(srat, pw) * o_pow(0.75 * p.acoef[k], pw1) *
                     o_exp((p.eactiv[k] + p.vactiv[k] * pres) / (p.pln[k] * r * (tmpr + 273.0))) * 1e6;
        if (vis < p.v_min) vis = p.v_min;
        if (vis > p.v_max) vis = p.v_max;
        ev = ev + ratio / vis;
    }
    ev = 1 / ev;
    double fm = (s.L->fmagma ? s.L->fmagma[e] : 0.0) + (s.L->fmagma2 ? s.L->fmagma2[e] : 0.0);
    double fma = std::min(fm, p.fmagma_max);
    if (p.itype_melting == 1) ev = ev * o_exp(p.weaken_ratio_viscous * fma / p.fmagma_max);
    return std::min(p.v_max, std::max(p.v_min, ev));
}

// --------------------------------------------------------------------------
// Constitutive updates (src/rh_elastic.f90, rh_maxwell.f90, rh_plastic.f90)

void elastic(double bulkm, double rmu, double &s11, double &s22, double &s33, double &s12, double de11, double de22,
             double de12) {
    const double c4d3 = 4.0 / 3.0, c2d3 = 2.0 / 3.0;
    double a1 = bulkm + c4d3 * rmu;
    double a2 = bulkm - c2d3 * rmu;
    s11 = s11 + a1 * de11 + a2 * de22;
    s22 = s22 + a2 * de11 + a1 * de22;
    s12 = s12 + 2 * rmu * de12;
    s33 = s33 + a2 * (de11 + de22);
}

void maxwell(double bulkm, double rmu0, double viscosity, double &s11, double &s22, double &s33, double &s12, double de11,
             double de22, double de33, double de12, double dv, int ndim, double dt) {
    const double c1d3 = 1.0 / 3.0, visc_cut = 1e19;
    double rmu = viscosity < visc_cut ? rmu0 * viscosity / visc_cut : rmu0;
    double temp = rmu / (2 * viscosity) * dt;
    if (temp > 0.5) throw Stop{22};
    double vic1 = 1 - temp;
    double vic2 = 1.0 / (1.0 + temp);
    double dev, de11d, de22d, de33d, s0, s11d, s22d, s33d;
    if (ndim == 2) {
        dev = de11 + de22;
        de11d = de11 - 0.5 * dev;
        de22d = de22 - 0.5 * dev;
        de33d = 0;
        s0 = 0.5 * (s11 + s22);
        s11d = s11 - s0;
        s22d = s22 - s0;
        s33d = 0;
    } else {
        dev = de11 + de22 + de33;
        de11d = de11 - c1d3 * dev;
        de22d = de22 - c1d3 * dev;
        de33d = de33 - c1d3 * dev;
        s0 = c1d3 * (s11 + s22 + s33);
        s11d = s11 - s0;
        s22d = s22 - s0;
        s33d = s33 - s0;
    }
    s11d = (s11d * vic1 + 2 * rmu * de11d) * vic2;
    s22d = (s22d * vic1 + 2 * rmu * de22d) * vic2;
    s33d = (s33d * vic1 + 2 * rmu * de33d) * vic2;
    s12 = (s12 * vic1 + 2 * rmu * de12) * vic2;
    s0 = s0 + bulkm * dv;
    s11 = s11d + s0;
    s22 = s22d + s0;
    s33 = s33d + s0;
}

void plastic(double bulkm, double rmu, double coh, double phi, double psi, double &depls, double hardn, double &s11,
             double &s22, double &s33, double &s12, double de11, double de22, double de33, double de12, double ten_off,
             int ndim) {
    const double pi = 3.14159265358979323846;
    const double degrad = pi / 180.0;
    const double c4d3 = 4.0 / 3.0, c2d3 = 2.0 / 3.0;
    depls = 0.0;
    double sphi = o_sin(phi * degrad);
    double spsi = o_sin(psi * degrad);
    double anphi = (1.0 + sphi) / (1.0 - sphi);
    double anpsi = (1.0 + spsi) / (1.0 - spsi);
    double amc = 2.0 * coh * std::sqrt(anphi);
    double e1 = bulkm + c4d3 * rmu;
    double e2 = bulkm - c2d3 * rmu;
    double x1 = (e1 - e2 * anpsi + e1 * anphi * anpsi - e2 * anphi);
    double ten_max = (phi == 0.0) ? ten_off : std::min(ten_off, coh / (o_tan(phi * degrad)));
    double s11i = s11 + (de22 + de33) * e2 + de11 * e1;
    double s22i = s22 + (de11 + de33) * e2 + de22 * e1;
    double s12i = s12 + de12 * 2.0 * rmu;
    double s33i = s33 + (de11 + de22) * e2 + de33 * e1;
    double sdif = s11i - s22i;
    double s0 = 0.5 * (s11i + s22i);
    double rad = 0.5 * std::sqrt(sdif * sdif + 4.0 * s12i * s12i);
    double si = s0 - rad, sii = s0 + rad, psdif = si - sii;
    int icase = 1;
    double s1 = si, s2 = s33i, s3 = sii;
    if (ndim == 3) {
        if (s33i > sii) {
            icase = 3; s1 = si; s2 = sii; s3 = s33i;
        } else if (s33i < si) {
            icase = 2; s1 = s33i; s2 = si; s3 = sii;
        } else {
            icase = 1; s1 = si; s2 = s33i; s3 = sii;
        }
    }
    if (s1 >= ten_max) {
        s11 = ten_max; s22 = ten_max; s12 = 0.0; s33 = ten_max;
        return;
    }
    if (s2 >= ten_max && ndim == 3) {
        s2 = ten_max;
        s3 = ten_max;
    }
    if (s3 >= ten_max) s3 = ten_max;
    double fs = s1 - s3 * anphi + amc;
    if (fs < 0.0) {
        double alams = fs / (x1 + hardn);
        s1 = s1 - alams * (e1 - e2 * anpsi);
        s2 = s2 - alams * e2 * (1.0 - anpsi);
        s3 = s3 - alams * (e2 - e1 * anpsi);
        double dep1 = alams;
        double dep3 = -alams * anpsi;
        depls = 0.5 * std::fabs(dep1 - dep3);
    } else {
        s11 = s11i; s22 = s22i; s33 = s33i; s12 = s12i;
        return;
    }
    if (s1 >= ten_max) {
        s11 = ten_max; s22 = ten_max; s12 = 0.0; s33 = ten_max;
        return;
    }
    if (s2 >= ten_max && ndim == 3) {
        s2 = ten_max;
        s3 = ten_max;
    } else if (s3 >= ten_max) {
        s3 = ten_max;
    }
    double cs2, si2;
    if (psdif == 0.0) {
        cs2 = 1.0;
        si2 = 0.0;
    } else {
        cs2 = sdif / psdif;
        si2 = 2.0 * s12i / psdif;
    }
    double dc2, dss;
    if (icase == 1) {
        dc2 = (s1 - s3) * cs2; dss = s1 + s3;
        s11 = 0.5 * (dss + dc2); s22 = 0.5 * (dss - dc2); s12 = 0.5 * (s1 - s3) * si2; s33 = s2;
    } else if (icase == 2) {
        dc2 = (s2 - s3) * cs2; dss = s2 + s3;
        s11 = 0.5 * (dss + dc2); s22 = 0.5 * (dss - dc2); s12 = 0.5 * (s2 - s3) * si2; s33 = s1;
    } else {
        dc2 = (s1 - s2) * cs2; dss = s1 + s2;
        s11 = 0.5 * (dss + dc2); s22 = 0.5 * (dss - dc2); s12 = 0.5 * (s1 - s2) * si2; s33 = s3;
    }
}

// pre_plast (rh_plastic.f90:231-291)
void pre_plast(St &s, long long e, double &coh, double &phi, double &psi, double &hardn) {
    const gf_params &p = *s.p;
    double pls_curr = s.L->aps[e];
    phi = 0; coh = 0; psi = 0; hardn = 0;
    for (int k = 0; k < p.nphase; ++k) {
        double ratio = s.L->phase_ratio[o_pr(s.d, e, k)];
        if (ratio < 0.01) continue;
        double f, c, d, h;
        if (pls_curr < p.plstrain1[k]) {
            f = p.fric1[k]; c = p.cohesion1[k]; d = p.dilat1[k]; h = 0;
        } else if (pls_curr < p.plstrain2[k]) {
            double dpl = (pls_curr - p.plstrain1[k]) / (p.plstrain2[k] - p.plstrain1[k]);
            f = p.fric1[k] + (p.fric2[k] - p.fric1[k]) * dpl;
            d = p.dilat1[k] + (p.dilat2[k] - p.dilat1[k]) * dpl;
            c = p.cohesion1[k] + (p.cohesion2[k] - p.cohesion1[k]) * dpl;
            h = (p.cohesion2[k] - p.cohesion1[k]) / (p.plstrain2[k] - p.plstrain1[k]);
        } else {
            f = p.fric2[k]; c = p.cohesion2[k]; d = p.dilat2[k]; h = 0;
        }
        phi = phi + ratio / f;
        coh = coh + ratio / c;
        psi = psi + ratio * d;
        hardn = hardn + ratio * h;
    }
    phi = 1 / phi;
    coh = 1 / coh;
    if (p.itype_melting == 1) {
        double fm = (s.L->fmagma ? s.L->fmagma[e] : 0.0) + (s.L->fmagma2 ? s.L->fmagma2[e] : 0.0);
        double fma = std::min(fm, p.fmagma_max);
        phi = phi * (1 - (1 - p.weaken_ratio_plastic) * fma / p.fmagma_max);
        coh = coh * (1 - (1 - p.weaken_ratio_plastic) * fma / p.fmagma_max);
    }
}

// --------------------------------------------------------------------------
// fl_rheol (src/fl_rheol.f90:4-424)

void fl_rheol_elem(St &s, int j, int i, double dt) {
    const gf_params &p = *s.p;
    gf_layout &L = *s.L;
    long long e = s.e(j, i);
    double vx1 = s.vel(j, i, 0), vy1 = s.vel(j, i, 1);
    double vx2 = s.vel(j + 1, i, 0), vy2 = s.vel(j + 1, i, 1);
    double vx3 = s.vel(j, i + 1, 0), vy3 = s.vel(j, i + 1, 1);
    double vx4 = s.vel(j + 1, i + 1, 0), vy4 = s.vel(j + 1, i + 1, 1);
    double x1 = s.cord(j, i, 0), y1 = s.cord(j, i, 1);
    double x2 = s.cord(j + 1, i, 0), y2 = s.cord(j + 1, i, 1);
    double x3 = s.cord(j, i + 1, 0), y3 = s.cord(j, i + 1, 1);
    double x4 = s.cord(j + 1, i + 1, 0), y4 = s.cord(j + 1, i + 1, 1);
    double ar1 = s.area(e, 0), ar2 = s.area(e, 1), ar3 = s.area(e, 2), ar4 = s.area(e, 3);
    double dx[3][4], dz[3][4], sr[3][4];
    dx[0][0] = (y2 - y3) * ar1; dx[1][0] = (y3 - y1) * ar1; dx[2][0] = (y1 - y2) * ar1;
    dz[0][0] = (x3 - x2) * ar1; dz[1][0] = (x1 - x3) * ar1; dz[2][0] = (x2 - x1) * ar1;
    dx[0][1] = (y2 - y4) * ar2; dx[1][1] = (y4 - y3) * ar2; dx[2][1] = (y3 - y2) * ar2;
    dz[0][1] = (x4 - x2) * ar2; dz[1][1] = (x3 - x4) * ar2; dz[2][1] = (x2 - x3) * ar2;
    dx[0][2] = (y2 - y4) * ar3; dx[1][2] = (y4 - y1) * ar3; dx[2][2] = (y1 - y2) * ar3;
    dz[0][2] = (x4 - x2) * ar3; dz[1][2] = (x1 - x4) * ar3; dz[2][2] = (x2 - x1) * ar3;
    dx[0][3] = (y4 - y3) * ar4; dx[1][3] = (y3 - y1) * ar4; dx[2][3] = (y1 - y4) * ar4;
    dz[0][3] = (x3 - x4) * ar4; dz[1][3] = (x1 - x3) * ar4; dz[2][3] = (x4 - x1) * ar4;
    // node triplets of the triangles A,B,C,D: (1,2,3), (3,2,4), (1,2,4), (1,4,3)
    const double vxa[4][3] = {{vx1, vx2, vx3}, {vx3, vx2, vx4}, {vx1, vx2, vx4}, {vx1, vx4, vx3}};
    const double vya[4][3] = {{vy1, vy2, vy3}, {vy3, vy2, vy4}, {vy1, vy2, vy4}, {vy1, vy4, vy3}};
    for (int k = 0; k < 4; ++k) {
        sr[0][k] = vxa[k][0] * dx[0][k] + vxa[k][1] * dx[1][k] + vxa[k][2] * dx[2][k];
        sr[1][k] = vya[k][0] * dz[0][k] + vya[k][1] * dz[1][k] + vya[k][2] * dz[2][k];
        sr[2][k] = 0.5 * (vxa[k][0] * dz[0][k] + vxa[k][1] * dz[1][k] + vxa[k][2] * dz[2][k] + vya[k][0] * dx[0][k] +
                          vya[k][1] * dx[1][k] + vya[k][2] * dx[2][k]);
    }
    if (p.mix_strain == 1) {
        for (int k = 0; k < 4; k += 2) {
            double em = 0.5 * (sr[0][k] + sr[1][k] + sr[0][k + 1] + sr[1][k + 1]);
            double eda = sr[0][k] - sr[1][k];
            double edb = sr[0][k + 1] - sr[1][k + 1];
            sr[0][k] = 0.5 * (em + eda);
            sr[1][k] = 0.5 * (em - eda);
            sr[0][k + 1] = 0.5 * (em + edb);
            sr[1][k + 1] = 0.5 * (em - edb);
        }
    }
    double s11 = 0.25 * (sr[0][0] + sr[0][1] + sr[0][2] + sr[0][3]);
    double s22 = 0.25 * (sr[1][0] + sr[1][1] + sr[1][2] + sr[1][3]);
    double s12 = 0.25 * (sr[2][0] + sr[2][1] + sr[2][2] + sr[2][3]);
    double srII = 0.5 * std::sqrt((s11 - s22) * (s11 - s22) + 4.0 * s12 * s12);
    double srI = 0.5 * (s11 + s22);
    double srs2 = (s11 - srI) * (s11 - srI) + (s22 - srI) * (s22 - srI) + 2.0 * s12 * s12;
    L.se2sr[o_ek(s.d, e, 0)] = L.se2sr[o_ek(s.d, e, 0)] + s11 * dt;
    L.se2sr[o_ek(s.d, e, 1)] = L.se2sr[o_ek(s.d, e, 1)] + s22 * dt;
    L.se2sr[o_ek(s.d, e, 2)] = L.se2sr[o_ek(s.d, e, 2)] + s12 * dt;
    s11 = 0.25 * (s.st(e, 0, 0) + s.st(e, 0, 1) + s.st(e, 0, 2) + s.st(e, 0, 3));
    s22 = 0.25 * (s.st(e, 1, 0) + s.st(e, 1, 1) + s.st(e, 1, 2) + s.st(e, 1, 3));
    s12 = 0.25 * (s.st(e, 2, 0) + s.st(e, 2, 1) + s.st(e, 2, 2) + s.st(e, 2, 3));
    double stII = 0.5 * std::sqrt((s11 - s22) * (s11 - s22) + 4.0 * s12 * s12);
    if (srII != 0.0) L.sshrheat[e] = L.sshrheat[e] + stII / srII * srs2 * dt;

    int iph = L.iphase[e] - 1;
    int irh = p.irheol[iph];
    double bulkm = p.rl[iph] + 2.0 * p.rm[iph] / 3.0;
    double rmu = p.rm[iph];
    double stherm = 0.0;
    if (p.istress_therm > 0) stherm = -p.alfa[iph] * bulkm * (L.temp[o_node(s.d, j, i)] - L.temp0[o_node(s.d, j, i)]);
    double coh = 0, phi = 0, psi = 0, hardn = 0;
    if (irh == 6 || irh >= 11) pre_plast(s, e, coh, phi, psi, hardn);
    if (irh == 3 || irh >= 11) {
        if (s.c->nloop % p.ifreq_visc == 0) L.visn[e] = eff_visc(s, j, i);
    }
    double vis = L.visn[e];
    double s11s[4], s22s[4], s12s[4], s33s[4];
    for (int k = 0; k < 4; ++k) {
        s11s[k] = s.st(e, 0, k); s22s[k] = s.st(e, 1, k); s12s[k] = s.st(e, 2, k); s33s[k] = s.st(e, 3, k);
    }
    double s11p[4], s22p[4], s12p[4], s33p[4], s11v[4], s22v[4], s12v[4], s33v[4], depl[4] = {0, 0, 0, 0};
    double dike = L.dike_released ? L.dike_released[e] : 0.0;
    for (int k = 0; k < 4; ++k) {
        double de11 = sr[0][k] * dt, de22 = sr[1][k] * dt, de12 = sr[2][k] * dt, de33 = 0.0;
        double dv = L.dvol[o_ek(s.d, e, k)] - dike;
        s11p[k] = s.st(e, 0, k) + stherm;
        s22p[k] = s.st(e, 1, k) + stherm;
        s12p[k] = s.st(e, 2, k);
        s33p[k] = s.st(e, 3, k) + stherm;
        s11v[k] = s11p[k]; s22v[k] = s22p[k]; s12v[k] = s12p[k]; s33v[k] = s33p[k];
        if (irh == 1) {
            elastic(bulkm, rmu, s11p[k], s22p[k], s33p[k], s12p[k], de11, de22, de12);
            s.st(e, 0, k) = s11p[k]; s.st(e, 1, k) = s22p[k]; s.st(e, 2, k) = s12p[k]; s.st(e, 3, k) = s33p[k];
        } else if (irh == 3) {
            maxwell(bulkm, rmu, vis, s11v[k], s22v[k], s33v[k], s12v[k], de11, de22, de33, de12, dv, p.ndim, dt);
            s.st(e, 0, k) = s11v[k]; s.st(e, 1, k) = s22v[k]; s.st(e, 2, k) = s12v[k]; s.st(e, 3, k) = s33v[k];
        } else if (irh == 6) {
            plastic(bulkm, rmu, coh, phi, psi, depl[k], hardn, s11p[k], s22p[k], s33p[k], s12p[k], de11, de22, de33, de12,
                    p.ten_off, p.ndim);
            s.st(e, 0, k) = s11p[k]; s.st(e, 1, k) = s22p[k]; s.st(e, 2, k) = s12p[k]; s.st(e, 3, k) = s33p[k];
        } else if (irh >= 11) {
            plastic(bulkm, rmu, coh, phi, psi, depl[k], hardn, s11p[k], s22p[k], s33p[k], s12p[k], de11, de22, de33, de12,
                    p.ten_off, p.ndim);
            maxwell(bulkm, rmu, vis, s11v[k], s22v[k], s33v[k], s12v[k], de11, de22, de33, de12, dv, p.ndim, dt);
        }
    }
    if (irh >= 11) {
        double a = s11p[0] + s11p[1] + s11p[2] + s11p[3] - s22p[0] - s22p[1] - s22p[2] - s22p[3];
        double b = s12p[0] + s12p[1] + s12p[2] + s12p[3];
        double sII_plas = a * a + 4.0 * (b * b);
        a = s11v[0] + s11v[1] + s11v[2] + s11v[3] - s22v[0] - s22v[1] - s22v[2] - s22v[3];
        b = s12v[0] + s12v[1] + s12v[2] + s12v[3];
        double sII_visc = a * a + 4.0 * (b * b);
        if (sII_plas < sII_visc) {
            for (int k = 0; k < 4; ++k) {
                s.st(e, 0, k) = s11p[k]; s.st(e, 1, k) = s22p[k]; s.st(e, 2, k) = s12p[k]; s.st(e, 3, k) = s33p[k];
            }
        } else {
            for (int k = 0; k < 4; ++k) {
                s.st(e, 0, k) = s11v[k]; s.st(e, 1, k) = s22v[k]; s.st(e, 2, k) = s12v[k]; s.st(e, 3, k) = s33v[k];
            }
        }
    }
    if (p.mix_stress == 1) {
        for (int h = 0; h < 4; h += 2) {
            double ra = s.area(e, h), rb = s.area(e, h + 1);
            double quad_area = 1.0 / ra + 1.0 / rb;
            double s0a = 0.5 * (s.st(e, 0, h) + s.st(e, 1, h));
            double s0b = 0.5 * (s.st(e, 0, h + 1) + s.st(e, 1, h + 1));
            double s0 = (s0a / rb + s0b / ra) / quad_area;
            s.st(e, 0, h) = s.st(e, 0, h) - s0a + s0;
            s.st(e, 1, h) = s.st(e, 1, h) - s0a + s0;
            s.st(e, 0, h + 1) = s.st(e, 0, h + 1) - s0b + s0;
            s.st(e, 1, h + 1) = s.st(e, 1, h + 1) - s0b + s0;
        }
    }
    for (int k = 0; k < 4; ++k) {
        s.st(e, 0, k) = s.st(e, 0, k) - stherm;
        s.st(e, 1, k) = s.st(e, 1, k) - stherm;
        s.st(e, 3, k) = s.st(e, 3, k) - stherm;
    }
    if (irh == 6 || irh >= 11) {
        double quad_area = ar1 + ar2 + ar3 + ar4;
        L.aps[e] = L.aps[e] + (depl[0] * ar1 + depl[1] * ar2 + depl[2] * ar3 + depl[3] * ar4) / quad_area;
        if (L.aps[e] < 0.0) L.aps[e] = 0.0;
        if (p.tau_heal != 0.0) L.aps[e] = L.aps[e] / (1.0 + dt / p.tau_heal);
    }
    // the reference accumulates the element-averaged *stress* here
    // (s11/s22/s12 were reassigned at fl_rheol.f90:181-183)
    L.strain[o_ek(s.d, e, 0)] = L.strain[o_ek(s.d, e, 0)] + s11 * dt;
    L.strain[o_ek(s.d, e, 1)] = L.strain[o_ek(s.d, e, 1)] + s22 * dt;
    L.strain[o_ek(s.d, e, 2)] = L.strain[o_ek(s.d, e, 2)] + s12 * dt;
    if (p.ishearh == 1) {
        double q = 0.0;
        for (int k = 0; k < 4; ++k) {
            double f11 = s.st(e, 0, k), f22 = s.st(e, 1, k), f12 = s.st(e, 2, k), f33 = s.st(e, 3, k);
            double lambda = bulkm - 2.0 / 3.0 * rmu, mu = rmu;
            double den_el = 3.0 * lambda + 2.0 * mu;
            if (std::fabs(den_el) < 1e-30) den_el = std::copysign(1e-30, den_el);
            double tr0 = s11s[k] + s22s[k] + s33s[k];
            double e11a = (s11s[k] - (lambda / den_el) * tr0) / (2.0 * mu);
            double e22a = (s22s[k] - (lambda / den_el) * tr0) / (2.0 * mu);
            double e33a = (s33s[k] - (lambda / den_el) * tr0) / (2.0 * mu);
            double e12a = s12s[k] / (2.0 * mu);
            double tr1 = f11 + f22 + f33;
            double e11b = (f11 - (lambda / den_el) * tr1) / (2.0 * mu);
            double e22b = (f22 - (lambda / den_el) * tr1) / (2.0 * mu);
            double e33b = (f33 - (lambda / den_el) * tr1) / (2.0 * mu);
            double e12b = f12 / (2.0 * mu);
            double d11 = sr[0][k] * dt - (e11b - e11a);
            double d22 = sr[1][k] * dt - (e22b - e22a);
            double d12 = sr[2][k] * dt - (e12b - e12a);
            double d33 = 0.0 - (e33b - e33a);
            double a11 = 0.5 * (s11s[k] + f11), a22 = 0.5 * (s22s[k] + f22), a12 = 0.5 * (s12s[k] + f12),
                   a33 = 0.5 * (s33s[k] + f33);
            double qk = a11 * d11 + a22 * d22 + 2.0 * a12 * d12 + a33 * d33;
            q = q + 0.25 * qk;
        }
        L.sshrheat[e] = L.sshrheat[e] + q;
    }
}

void fl_rheol(St &s) {
    const gf_params &p = *s.p;
    gf_clock &c = *s.c;
    c.dtavg = c.dtavg + c.dt;
    int nx = p.nx, nz = p.nz;
    int err = 0;
#pragma omp parallel for schedule(guided) num_threads(g_threads) if (g_threads > 1)
    for (int i = 0; i < nx - 1; ++i)
        for (int j = 0; j < nz - 1; ++j) {
            try {
                fl_rheol_elem(s, j, i, c.dt);
            } catch (const Stop &st) {
#pragma omp critical
                if (!err) err = st.code;
            }
        }
    if (err) throw Stop{err};
    gf_layout &L = *s.L;
    if (c.nsrate == p.ifreq_avgsr || c.nsrate == -1) {
        bool reset = c.nsrate == p.ifreq_avgsr;
        for (long long e = 0; e < s.d.E; ++e) {
            double a = L.se2sr[o_ek(s.d, e, 0)], b = L.se2sr[o_ek(s.d, e, 1)], q = L.se2sr[o_ek(s.d, e, 2)];
            L.e2sr[e] = (0.5 * std::sqrt((a - b) * (a - b) + 4.0 * q * q)) / c.dtavg;
            L.shrheat[e] = L.sshrheat[e] / c.dtavg;
            if (reset) {
                L.se2sr[o_ek(s.d, e, 0)] = 0.0;
                L.se2sr[o_ek(s.d, e, 1)] = 0.0;
                L.se2sr[o_ek(s.d, e, 2)] = 0.0;
                L.sshrheat[e] = 0.0;
            }
        }
        if (reset) {
            c.dtavg = 0.0;
            c.nsrate = 0;
        }
    }
    c.nsrate = c.nsrate + 1;
}

// --------------------------------------------------------------------------
// fl_node (src/fl_node.f90:3-393)

void fl_node(St &s) {
    const gf_params &p = *s.p;
    gf_layout &L = *s.L;
    const gf_clock &c = *s.c;
    int nx = p.nx, nz = p.nz;
    if (p.nystressbc != 0) throw Stop{GF_ERR_UNSUPPORTED};
    static const int kk[4][3] = {{2, 3, 4}, {1, 2, 3}, {1, 2, 4}, {1, 3, 4}};
    static const int mm[4][3] = {{3, 3, 2}, {2, 2, 2}, {3, 1, 3}, {1, 1, 1}};
    double drat = c.dt / c.dt_elastic;
    if (drat < 1.0) drat = 1.0;
    std::vector<double> force(2 * (size_t)s.d.N, 0.0);
#pragma omp parallel for num_threads(g_threads) if (g_threads > 1)
    for (int i = 0; i < nx; ++i)
        for (int j = 0; j < nz; ++j) {
            double fx0 = 0.0, fy0 = 0.0;
            // elements (j-1,i-1), (j-1,i), (j,i-1), (j,i) in that order
            const int dj[4] = {-1, -1, 0, 0}, di[4] = {-1, 0, -1, 0};
            for (int q = 0; q < 4; ++q) {
                int je = j + dj[q], ie = i + di[q];
                if (je < 0 || ie < 0 || je > nz - 2 || ie > nx - 2) continue;
                long long e = s.e(je, ie);
                double x1 = s.cord(je, ie, 0), y1 = s.cord(je, ie, 1);
                double x2 = s.cord(je + 1, ie, 0), y2 = s.cord(je + 1, ie, 1);
                double x3 = s.cord(je, ie + 1, 0), y3 = s.cord(je, ie + 1, 1);
                double x4 = s.cord(je + 1, ie + 1, 0), y4 = s.cord(je + 1, ie + 1, 1);
                double ar[4] = {s.area(e, 0), s.area(e, 1), s.area(e, 2), s.area(e, 3)};
                double dx[3][4], dz[3][4];
                dx[0][0] = (y2 - y3) * ar[0]; dx[1][0] = (y3 - y1) * ar[0]; dx[2][0] = (y1 - y2) * ar[0];
                dz[0][0] = (x3 - x2) * ar[0]; dz[1][0] = (x1 - x3) * ar[0]; dz[2][0] = (x2 - x1) * ar[0];
                dx[0][1] = (y2 - y4) * ar[1]; dx[1][1] = (y4 - y3) * ar[1]; dx[2][1] = (y3 - y2) * ar[1];
                dz[0][1] = (x4 - x2) * ar[1]; dz[1][1] = (x3 - x4) * ar[1]; dz[2][1] = (x2 - x3) * ar[1];
                dx[0][2] = (y2 - y4) * ar[2]; dx[1][2] = (y4 - y1) * ar[2]; dx[2][2] = (y1 - y2) * ar[2];
                dz[0][2] = (x4 - x2) * ar[2]; dz[1][2] = (x1 - x4) * ar[2]; dz[2][2] = (x2 - x1) * ar[2];
                dx[0][3] = (y4 - y3) * ar[3]; dx[1][3] = (y3 - y1) * ar[3]; dx[2][3] = (y1 - y4) * ar[3];
                dz[0][3] = (x3 - x4) * ar[3]; dz[1][3] = (x1 - x3) * ar[3]; dz[2][3] = (x4 - x1) * ar[3];
                for (int k = 0; k < 3; ++k) {
                    int t = kk[q][k] - 1, m = mm[q][k] - 1;
                    double factor = 0.25 / ar[t];
                    double fx = factor * (L.stress0[o_s(s.d, e, 0, t)] * dx[m][t] + L.stress0[o_s(s.d, e, 2, t)] * dz[m][t]);
                    double fy = factor * (L.stress0[o_s(s.d, e, 2, t)] * dx[m][t] + L.stress0[o_s(s.d, e, 1, t)] * dz[m][t]);
                    fx0 = fx0 - fx;
                    fy0 = fy0 - fy;
                }
            }
            fy0 = fy0 - L.rmass[o_node(s.d, j, i)] * p.g;
            force[o_n2(s.d, j, i, 0)] = fx0;
            force[o_n2(s.d, j, i, 1)] = fy0;
        }
    if (p.nyhydro > 0) {
        for (int i = 0; i < nx; ++i) {
            double rho_water_g = 1030.0 * p.g;
            double water_depth = (i < nx - 1) ? 0.5 * (s.cord(0, i + 1, 1) + s.cord(0, i, 1))
                                              : 0.5 * (s.cord(0, i - 1, 1) + s.cord(0, i, 1));
            if (water_depth < 0.0) {
                double pl = 0, dlxl = 0, dlyl = 0, pr = 0, dlxr = 0, dlyr = 0;
                if (i > 0) {
                    pl = rho_water_g * ((s.cord(0, i - 1, 1) + s.cord(0, i, 1)) / 2.0);
                    dlxl = s.cord(0, i, 0) - s.cord(0, i - 1, 0);
                    dlyl = s.cord(0, i, 1) - s.cord(0, i - 1, 1);
                }
                if (i < nx - 1) {
                    pr = rho_water_g * ((s.cord(0, i + 1, 1) + s.cord(0, i, 1)) / 2.0);
                    dlxr = s.cord(0, i + 1, 0) - s.cord(0, i, 0);
                    dlyr = s.cord(0, i + 1, 1) - s.cord(0, i, 1);
                }
                double &f0 = force[o_n2(s.d, 0, i, 0)];
                double &f1 = force[o_n2(s.d, 0, i, 1)];
                f0 = f0 - 0.5 * pl * dlyl - 0.5 * pr * dlyr;
                f1 = f1 + 0.5 * pl * dlxl + 0.5 * pr * dlxr;
            }
        }
        int ips = p.iphsub - 1;
        for (int i = 0; i < nx; ++i) {
            double p_est = p.pisos + 0.5 * (p.den[ips] + p.drosub) * p.g * (s.cord(nz - 1, i, 1) - p.rzbo);
            double rosubg = p.g * (p.den[ips] + p.drosub) *
                            (1 - p.alfa[ips] * L.temp[o_node(s.d, nz - 1, i)] + p.beta[ips] * p_est);
            double pl = 0, dlxl = 0, dlyl = 0, pr = 0, dlxr = 0, dlyr = 0;
            if (i > 0) {
                pl = p.pisos - rosubg * ((s.cord(nz - 1, i - 1, 1) + s.cord(nz - 1, i, 1)) / 2.0 - p.rzbo);
                dlxl = s.cord(nz - 1, i, 0) - s.cord(nz - 1, i - 1, 0);
                dlyl = s.cord(nz - 1, i, 1) - s.cord(nz - 1, i - 1, 1);
            }
            if (i < nx - 1) {
                pr = p.pisos - rosubg * ((s.cord(nz - 1, i + 1, 1) + s.cord(nz - 1, i, 1)) / 2.0 - p.rzbo);
                dlxr = s.cord(nz - 1, i + 1, 0) - s.cord(nz - 1, i, 0);
                dlyr = s.cord(nz - 1, i + 1, 1) - s.cord(nz - 1, i, 1);
            }
            double &f0 = force[o_n2(s.d, nz - 1, i, 0)];
            double &f1 = force[o_n2(s.d, nz - 1, i, 1)];
            f0 = f0 - 0.5 * pl * dlyl - 0.5 * pr * dlyr;
            f1 = f1 + 0.5 * pl * dlxl + 0.5 * pr * dlxr;
        }
    }
#pragma omp parallel for num_threads(g_threads) if (g_threads > 1)
    for (int i = 0; i < nx; ++i)
        for (int j = 0; j < nz; ++j) {
            long long n0 = o_n2(s.d, j, i, 0), n1 = o_n2(s.d, j, i, 1);
            double f0 = force[n0], f1 = force[n1];
            int c0 = L.ncod[n0], c1 = L.ncod[n1];
            if ((c0 & 1) != 1 && std::fabs(L.vel[n0]) > 1.0e-13) f0 = f0 - p.demf * std::copysign(std::fabs(f0), L.vel[n0]);
            if ((c1 & 2) != 2 && std::fabs(L.vel[n1]) > 1.0e-13) f1 = f1 - p.demf * std::copysign(std::fabs(f1), L.vel[n1]);
            double am = L.amass[o_node(s.d, j, i)];
            if (c0 == 1)
                L.vel[n0] = L.bc[n0];
            else
                L.vel[n0] = L.vel[n0] + c.dt * f0 / (am * drat * drat);
            if (c1 == 1)
                L.vel[n1] = L.bc[n1];
            else
                L.vel[n1] = L.vel[n1] + c.dt * f1 / (am * drat * drat);
        }
    if (p.i_prestress == 1 && c.time < 600e3 * GF_SEC_YEAR) {
        for (int k = 0; k < 2; ++k)
            for (int i = 0; i < nx; ++i) L.vel[o_n2(s.d, nz - 1, i, k)] = 0.0;
        for (int k = 0; k < 2; ++k)
            for (int j = 0; j < nz; ++j) {
                L.vel[o_n2(s.d, j, 0, k)] = 0.0;
                L.vel[o_n2(s.d, j, nx - 1, k)] = 0.0;
            }
    }
}

// --------------------------------------------------------------------------
// fl_move (src/fl_move.f90:3-132)

void count_phase_ratio(St &s, int j, int i);
int add_marker(St &s, double x, double y, int iph, double age, int j, int i);
void newphase2marker(St &s, int j1, int j2, int i1, int i2, int iph);

// phase ids with special rules (phases.f90)
constexpr int K_SED1 = 1, K_OCEAN1 = 3, K_MANT1 = 4, K_SCHIST = 5, K_OCEAN2 = 7, K_MANT2 = 8, K_SERP = 9,
              K_OCEANDRY = 10, K_SED2 = 11, K_ECLG = 13, K_ARC1 = 14, K_HYDMANT = 16, K_METASED = 17;

// Fortran MIN / MAX of two reals as gfortran evaluates them for ordered values
inline double fmin2(double a, double b) { return b < a ? b : a; }
inline double fmax2(double a, double b) { return b > a ? b : a; }
// ceiling() of a ratio that may be huge, held to +-2^29 (beyond every loop
// bound it feeds)
inline int ceil_int(double x) {
    double c = std::ceil(x);
    if (!(c < 536870912.0)) return 536870912;
    if (c < -536870912.0) return -536870912;
    return (int)c;
}

// add_marker_at_top (fl_move.f90:429-472): a marker of phase kph at a
// random point of the top element of column i, in the upper dz_ratio of it;
// stop 134 after 100 misses
void add_marker_at_top(St &s, int i, double dz_ratio, double time, int loop, int kph) {
    int iseed = loop + (i + 1);
    int icount = 0;
    while (true) {
        double r1 = o_myrandom(iseed);
        double r2 = o_myrandom(iseed);
        double x1 = s.cord(0, i, 0) * (1 - r1) + s.cord(0, i + 1, 0) * r1;
        double y1 = s.cord(0, i, 1) * (1 - r1) + s.cord(0, i + 1, 1) * r1;
        double x2 = s.cord(1, i, 0) * (1 - r1) + s.cord(1, i + 1, 0) * r1;
        double y2 = s.cord(1, i, 1) * (1 - r1) + s.cord(1, i + 1, 1) * r1;
        r2 = r2 * dz_ratio;
        double xx = x1 * (1 - r2) + x2 * r2;
        double yy = y1 * (1 - r2) + y2 * r2;
        int inc = add_marker(s, xx, yy, kph, time, 0, i);
        if (inc == 1 || inc == -1) break;
        icount = icount + 1;
        if (icount > 100) throw Stop{134};
    }
}

// resurface (fl_move.f90:320-426), serial over the surface elements: an
// element whose accumulated erosion exceeds its thickness / markers loses its
// topmost marker, one whose deposition does gains a sediment marker (phase
// ksed1 = 1), one whose accumulated extrusion does gains arc markers
// (phase kocean1)
void resurface(St &s) {
    const gf_params &p = *s.p;
    gf_layout &L = *s.L;
    const int nx = p.nx, M = GF_MAX_MARKERS_PER_ELEM;
    for (int i = 0; i < nx - 1; ++i) {
        double elz = 0.5 * (s.cord(0, i, 1) - s.cord(1, i, 1) + s.cord(0, i + 1, 1) - s.cord(1, i + 1, 1));
        double chgtopo = L.dhacc[i];
        long long e = s.e(0, i);
        int kinc = L.nmark_elem[e];
        int ichanged = 0;
        if (-chgtopo * kinc >= elz && kinc > 1) {
            double ymax = -1e30;
            int kmax = 0;
            for (int k = 1; k <= kinc; ++k) {
                int n = L.mark_id_elem[e * M + k - 1];
                int m = L.mark_ntriag[n - 1];
                int kk = (m - 1) % 2 + 1;
                int jj = ((m - kk) / 2) % (p.nz - 1);
                int ii = (m - kk) / 2 / (p.nz - 1);
                double ba1 = L.mark_a1[n - 1], ba2 = L.mark_a2[n - 1];
                double ba3 = 1.0 - ba1 - ba2;
                int i1, i2, i3, j1, j2, j3;
                if (kk == 1) {
                    i1 = ii; i2 = ii; i3 = ii + 1; j1 = jj; j2 = jj + 1; j3 = jj;
                } else {
                    i1 = ii + 1; i2 = ii; i3 = ii + 1; j1 = jj; j2 = jj + 1; j3 = jj + 1;
                }
                double y = s.cord(j1, i1, 1) * ba1 + s.cord(j2, i2, 1) * ba2 + s.cord(j3, i3, 1) * ba3;
                if (ymax < y) {
                    ymax = y;
                    kmax = k;
                }
            }
            if (kmax != 0) {
                int nmax = L.mark_id_elem[e * M + kmax - 1];
                L.mark_id_elem[e * M + kmax - 1] = L.mark_id_elem[e * M + kinc - 1];
                L.mark_id_elem[e * M + kinc - 1] = 0;
                L.mark_dead[nmax - 1] = 0;
                L.nmark_elem[e] = L.nmark_elem[e] - 1;
            }
            L.dhacc[i] = 0.0;
            ichanged = 1;
        }
        if (chgtopo * kinc >= elz && kinc != M) {
            add_marker_at_top(s, i, 0.1, s.c->time, s.c->nloop, 1);
            L.dhacc[i] = 0.0;
            ichanged = 1;
        }
        // volcanic extrusion: arc markers (phase kocean1) in the upper
        // part of the element (fl_move.f90:403-416)
        double chgtopo2 = L.extr_acc ? L.extr_acc[i] : 0.0;
        if (chgtopo2 * kinc >= elz && kinc != M) {
            int n_to_add = std::min(ceil_int(chgtopo2 / elz * kinc), M - kinc);
            double dz_ratio = fmin2(chgtopo2 / elz, 1.0);
            for (int ii = 1; ii <= n_to_add; ++ii)
                add_marker_at_top(s, i, dz_ratio, s.c->time, s.c->nloop + (i + 1) + ii, K_OCEAN1);
            L.extr_acc[i] = 0;
            ichanged = 1;
        }
        if (ichanged == 1) count_phase_ratio(s, 0, i);
    }
}

// diff_topo (fl_move.f90:138-315): diffusion of the surface with topo_kappa
// and the erodibility of the surface phase where it erodes, limited to half
// the top element's thickness; accumulates dhacc_correction and dhacc;
// then arc extrusion and MOR crust from the magma pools (zero without melt);
// resurface every ifreq_avgsr steps.
void diff_topo(St &s) {
    const gf_params &p = *s.p;
    gf_layout &L = *s.L;
    const int nx = p.nx;
    const double dt = s.c->dt;
    std::vector<double> dtopo(nx, 0.0);
    for (int i = 1; i < nx - 1; ++i) {
        double snder = (p.topo_kappa * (s.cord(0, i + 1, 1) - s.cord(0, i, 1)) / (s.cord(0, i + 1, 0) - s.cord(0, i, 0)) -
                        p.topo_kappa * (s.cord(0, i, 1) - s.cord(0, i - 1, 1)) / (s.cord(0, i, 0) - s.cord(0, i - 1, 0))) /
                       (s.cord(0, i + 1, 0) - s.cord(0, i - 1, 0));
        if (snder < 0) {
            int iph = L.iphase[s.e(0, i)];
            snder = snder * p.erodibility[iph - 1];
        }
        dtopo[i] = dt * snder;
    }
    dtopo[0] = dtopo[1];
    dtopo[nx - 1] = dtopo[nx - 2];
    for (int i = 0; i < nx; ++i) dtopo[i] = std::min(dtopo[i], 0.5 * (s.cord(0, i, 1) - s.cord(1, i, 1)));
    for (int i = 0; i < nx; ++i) L.dhacc_correction[i] = L.dhacc_correction[i] + dtopo[i];
    for (int i = 0; i < nx - 1; ++i) L.dhacc[i] = L.dhacc[i] + 0.5 * (dtopo[i] + dtopo[i + 1]);
    for (int i = 0; i < nx; ++i) s.cordr(0, i, 1) = s.cord(0, i, 1) + dtopo[i];
    const int nz = p.nz;
    // arc extrusion (fl_move.f90:213-237): the melt of each inner column
    // erupts as a layer over the column and half its neighbours
    const double arc_extrusion_rate = 1.0 - p.ratio_mantle_mzone - p.ratio_crust_mzone;
    if (arc_extrusion_rate > 0 && L.fmelt && L.extrusion) {
        for (int i = 1; i < nx - 2; ++i) {
            double totalmelt = 0;
            for (int j = 0; j < nz - 1; ++j) {
                long long e = s.e(j, i);
                double quad_area = 0.5 / s.area(e, 0) + 0.5 / s.area(e, 1);
                totalmelt = totalmelt + quad_area * L.fmelt[e];
            }
            double ext = arc_extrusion_rate * dt * totalmelt * p.prod_magma /
                         (s.cord(0, i + 1, 0) - s.cord(0, i, 0) +
                          0.5 * (s.cord(0, i, 0) - s.cord(0, i - 1, 0) + s.cord(0, i + 2, 0) - s.cord(0, i + 1, 0)));
            L.extrusion[i] = ext;
            L.extr_acc[i] = L.extr_acc[i] + ext;
            L.dhacc_correction[i] = L.dhacc_correction[i] + ext;
            L.dhacc_correction[i + 1] = L.dhacc_correction[i + 1] + ext;
            L.dhacc[i] = L.dhacc[i] + ext;
            s.cordr(0, i, 1) = s.cord(0, i, 1) + ext;
            s.cordr(0, i + 1, 1) = s.cord(0, i + 1, 1) + ext;
        }
    }
    // new oceanic crust from the MOR magma pool fmagma2 (fl_move.f90:243-302)
    for (int i = 1; i < nx - 2 && L.fmagma2; ++i) {
        double total_melt = 0;
        for (int j = 0; j < nz - 1; ++j) {
            long long e = s.e(j, i);
            double quad_area = 0.5 / s.area(e, 0) + 0.5 / s.area(e, 1);
            total_melt = total_melt + quad_area * L.fmagma2[e];
            double delta = fmin2(L.fmagma2[e], L.fmagma2[e] * p.prod_magma2 * dt);
            L.fmagma2[e] = L.fmagma2[e] - delta;
        }
        double extrusion_height = dt * total_melt * p.prod_magma2 / (s.cord(0, i + 1, 0) - s.cord(0, i, 0));
        double ele_height = 0, quotient = 0, remainder = 0;
        int j_oc = 1;
        for (int j = 0; j < nz - 1; ++j) {
            ele_height = ele_height + std::fabs(0.5 * (s.cord(j + 1, i + 1, 1) + s.cord(j + 1, i, 1)) -
                                                0.5 * (s.cord(j, i + 1, 1) + s.cord(j, i, 1)));
            quotient = extrusion_height / ele_height;
            remainder = std::fmod(extrusion_height, ele_height);
            if (quotient >= 0.0 && quotient < 2.0) {
                j_oc = j + 1;
                break;
            }
        }
        for (int j = 1; j <= nz - 1; ++j) {
            int iph = L.iphase[s.e(j - 1, i)];
            if (iph != K_OCEAN1 && quotient >= 1) {
                newphase2marker(s, j, std::min(nz - 1, j + j_oc - 1), i + 1, i + 1, K_OCEAN1);
                break;
            }
        }
        L.extr_acc[i] = L.extr_acc[i] + remainder / 2;
        s.cordr(0, i, 1) = s.cord(0, i, 1) + remainder / 2;
        s.cordr(0, i + 1, 1) = s.cord(0, i + 1, 1) + remainder / 2;
    }
    for (int i = 0; i < nx; ++i) L.dtopo[i] = dtopo[i];
    if (s.c->nloop % p.ifreq_avgsr == 0) resurface(s);
}

// fl_flexure (fl_flexure.f90:1-189) with get_column_weights (:192-231) and
// solve_block_tridiagonal (:234-294): the bottom of a model with the
// flexural boundary condition (nbc 200 on side 2) follows an elastic plate of
// thickness bca on a fluid of density bcb, loaded by the change of the
// columns' weight; the plate's deflection rate is added to the columns'
// vertical velocities
void fl_flexure(St &s) {
    const gf_params &p = *s.p;
    gf_layout &L = *s.L;
    int bc_idx = -1;
    for (int b = 0; b < p.nofbc; ++b)
        if (p.nbc[b] == 200 && p.nofside[b] == 2) {
            bc_idx = b;
            break;
        }
    if (bc_idx < 0) return;
    const int nx = p.nx, nz = p.nz;
    const double Te = p.bca[bc_idx], rho_m = p.bcb[bc_idx], g = p.g;
    const long long N = s.d.N;
    auto ED = [&](int j, int i) { return eff_dens(s, j, i, &s.c->frac); };
    std::vector<double> q(nx), Load(nx), x(nx), dx(nx), D(nx);
    for (int i = 0; i < nx; ++i) { // get_column_weights
        q[i] = 0.0;
        for (int j = 0; j < nz - 1; ++j) {
            double rho;
            if (i == 0)
                rho = ED(j, 0);
            else if (i == nx - 1)
                rho = ED(j, nx - 2);
            else {
                double r1 = ED(j, i - 1), r2 = ED(j, i); // left operand first
                rho = 0.5 * (r1 + r2);
            }
            double dz = s.cord(j, i, 1) - s.cord(j + 1, i, 1);
            q[i] = q[i] + rho * g * dz;
        }
        double rho_b;
        if (i == 0)
            rho_b = ED(nz - 2, 0);
        else if (i == nx - 1)
            rho_b = ED(nz - 2, nx - 2);
        else {
            double r1 = ED(nz - 2, i - 1), r2 = ED(nz - 2, i);
            rho_b = 0.5 * (r1 + r2);
        }
        q[i] = q[i] - rho_b * g * (L.zoriginal[o_node(s.d, nz - 1, i)] - s.cord(nz - 1, i, 1));
    }
    bool all_zero = true;
    for (int i = 0; i < nx; ++i) all_zero = all_zero && L.q_init[i] == 0.0;
    if (all_zero)
        for (int i = 0; i < nx; ++i) L.q_init[i] = q[i];
    for (int i = 0; i < nx; ++i) Load[i] = q[i] - L.q_init[i];
    for (int i = 0; i < nx; ++i) x[i] = s.cord(nz - 1, i, 0);
    for (int i = 0; i < nx - 1; ++i) {
        dx[i] = x[i + 1] - x[i];
        if (dx[i] <= 0.0) dx[i] = 1.0;
    }
    for (int i = 0; i < nx; ++i) {
        int iph = i < nx - 1 ? L.iphase[s.e(nz - 2, i)] : L.iphase[s.e(nz - 2, nx - 2)];
        if (iph < 1 || iph > p.nphase) iph = 1;
        double lambda = p.rl[iph - 1], mu = p.rm[iph - 1], E, nu;
        if (lambda + mu > 0.0) {
            E = mu * (3.0 * lambda + 2.0 * mu) / (lambda + mu);
            nu = lambda / (2.0 * (lambda + mu));
        } else {
            E = 1.0e11;
            nu = 0.25;
        }
        if (nu >= 1.0 || nu <= -1.0) nu = 0.25;
        D[i] = (E * (Te * Te * Te)) / (12.0 * (1.0 - (nu * nu)));
        if (D[i] <= 0.0) D[i] = 1.0e15;
    }
    // block tridiagonal system (2x2 blocks; the a and c blocks are diagonal)
    // solved by the forward sweep and back substitution of the reference
    std::vector<double> cp(4 * nx), rp(2 * nx), u(2 * nx);
    auto W = [&](double load) { return rho_m * g > 0.0 ? load / (rho_m * g) : 0.0; };
    // i = 0: B = I, C = 0, r = (0, w_winkler_1)
    cp[0] = cp[1] = cp[2] = cp[3] = 0.0;
    rp[0] = 0.0;
    rp[1] = W(Load[0]);
    for (int i = 1; i < nx - 1; ++i) {
        double a_i = 2.0 / (dx[i - 1] * (dx[i] + dx[i - 1]));
        double c_i = 2.0 / (dx[i] * (dx[i] + dx[i - 1]));
        double b_i = -(a_i + c_i);
        double b11 = b_i, b12 = -rho_m * g, b21 = 1.0 / D[i], b22 = b_i;
        double r1 = -Load[i], r2 = 0.0;
        double d11 = b11 - a_i * cp[4 * (i - 1) + 0];
        double d12 = b12 - a_i * cp[4 * (i - 1) + 1];
        double d21 = b21 - a_i * cp[4 * (i - 1) + 2];
        double d22 = b22 - a_i * cp[4 * (i - 1) + 3];
        double det = d11 * d22 - d12 * d21;
        if (std::fabs(det) < 1e-30) det = std::copysign(1e-30, det);
        double i11 = d22 / det, i12 = -d12 / det, i21 = -d21 / det, i22 = d11 / det;
        cp[4 * i + 0] = i11 * c_i;
        cp[4 * i + 1] = i12 * c_i;
        cp[4 * i + 2] = i21 * c_i;
        cp[4 * i + 3] = i22 * c_i;
        double t1 = r1 - a_i * rp[2 * (i - 1)], t2 = r2 - a_i * rp[2 * (i - 1) + 1];
        rp[2 * i] = i11 * t1 + i12 * t2;
        rp[2 * i + 1] = i21 * t1 + i22 * t2;
    }
    u[2 * (nx - 1)] = 0.0;
    u[2 * (nx - 1) + 1] = W(Load[nx - 1]);
    for (int i = nx - 2; i >= 0; --i) {
        u[2 * i] = rp[2 * i] - (cp[4 * i + 0] * u[2 * (i + 1)] + cp[4 * i + 1] * u[2 * (i + 1) + 1]);
        u[2 * i + 1] = rp[2 * i + 1] - (cp[4 * i + 2] * u[2 * (i + 1)] + cp[4 * i + 3] * u[2 * (i + 1) + 1]);
    }
    const double dt = s.c->dt;
    for (int i = 0; i < nx; ++i) {
        for (int j = 0; j < nz - 1; ++j) L.vel[N + o_node(s.d, j, i)] = L.vel[N + o_node(s.d, j, i)] - L.vel_flex_old[i];
        double cord_old_z = s.cord(nz - 1, i, 1);
        s.cordr(nz - 1, i, 1) = L.zoriginal[o_node(s.d, nz - 1, i)] - u[2 * i + 1];
        double vel_flex = 0.0;
        if (dt > 0.0) vel_flex = (s.cord(nz - 1, i, 1) - cord_old_z) / dt;
        for (int j = 0; j < nz - 1; ++j) L.vel[N + o_node(s.d, j, i)] = L.vel[N + o_node(s.d, j, i)] + vel_flex;
        L.vel[N + o_node(s.d, nz - 1, i)] = vel_flex;
        L.vel_flex_old[i] = vel_flex;
    }
}

void fl_move(St &s) {
    const gf_params &p = *s.p;
    gf_layout &L = *s.L;
    double dt = s.c->dt;
    if (p.movegrid == 0) return;
    int nx = p.nx, nz = p.nz;
    for (long long n = 0; n < s.d.N; ++n) {
        L.cord[n] = L.cord[n] + L.vel[n] * dt;
        L.cord[s.d.N + n] = L.cord[s.d.N + n] + L.vel[s.d.N + n] * dt;
    }
    fl_flexure(s);
    if (p.topo_kappa > 0.0) diff_topo(s);
    static const int nd1[4] = {1, 3, 1, 1}, nd2[4] = {2, 2, 2, 4}, nd3[4] = {3, 4, 4, 3};
    int err = 0;
#pragma omp parallel for num_threads(g_threads) if (g_threads > 1)
    for (int i = 0; i < nx - 1; ++i)
        for (int j = 0; j < nz - 1; ++j) {
            long long e = s.e(j, i);
            double xc[4] = {s.cord(j, i, 0), s.cord(j + 1, i, 0), s.cord(j, i + 1, 0), s.cord(j + 1, i + 1, 0)};
            double yc[4] = {s.cord(j, i, 1), s.cord(j + 1, i, 1), s.cord(j, i + 1, 1), s.cord(j + 1, i + 1, 1)};
            double xv[4] = {s.vel(j, i, 0), s.vel(j + 1, i, 0), s.vel(j, i + 1, 0), s.vel(j + 1, i + 1, 0)};
            double yv[4] = {s.vel(j, i, 1), s.vel(j + 1, i, 1), s.vel(j, i + 1, 1), s.vel(j + 1, i + 1, 1)};
            bool neg = false;
            for (int k = 0; k < 4; ++k) {
                int a = nd1[k] - 1, b = nd2[k] - 1, cc = nd3[k] - 1;
                double det = ((xc[b] * yc[cc] - yc[b] * xc[cc]) - (xc[a] * yc[cc] - yc[a] * xc[cc])) + (xc[a] * yc[b] - yc[a] * xc[b]);
                L.dvol[o_ek(s.d, e, k)] = det * L.area[o_ek(s.d, e, k)] - 1.0;
                L.area[o_ek(s.d, e, k)] = 1.0 / det;
                double dw12 = 0.5 * (xv[a] * (xc[cc] - xc[b]) + xv[b] * (xc[a] - xc[cc]) + xv[cc] * (xc[b] - xc[a]) +
                                     yv[a] * (yc[cc] - yc[b]) + yv[b] * (yc[a] - yc[cc]) + yv[cc] * (yc[b] - yc[a])) /
                              det * dt;
                double s11 = s.st(e, 0, k), s22 = s.st(e, 1, k), s12 = s.st(e, 2, k);
                s.st(e, 0, k) = s11 + s12 * 2 * dw12;
                s.st(e, 1, k) = s22 - s12 * 2 * dw12;
                s.st(e, 2, k) = s12 + dw12 * (s22 - s11);
                if (k == 0) {
                    double e11 = L.strain[o_ek(s.d, e, 0)], e22 = L.strain[o_ek(s.d, e, 1)], e12 = L.strain[o_ek(s.d, e, 2)];
                    L.strain[o_ek(s.d, e, 0)] = e11 + e12 * 2 * dw12;
                    L.strain[o_ek(s.d, e, 1)] = e22 - e12 * 2 * dw12;
                    L.strain[o_ek(s.d, e, 2)] = e12 + dw12 * (e22 - e11);
                }
            }
            for (int k = 0; k < 4; ++k)
                if (L.area[o_ek(s.d, e, k)] <= 0) neg = true;
            if (neg) {
#pragma omp critical
                err = 40;
            }
        }
    if (err) throw Stop{40};
}

// --------------------------------------------------------------------------
// rmasses (src/rmasses.f90:4-63) and dt_mass (src/dt_mass.f90:16-232)

void rmasses(St &s) {
    const gf_params &p = *s.p;
    gf_layout &L = *s.L;
    const double c1d12 = 1.0 / 12.0;
    int nx = p.nx, nz = p.nz;
    for (long long n = 0; n < s.d.N; ++n) L.rmass[n] = 0;
    // serial order of frac writes: colour by colour, i then j
    for (int ib = 0; ib < 2; ++ib)
        for (int jb = 0; jb < 2; ++jb) {
#pragma omp parallel for num_threads(g_threads) if (g_threads > 1)
            for (int i = ib; i < nx - 1; i += 2)
                for (int j = jb; j < nz - 1; j += 2) {
                    double dens = eff_dens(s, j, i, &s.c->frac);
                    long long e = s.e(j, i);
                    double a0 = s.area(e, 0), a1 = s.area(e, 1), a2 = s.area(e, 2), a3 = s.area(e, 3);
                    double *rm = L.rmass;
                    long long n11 = o_node(s.d, j, i), n21 = o_node(s.d, j + 1, i), n12 = o_node(s.d, j, i + 1),
                              n22 = o_node(s.d, j + 1, i + 1);
                    rm[n11] = rm[n11] + c1d12 / a0 * dens;
                    rm[n21] = rm[n21] + c1d12 / a0 * dens;
                    rm[n12] = rm[n12] + c1d12 / a0 * dens;
                    rm[n22] = rm[n22] + c1d12 / a1 * dens;
                    rm[n21] = rm[n21] + c1d12 / a1 * dens;
                    rm[n12] = rm[n12] + c1d12 / a1 * dens;
                    rm[n11] = rm[n11] + c1d12 / a2 * dens;
                    rm[n21] = rm[n21] + c1d12 / a2 * dens;
                    rm[n22] = rm[n22] + c1d12 / a2 * dens;
                    rm[n11] = rm[n11] + c1d12 / a3 * dens;
                    rm[n22] = rm[n22] + c1d12 / a3 * dens;
                    rm[n12] = rm[n12] + c1d12 / a3 * dens;
                }
        }
}

double dlmin_prop(St &s) {
    int nx = s.p->nx, nz = s.p->nz;
    double dlmin = 1e28;
#pragma omp parallel for reduction(min : dlmin) num_threads(g_threads) if (g_threads > 1)
    for (int i = 0; i < nx - 1; ++i)
        for (int j = 0; j < nz - 1; ++j) {
            long long e = s.e(j, i);
            auto len = [&](int ja, int ia, int jb, int ib) {
                double ddx = s.cord(ja, ia, 0) - s.cord(jb, ib, 0), ddy = s.cord(ja, ia, 1) - s.cord(jb, ib, 1);
                return std::sqrt(ddx * ddx + ddy * ddy);
            };
            double dl;
            dl = len(j + 1, i, j, i);
            dlmin = std::min(dlmin, 1.0 / (s.area(e, 0) * dl));
            dlmin = std::min(dlmin, 1.0 / (s.area(e, 2) * dl));
            dl = len(j + 1, i + 1, j + 1, i);
            dlmin = std::min(dlmin, 1.0 / (s.area(e, 1) * dl));
            dlmin = std::min(dlmin, 1.0 / (s.area(e, 2) * dl));
            dl = len(j + 1, i + 1, j, i + 1);
            dlmin = std::min(dlmin, 1.0 / (s.area(e, 1) * dl));
            dlmin = std::min(dlmin, 1.0 / (s.area(e, 3) * dl));
            dl = len(j, i + 1, j, i);
            dlmin = std::min(dlmin, 1.0 / (s.area(e, 0) * dl));
            dlmin = std::min(dlmin, 1.0 / (s.area(e, 3) * dl));
            dl = len(j + 1, i + 1, j, i);
            dlmin = std::min(dlmin, 1.0 / (s.area(e, 2) * dl));
            dlmin = std::min(dlmin, 1.0 / (s.area(e, 3) * dl));
            dl = len(j + 1, i, j, i + 1);
            dlmin = std::min(dlmin, 1.0 / (s.area(e, 0) * dl));
            dlmin = std::min(dlmin, 1.0 / (s.area(e, 1) * dl));
        }
    return dlmin;
}

void dt_mass(St &s) {
    const gf_params &p = *s.p;
    gf_layout &L = *s.L;
    gf_clock &c = *s.c;
    const double c1d12 = 1.0 / 12.0;
    int nx = p.nx, nz = p.nz;
    double dlmin = dlmin_prop(s);
    c.dlmin = dlmin;
    if (p.idt_scale == 1)
        c.dt_elastic = p.dt_scale;
    else if (p.idt_scale == 2) {
        if (p.vbc == 0)
            c.dt_elastic = dlmin * c.frac * p.strain_inert / (1.0 / GF_SEC_YEAR / 100);
        else
            c.dt_elastic = dlmin * c.frac * p.strain_inert / p.vbc;
    }
    double dtmax_therm = 1e28, dt_maxwell = 1e28, dt_elastic = c.dt_elastic;
    double vel_max = 0.0;
    for (long long n = 0; n < 2 * s.d.N; ++n) vel_max = std::max(vel_max, std::fabs(L.vel[n]));
    c.vel_max = vel_max;
    for (long long n = 0; n < s.d.N; ++n) L.amass[n] = (p.idt_scale == 0) ? L.rmass[n] : 0.0;
    for (int ib = 0; ib < 2; ++ib)
        for (int jb = 0; jb < 2; ++jb) {
            double dte_min = dt_elastic, dtt_min = dtmax_therm, dtm_min = dt_maxwell;
#pragma omp parallel for reduction(min : dte_min, dtt_min, dtm_min) num_threads(g_threads) if (g_threads > 1)
            for (int i = ib; i < nx - 1; i += 2)
                for (int j = jb; j < nz - 1; j += 2) {
                    long long e = s.e(j, i);
                    int iph = L.iphase[e] - 1;
                    double pwave = p.rl[iph] + 0.6666 * p.rm[iph];
                    double dens = p.den[iph];
                    double vel_sound = dlmin * c.frac / dt_elastic;
                    double rho_inert = pwave / (vel_sound * vel_sound);
                    if (p.i_rey == 1 && vel_max > 0.0) {
                        double rho_inert2 = (p.xReyn * p.v_min) / (vel_max * std::fabs(p.rzbo));
                        if (rho_inert > rho_inert2) rho_inert = rho_inert2;
                    }
                    if (p.idt_scale > 0) {
                        double *am = L.amass;
                        long long n11 = o_node(s.d, j, i), n21 = o_node(s.d, j + 1, i), n12 = o_node(s.d, j, i + 1),
                                  n22 = o_node(s.d, j + 1, i + 1);
                        double am3 = c1d12 * rho_inert / s.area(e, 0);
                        am[n11] = am[n11] + am3; am[n21] = am[n21] + am3; am[n12] = am[n12] + am3;
                        am3 = c1d12 * rho_inert / s.area(e, 1);
                        am[n21] = am[n21] + am3; am[n22] = am[n22] + am3; am[n12] = am[n12] + am3;
                        am3 = c1d12 * rho_inert / s.area(e, 2);
                        am[n11] = am[n11] + am3; am[n21] = am[n21] + am3; am[n22] = am[n22] + am3;
                        am3 = c1d12 * rho_inert / s.area(e, 3);
                        am[n11] = am[n11] + am3; am[n22] = am[n22] + am3; am[n12] = am[n12] + am3;
                    } else {
                        double dte = c.frac * dlmin * std::sqrt(dens / pwave);
                        dte_min = std::min(dte_min, dte);
                    }
                    double diff = p.conduct[iph] / p.den[iph] / p.cp[iph];
                    double dtt = dlmin * dlmin / diff;
                    dtt_min = std::min(dtt_min, dtt);
                    if (p.ivis_present == 1) {
                        if ((p.irheol[iph] == 3 || p.irheol[iph] == 12) && p.rm[iph] < 1e11) {
                            double visc_cut = 1e10;
                            double rmu = (p.v_min < visc_cut) ? p.rm[iph] * p.v_min / visc_cut : p.rm[iph];
                            double dt_m = p.v_min / rmu * p.fracm;
                            dtm_min = std::min(dt_m, dtm_min);
                        }
                    }
                }
            dt_elastic = dte_min;
            dtmax_therm = dtt_min;
            dt_maxwell = dtm_min;
        }
    c.dt_elastic = dt_elastic;
    c.dt_maxwell = dt_maxwell;
    c.dtmax_therm = dtmax_therm;
    c.dt = std::min(std::min(dt_elastic, dt_maxwell), dtmax_therm);
}

void init_visc(St &s) {
    int nx = s.p->nx, nz = s.p->nz;
#pragma omp parallel for num_threads(g_threads) if (g_threads > 1)
    for (int i = 0; i < nx - 1; ++i)
        for (int j = 0; j < nz - 1; ++j) s.L->visn[s.e(j, i)] = eff_visc(s, j, i);
}

// --------------------------------------------------------------------------
// fl_therm's magma sub-model (fl_therm.f90:56-391, itype_melting = 1), run
// after temp0 = temp and before the diffusion: freezing of the magma pools
// with its latent heat, the centre and widths of the MOR melting zone,
// migration of the melt (dikes through the crust, percolation through the
// mantle wedge, the MOR pool), then the rate-capped dike release and new
// arc / oceanic-crust markers.  Serial order (i outer, j inner) throughout:
// the reference's atomics and reductions taken in that order.

void therm_magma(St &s) {
    const gf_params &p = *s.p;
    gf_layout &L = *s.L;
    const int nx = p.nx, nz = p.nz, M = GF_MAX_MARKERS_PER_ELEM;
    const double dt = s.c->dt;
    auto X = [&](int j, int i) { return s.cord(j, i, 0); };
    auto Z = [&](int j, int i) { return s.cord(j, i, 1); };
    auto T = [&](int j, int i) -> double & { return L.temp[o_node(s.d, j, i)]; };
    auto T0 = [&](int j, int i) { return L.temp0[o_node(s.d, j, i)]; };
    const double tan_mzone = o_tan(0.5 * p.angle_mzone * 3.14159265358979323846 / 180.0);
    const int ihw = ceil_int(tan_mzone * 200e3 / p.dxmin);
    const double w_barrier = 1.0e-4;

    // freezing: dM = min(M, M dt lambda(T)), latent heat to the 4 corners
    for (int i = 0; i < nx - 1; ++i)
        for (int j = 0; j < nz - 1; ++j) {
            long long e = s.e(j, i);
            double cp_eff = p.cp[L.iphase[e] - 1];
            double tmpr = 0.25 * (T0(j, i) + T0(j + 1, i) + T0(j, i + 1) + T0(j + 1, i + 1));
            double fr_lambda = p.lambda_freeze * o_exp(-p.lambda_freeze_tdep * (tmpr - p.t_top));
            double d1 = fmin2(L.fmagma[e], L.fmagma[e] * dt * fr_lambda);
            double d2 = fmin2(L.fmagma2[e], L.fmagma2[e] * dt * fr_lambda);
            L.fmagma[e] = L.fmagma[e] - d1;
            L.fmagma2[e] = L.fmagma2[e] - d2;
            double dT = d1 * p.latent_heat_magma / cp_eff / 4 + d2 * p.latent_heat_magma / cp_eff / 4;
            T(j, i) = T(j, i) + dT;
            T(j, i + 1) = T(j, i + 1) + dT;
            T(j + 1, i) = T(j + 1, i) + dT;
            T(j + 1, i + 1) = T(j + 1, i + 1) + dT;
        }
    for (long long n = 0; n < s.d.N; ++n) L.temp[n] = fmin2(L.temp[n], p.t_bot);

    // MOR melting zone: fmelt2-weighted centre, the element holding it,
    // then the weighted widths on either side
    double x_sum = 0, z_sum = 0, w_sum = 0;
    for (int i = 0; i < nx - 1; ++i)
        for (int j = 0; j < nz - 1; ++j) {
            double w = L.fmelt2[s.e(j, i)];
            if (w > w_barrier) {
                x_sum = x_sum + 0.25 * (X(j, i) + X(j, i + 1) + X(j + 1, i) + X(j + 1, i + 1)) * w;
                z_sum = z_sum + 0.25 * (Z(j, i) + Z(j, i + 1) + Z(j + 1, i) + Z(j + 1, i + 1)) * w;
                w_sum = w_sum + w;
            }
        }
    bool valid = false;
    int ic = 0, jc = 0; // 0-based element of the centre
    double x_center = 0, z_center = 0, z_surf = 0, h2 = 0, tan_l = 0, tan_r = 0;
    int ihw_l = 0, ihw_r = 0;
    if (w_sum > 0.0) {
        x_center = x_sum / w_sum;
        z_center = z_sum / w_sum;
        for (int i = 0; i < nx - 1 && !valid; ++i)
            for (int j = 0; j < nz - 1; ++j)
                if (X(j, i) <= x_center && X(j, i + 1) >= x_center && Z(j, i) >= z_center && Z(j + 1, i) <= z_center) {
                    ic = i;
                    jc = j;
                    valid = true;
                    break;
                }
    }
    if (valid) {
        double xl = 0, xr = 0, wl = 0, wr = 0;
        for (int i = 0; i < nx - 1; ++i)
            for (int j = 0; j < nz - 1; ++j) {
                double w = L.fmelt2[s.e(j, i)];
                double x = 0.25 * (X(j, i) + X(j, i + 1) + X(j + 1, i) + X(j + 1, i + 1));
                if (w > w_barrier && x < x_center) {
                    xl = xl + (x_center - x) * (x_center - x) * w;
                    wl = wl + w;
                } else if (w > w_barrier && x > x_center) {
                    xr = xr + (x - x_center) * (x - x_center) * w;
                    wr = wr + w;
                }
            }
        xl = 1.8 * std::sqrt(xl / wl);
        xr = 1.8 * std::sqrt(xr / wr);
        if (xl < p.dxmin) xl = p.dxmin;
        if (xr < p.dxmin) xr = p.dxmin;
        if (xl != xl) xl = p.dxmin;
        if (xr != xr) xr = p.dxmin;
        z_surf = 0.5 * (Z(0, ic) + Z(0, ic + 1));
        h2 = z_surf - z_center;
        tan_l = xl / h2;
        tan_r = xr / h2;
        ihw_l = ceil_int(tan_l * 150e3 / p.dxmin);
        ihw_r = ceil_int(tan_r * 150e3 / p.dxmin);
    }

    // migration (1-based column / row numbers as in the reference)
    std::vector<double> dike_added(s.d.E, 0.0);
    for (int i = 0; i < nx - 1; ++i)
        for (int j = 0; j < nz - 1; ++j) {
            long long e = s.e(j, i);
            const int i1 = i + 1, j1 = j + 1, jm = L.jmoho[i];
            double quad_area = 0.5 / s.area(e, 0) + 0.5 / s.area(e, 1);
            if (j1 > jm && L.fmelt[e] > 0) {
                // crust: dikes over nelem_dike columns, from the topmost
                // non-sediment element down to the Moho
                double area_ratio = (Z(0, i) + Z(0, i + 1) - Z(jm - 1, i) - Z(jm - 1, i + 1)) /
                                    (Z(j, i) + Z(j, i + 1) - Z(j + 1, i) - Z(j + 1, i + 1));
                const int nd = p.nelem_dike;
                int ihalf = std::max(0, (nd - 1) / 2);
                int ii_start = std::max(1, i1 - ihalf);
                int ii_end = std::min(nx - 1, ii_start + std::max(1, nd) - 1);
                ii_start = std::max(1, ii_end - std::max(1, nd) + 1);
                int ncol = ii_end - ii_start + 1;
                for (int ii = ii_start; ii <= ii_end; ++ii) {
                    int jtop = 1;
                    while (jtop < L.jmoho[ii - 1] &&
                           (L.iphase[s.e(jtop - 1, ii - 1)] == K_SED1 || L.iphase[s.e(jtop - 1, ii - 1)] == K_SED2))
                        ++jtop;
                    for (int jj = jtop; jj <= L.jmoho[ii - 1]; ++jj) {
                        long long t = s.e(jj - 1, ii - 1);
                        L.fmagma[t] = L.fmagma[t] + L.fmelt[e] * p.ratio_crust_mzone * area_ratio * p.prod_magma * dt / ncol;
                        dike_added[t] = dike_added[t] + L.fmelt[e] * p.ratio_crust_mzone * area_ratio * p.prod_magma * dt / ncol;
                    }
                }
                // mantle: percolation upwards within the cone of half
                // angle angle_mzone / 2 above the melting element
                double z_moho = 0.5 * (Z(jm - 1, i) + Z(jm - 1, i + 1));
                double z_melt = 0.5 * (Z(j + 1, i) + Z(j + 1, i + 1));
                double x_melt = 0.5 * (X(j + 1, i) + X(j + 1, i + 1));
                double h = z_moho - z_melt;
                area_ratio = h * h * tan_mzone / quad_area;
                for (int ii = std::max(1, i1 - ihw); ii <= std::min(nx - 1, i1 + ihw); ++ii)
                    for (int jj = L.jmoho[ii - 1] + 1; jj <= j1; ++jj) {
                        double x = 0.5 * (X(jj - 1, ii - 1) + X(jj - 1, ii));
                        double z = 0.5 * (Z(jj - 1, ii - 1) + Z(jj - 1, ii));
                        if (std::fabs(x - x_melt) <= tan_mzone * (z - z_melt)) {
                            long long t = s.e(jj - 1, ii - 1);
                            L.fmagma[t] = L.fmagma[t] + L.fmelt[e] * p.ratio_mantle_mzone * area_ratio * p.prod_magma * dt;
                        }
                    }
            }
            if (L.fmelt2[e] > 0 && valid) {
                // MOR melt: into the zone above the melting centre
                double area_ratio = 0.5 * (h2 * h2 * tan_l / quad_area + h2 * h2 * tan_r / quad_area);
                for (int ii = std::max(1, ic + 1 - ihw_l); ii <= std::min(nx - 1, ic + 1 + ihw_r); ++ii)
                    for (int jj = 1; jj <= jc + 1; ++jj) {
                        double x = 0.5 * (X(jj - 1, ii - 1) + X(jj - 1, ii));
                        double z = 0.5 * (Z(jj - 1, ii - 1) + Z(jj - 1, ii));
                        long long t = s.e(jj - 1, ii - 1);
                        if (x < x_center && std::fabs(x_center - x) <= tan_l * (z_surf - z)) {
                            L.fmagma2[t] = L.fmagma2[t] + L.fmelt2[e] * area_ratio * p.prod_magma2 * dt;
                            L.mor_marker_vol[t] = L.mor_marker_vol[t] + L.fmelt2[e] * area_ratio * p.prod_magma2 * dt;
                        }
                        if (x >= x_center && std::fabs(x - x_center) <= tan_r * (z_surf - z)) {
                            L.fmagma2[t] = L.fmagma2[t] + L.fmelt2[e] * area_ratio * p.prod_magma2 * dt;
                            L.mor_marker_vol[t] = L.mor_marker_vol[t] + L.fmelt2[e] * area_ratio * p.prod_magma2 * dt;
                        }
                    }
            }
            L.fmagma[e] = fmin2(L.fmagma[e], p.fmagma_max);
            L.fmagma2[e] = fmin2(L.fmagma2[e], p.fmagma_max);
        }

    // dike release, capped at 1e-4 Amin per step, and new markers at the
    // element centre once a marker's share of the element has accumulated
    for (int i = 0; i < nx - 1; ++i)
        for (int j = 0; j < nz - 1; ++j) {
            long long e = s.e(j, i);
            double elem_area = 0.5 / s.area(e, 0) + 0.5 / s.area(e, 1);
            double pending = dike_added[e] * elem_area + L.dike_backlog[e];
            double released = fmin2(pending, 1.0e-4 * p.Amin);
            L.dike_backlog[e] = pending - released;
            L.dike_released[e] = released / elem_area;
            L.dike_marker_vol[e] = L.dike_marker_vol[e] + released;
            for (int path = 0; path < 2; ++path) {
                double &vol = path == 0 ? L.dike_marker_vol[e] : L.mor_marker_vol[e];
                int kinc = L.nmark_elem[e];
                if (kinc > 0 && kinc < M) {
                    double unit = elem_area / kinc;
                    if (vol >= unit) {
                        int n_to_add = std::min(ceil_int(vol / unit), M - kinc);
                        double xc = 0.25 * (X(j, i) + X(j + 1, i) + X(j, i + 1) + X(j + 1, i + 1));
                        double yc = 0.25 * (Z(j, i) + Z(j + 1, i) + Z(j, i + 1) + Z(j + 1, i + 1));
                        for (int k = 0; k < n_to_add; ++k)
                            add_marker(s, xc, yc, path == 0 ? K_ARC1 : K_OCEAN1, s.c->time, j, i);
                        vol = 0.0;
                        count_phase_ratio(s, j, i);
                    }
                }
            }
        }
}

// --------------------------------------------------------------------------
// fl_therm (src/fl_therm.f90:4-598): temp0 = temp, the magma sub-model when
// itype_melting = 1, then the explicit diffusion and the boundary values.

void fl_therm(St &s) {
    const gf_params &p = *s.p;
    gf_layout &L = *s.L;
    double dt = s.c->dt;
    int nx = p.nx, nz = p.nz;
    std::memcpy(L.temp0, L.temp, sizeof(double) * (size_t)s.d.N);
    if (p.itype_melting == 1) therm_magma(s);
    std::vector<double> diff(s.d.E), src(s.d.E);
#pragma omp parallel for num_threads(g_threads) if (g_threads > 1)
    for (int i = 0; i < nx - 1; ++i)
        for (int j = 0; j < nz - 1; ++j) {
            long long e = s.e(j, i);
            int iph = L.iphase[e] - 1;
            double cp_eff = p.cp[iph], cond_eff = p.conduct[iph];
            double dissip = (p.ishearh == 1 && p.itherm != 2) ? L.shrheat[e] : 0;
            diff[e] = cond_eff / p.den[iph] / cp_eff;
            src[e] = (L.source[e] + dissip / p.den[iph]) / cp_eff;
        }
    auto C = [&](int j, int i, int k) { return L.cord[o_n2(s.d, j, i, k)]; };
    auto T = [&](int j, int i) { return L.temp[o_node(s.d, j, i)]; };
    // in place, lexicographic (i outer, j inner): a Gauss-Seidel sweep
#pragma omp parallel for num_threads(g_threads) if (g_threads > 1)
    for (int i = 0; i < nx; ++i)
        for (int j = 0; j < nz; ++j) {
            double rhs = 0.0, area_n = 0.0;
            if (j != 0 && i != 0) { // element (j-1,i-1), triangle B
                long long e = s.e(j - 1, i - 1);
                double a = s.area(e, 1), inv_area = 1.0 / a, ra = inv_area / 6.0;
                area_n = area_n + ra;
                double y2 = C(j, i - 1, 1), y3 = C(j - 1, i, 1), y4 = C(j, i, 1);
                double x2 = C(j, i - 1, 0), x3 = C(j - 1, i, 0), x4 = C(j, i, 0);
                double d1 = (y2 - y4) * a, d2 = (y4 - y3) * a, d3 = (y3 - y2) * a;
                double z1 = (x4 - x2) * a, z2 = (x3 - x4) * a, z3 = (x2 - x3) * a;
                rhs = rhs + src[e] * ra -
                      0.5 * diff[e] * inv_area *
                          (T(j - 1, i) * (d1 * d3 + z1 * z3) + T(j, i - 1) * (d2 * d3 + z2 * z3) + T(j, i) * (d3 * d3 + z3 * z3));
            }
            if (j != 0 && i != nx - 1) { // element (j-1,i), triangles A and B
                long long e = s.e(j - 1, i);
                double a = s.area(e, 0), inv_area = 1.0 / a, ra = inv_area / 6.0;
                area_n = area_n + ra;
                double y1 = C(j - 1, i, 1), y2 = C(j, i, 1), y3 = C(j - 1, i + 1, 1);
                double x1 = C(j - 1, i, 0), x2 = C(j, i, 0), x3 = C(j - 1, i + 1, 0);
                double d1 = (y2 - y3) * a, d2 = (y3 - y1) * a, d3 = (y1 - y2) * a;
                double z1 = (x3 - x2) * a, z2 = (x1 - x3) * a, z3 = (x2 - x1) * a;
                rhs = rhs + src[e] * ra -
                      0.5 * diff[e] * inv_area *
                          (T(j - 1, i) * (d1 * d2 + z1 * z2) + T(j, i) * (d2 * d2 + z2 * z2) + T(j - 1, i + 1) * (d3 * d2 + z3 * z2));
                a = s.area(e, 1); inv_area = 1.0 / a; ra = inv_area / 6.0;
                area_n = area_n + ra;
                y2 = C(j, i, 1); y3 = C(j - 1, i + 1, 1); double y4 = C(j, i + 1, 1);
                x2 = C(j, i, 0); x3 = C(j - 1, i + 1, 0); double x4 = C(j, i + 1, 0);
                d1 = (y2 - y4) * a; d2 = (y4 - y3) * a; d3 = (y3 - y2) * a;
                z1 = (x4 - x2) * a; z2 = (x3 - x4) * a; z3 = (x2 - x3) * a;
                rhs = rhs + src[e] * ra -
                      0.5 * diff[e] * inv_area *
                          (T(j - 1, i + 1) * (d1 * d2 + z1 * z2) + T(j, i) * (d2 * d2 + z2 * z2) + T(j, i + 1) * (d3 * d2 + z3 * z2));
            }
            if (j != nz - 1 && i != 0) { // element (j,i-1), triangles A and B
                long long e = s.e(j, i - 1);
                double a = s.area(e, 0), inv_area = 1.0 / a, ra = inv_area / 6.0;
                area_n = area_n + ra;
                double y1 = C(j, i - 1, 1), y2 = C(j + 1, i - 1, 1), y3 = C(j, i, 1);
                double x1 = C(j, i - 1, 0), x2 = C(j + 1, i - 1, 0), x3 = C(j, i, 0);
                double d1 = (y2 - y3) * a, d2 = (y3 - y1) * a, d3 = (y1 - y2) * a;
                double z1 = (x3 - x2) * a, z2 = (x1 - x3) * a, z3 = (x2 - x1) * a;
                rhs = rhs + src[e] * ra -
                      0.5 * diff[e] * inv_area *
                          (T(j, i - 1) * (d1 * d3 + z1 * z3) + T(j + 1, i - 1) * (d2 * d3 + z2 * z3) + T(j, i) * (d3 * d3 + z3 * z3));
                a = s.area(e, 1); inv_area = 1.0 / a; ra = inv_area / 6.0;
                area_n = area_n + ra;
                y2 = C(j + 1, i - 1, 1); y3 = C(j, i, 1); double y4 = C(j + 1, i, 1);
                x2 = C(j + 1, i - 1, 0); x3 = C(j, i, 0); double x4 = C(j + 1, i, 0);
                d1 = (y2 - y4) * a; d2 = (y4 - y3) * a; d3 = (y3 - y2) * a;
                z1 = (x4 - x2) * a; z2 = (x3 - x4) * a; z3 = (x2 - x3) * a;
                rhs = rhs + src[e] * ra -
                      0.5 * diff[e] * inv_area *
                          (T(j, i) * (d1 * d1 + z1 * z1) + T(j + 1, i - 1) * (d2 * d1 + z2 * z1) + T(j + 1, i) * (d3 * d1 + z3 * z1));
            }
            if (j != nz - 1 && i != nx - 1) { // element (j,i), triangle A
                long long e = s.e(j, i);
                double a = s.area(e, 0), inv_area = 1.0 / a, ra = inv_area / 6.0;
                area_n = area_n + ra;
                double y1 = C(j, i, 1), y2 = C(j + 1, i, 1), y3 = C(j, i + 1, 1);
                double x1 = C(j, i, 0), x2 = C(j + 1, i, 0), x3 = C(j, i + 1, 0);
                double d1 = (y2 - y3) * a, d2 = (y3 - y1) * a, d3 = (y1 - y2) * a;
                double z1 = (x3 - x2) * a, z2 = (x1 - x3) * a, z3 = (x2 - x1) * a;
                rhs = rhs + src[e] * ra -
                      0.5 * diff[e] * inv_area *
                          (T(j, i) * (d1 * d1 + z1 * z1) + T(j + 1, i) * (d2 * d1 + z2 * z1) + T(j, i + 1) * (d3 * d1 + z3 * z1));
            }
            L.temp[o_node(s.d, j, i)] = T(j, i) + rhs * dt / area_n;
        }
    for (int i = 0; i < nx; ++i) {
        L.temp[o_node(s.d, 0, i)] = p.t_top;
        if (p.itemp_bc == 1)
            L.temp[o_node(s.d, nz - 1, i)] = p.bot_bc;
        else if (p.itemp_bc == 2) {
            int ie = std::min(i, nx - 2);
            double cond_eff = p.conduct[L.iphase[s.e(nz - 2, ie)] - 1];
            L.temp[o_node(s.d, nz - 1, i)] = T(nz - 2, i) + p.bot_bc * (C(nz - 2, i, 1) - C(nz - 1, i, 1)) / cond_eff;
        }
    }
    for (int j = 0; j < nz; ++j) {
        L.temp[o_node(s.d, j, 0)] = T(j, 1);
        L.temp[o_node(s.d, j, nx - 1)] = T(j, nx - 2);
    }
}

// --------------------------------------------------------------------------
// Markers: count_phase_ratio, marker2elem, change_phase

void count_phase_ratio(St &s, int j, int i) {
    gf_layout &L = *s.L;
    long long e = s.e(j, i);
    int nm = L.nmark_elem[e];
    if (nm == 0) throw Stop{134};
    int cnt[GF_MAXPH + 1] = {0};
    for (int n = 0; n < nm; ++n) {
        int kk = L.mark_id_elem[e * GF_MAX_MARKERS_PER_ELEM + n];
        int iph = L.mark_phase[kk - 1];
        if (iph >= 1 && iph <= GF_MAXPH) cnt[iph] += 1;
    }
    for (int k = 1; k <= s.p->nphase; ++k) L.phase_ratio[o_pr(s.d, e, k - 1)] = cnt[k] / (nm * 1.0);
    int iph = 1, best = 0;
    for (int k = 1; k <= s.p->nphase; ++k)
        if (cnt[k] > best) {
            best = cnt[k];
            iph = k;
        }
    L.iphase[e] = iph;
}

int check_inside(St &s, double x, double y, double &bar1, double &bar2, int &ntr, int i, int j) {
    for (int k = 0; k < 2; ++k) {
        double x1, x2, x3, y1, y2, y3;
        if (k == 0) {
            x1 = s.cord(j, i, 0); x2 = s.cord(j + 1, i, 0); x3 = s.cord(j, i + 1, 0);
            y1 = s.cord(j, i, 1); y2 = s.cord(j + 1, i, 1); y3 = s.cord(j, i + 1, 1);
        } else {
            x1 = s.cord(j, i + 1, 0); x2 = s.cord(j + 1, i, 0); x3 = s.cord(j + 1, i + 1, 0);
            y1 = s.cord(j, i + 1, 1); y2 = s.cord(j + 1, i, 1); y3 = s.cord(j + 1, i + 1, 1);
        }
        double det = ((x2 * y3 - y2 * x3) - (x1 * y3 - y1 * x3)) + (x1 * y2 - y1 * x2);
        double m11 = (x2 * y3 - y2 * x3) / det, m12 = (y2 - y3) / det, m13 = (x3 - x2) / det;
        double m21 = (x3 * y1 - y3 * x1) / det, m22 = (y3 - y1) / det, m23 = (x1 - x3) / det;
        bar1 = m11 + m12 * x + y * m13;
        bar2 = m21 + m22 * x + y * m23;
        if (bar1 >= 0.0 && bar2 >= 0.0 && bar1 + bar2 <= 1.0) {
            ntr = 2 * ((s.p->nz - 1) * i + j) + k + 1;
            return 1;
        }
    }
    return 0;
}

int add_marker(St &s, double x, double y, int iph, double age, int j, int i) {
    double b1, b2;
    int ntr;
    if (!check_inside(s, x, y, b1, b2, ntr, i, j)) return 0;
    gf_layout &L = *s.L;
    int kk = s.c->nmarkers + 1;
    long long e = s.e(j, i);
    int nm = L.nmark_elem[e] + 1;
    if (nm > GF_MAX_MARKERS_PER_ELEM || kk > L.max_markers) return -1;
    s.c->nmarkers = kk;
    L.nmark_elem[e] = nm;
    L.mark_id_elem[e * GF_MAX_MARKERS_PER_ELEM + (nm - 1)] = kk;
    L.mark_dead[kk - 1] = 1;
    L.mark_a1[kk - 1] = b1;
    L.mark_a2[kk - 1] = b2;
    L.mark_age[kk - 1] = age;
    L.mark_ntriag[kk - 1] = ntr;
    L.mark_phase[kk - 1] = (int8_t)iph;
    return 1;
}

void marker2elem(St &s) {
    int nx = s.p->nx, nz = s.p->nz;
    gf_layout &L = *s.L;
    for (int i = 0; i < nx - 1; ++i)
        for (int j = 0; j < nz - 1; ++j) {
            int iseed = s.c->nloop + (i + 1) + (j + 1);
            int kinc = L.nmark_elem[s.e(j, i)];
            int icount = 0;
            while (kinc <= 4) {
                double r1 = o_myrandom(iseed), r2 = o_myrandom(iseed);
                double x1 = s.cord(j, i, 0) * (1 - r1) + s.cord(j, i + 1, 0) * r1;
                double y1 = s.cord(j, i, 1) * (1 - r1) + s.cord(j, i + 1, 1) * r1;
                double x2 = s.cord(j + 1, i, 0) * (1 - r1) + s.cord(j + 1, i + 1, 0) * r1;
                double y2 = s.cord(j + 1, i, 1) * (1 - r1) + s.cord(j + 1, i + 1, 1) * r1;
                double xx = x1 * (1 - r2) + x2 * r2, yy = y1 * (1 - r2) + y2 * r2;
                int inc = add_marker(s, xx, yy, L.iphase[s.e(j, i)], 0.0, j, i);
                icount = icount + 1;
                if (icount > 100) throw Stop{133};
                if (inc <= 0) continue;
                kinc = kinc + 1;
            }
            count_phase_ratio(s, j, i);
        }
    static const int mantle[5] = {4, 8, 9, 16, 18};
    if (L.jmoho)
        for (int i = 0; i < nx - 1; ++i) {
            L.jmoho[i] = nz - 1;
            for (int j = 0; j < nz - 1; ++j) {
                double sum = 0.0;
                for (int m = 0; m < 5; ++m) sum += s.pr(s.e(j, i), mantle[m]);
                if (sum > 0.5) {
                    L.jmoho[i] = j + 1;
                    break;
                }
            }
        }
}

// --------------------------------------------------------------------------
// Melting (change_phase.f90:264-483, itype_melting = 1): hydrous mantle
// (fmelt2, Katz 2003 solidus), sediments (Nichols 1994), basalt / eclogite
// (Gutscher 2000) and flux melting above serpentinite or chlorite
// (Grove 2009 water-saturated solidus) into fmelt.  A melting element's
// corners are cooled back to the solidus, in place and in serial order, so
// each element sees its predecessors' cooling.

void melting(St &s) {
    const gf_params &p = *s.p;
    gf_layout &L = *s.L;
    const int nx = p.nx, nz = p.nz;
    auto Z = [&](int j, int i) { return s.cord(j, i, 1); };
    auto T = [&](int j, int i) -> double & { return L.temp[o_node(s.d, j, i)]; };
    auto tmpr_of = [&](int j, int i) { return 0.25 * (T(j, i) + T(j, i + 1) + T(j + 1, i) + T(j + 1, i + 1)); };
    auto depth_of = [&](int j, int i) {
        double yy = 0.25 * (Z(j, i) + Z(j, i + 1) + Z(j + 1, i) + Z(j + 1, i + 1));
        return 0.5 * (Z(0, i) + Z(0, i + 1)) - yy;
    };
    auto cool = [&](int j, int i, double dt_melt) {
        T(j, i) = T(j, i) - dt_melt;
        T(j, i + 1) = T(j, i + 1) - dt_melt;
        T(j + 1, i) = T(j + 1, i) - dt_melt;
        T(j + 1, i + 1) = T(j + 1, i + 1) - dt_melt;
    };
    auto pmelt_of = [&](int kph, double over, double span) {
        if (p.latent_heat_magma > 0.0) return fmin2(p.cp[kph - 1] * over / p.latent_heat_magma, 0.1);
        return fmin2(over / span * 0.1, 0.1);
    };
    // hydrous mantle
    for (int i = 0; i < nx - 1; ++i)
        for (int j = 0; j < nz - 1; ++j) {
            long long e = s.e(j, i);
            L.fmelt2[e] = 0;
            double tpr = s.pr(e, K_MANT1) + s.pr(e, K_MANT2);
            if (tpr > 0.6 && Z(j, i) > -150e3) {
                double tmpr = tmpr_of(j, i), depth = depth_of(j, i);
                double press = std::fabs(3000.0 * p.g * depth * 1e-9);
                double solidus = -5.02 * (press * press) + 1.32e2 * press + 1.09e3;
                if (tmpr > solidus) {
                    L.fmelt2[e] = pmelt_of(K_MANT1, tmpr - solidus, 35.0) * tpr;
                    cool(j, i, tmpr - solidus);
                }
            }
        }
    // sediments
    for (int i = 0; i < nx - 1; ++i)
        for (int j = 0; j < nz - 1; ++j) {
            long long e = s.e(j, i);
            L.fmelt[e] = 0;
            double tpr = s.pr(e, K_SED1) + s.pr(e, K_SED2) + s.pr(e, K_METASED) + s.pr(e, K_SCHIST);
            if (tpr > 0.6 && Z(j, i) > -200e3) {
                double tmpr = tmpr_of(j, i), depth = depth_of(j, i);
                double solidus = fmax2(680 + 0.6e-3 * (depth - 140e3), 930 - 313 * (1 - o_exp(-depth / 7e3)));
                if (tmpr > solidus) {
                    L.fmelt[e] = pmelt_of(K_SED2, tmpr - solidus, 50.0) * tpr;
                    cool(j, i, tmpr - solidus);
                }
            }
        }
    // basalt and eclogite
    for (int i = 0; i < nx - 1; ++i)
        for (int j = 0; j < nz - 1; ++j) {
            long long e = s.e(j, i);
            double tpr = s.pr(e, K_OCEAN1) + s.pr(e, K_OCEAN2) + s.pr(e, K_OCEANDRY) + s.pr(e, K_ECLG);
            if (tpr > 0.6 && Z(j, i) > -200e3) {
                double tmpr = tmpr_of(j, i), depth = depth_of(j, i);
                double press = 3000 * 10 * depth / 1e9;
                double solidus;
                if (press < 1.0)
                    solidus = 1050.0 - 420.0 * (1.0 - o_exp(-press * 3.3));
                else if (press > 2.7)
                    solidus = (press + 14.0) * 43.0;
                else
                    solidus = 630.0 + 13.0 * (press * press);
                if (tmpr > solidus) {
                    L.fmelt[e] = L.fmelt[e] + pmelt_of(K_OCEAN1, tmpr - solidus, 20.0) * tpr;
                    cool(j, i, tmpr - solidus);
                }
            }
        }
    // flux melting: above the deepest serpentinite / chlorite element of
    // each column
    for (int i = 0; i < nx - 1; ++i)
        for (int j = nz - 2; j >= 0; --j) {
            long long e = s.e(j, i);
            if (s.pr(e, K_SERP) + s.pr(e, K_HYDMANT) > 0.6 && Z(j, i) > -200e3) {
                for (int jj = j; jj >= 0; --jj) {
                    long long t = s.e(jj, i);
                    double tmpr = tmpr_of(jj, i), depth = depth_of(jj, i);
                    double solidus;
                    if (depth > 80e3)
                        solidus = 800;
                    else
                        solidus = 800 + (double)6.2e-8f * ((depth - 80e3) * (depth - 80e3));
                    if (tmpr > solidus) {
                        L.fmelt[t] = L.fmelt[t] + pmelt_of(K_MANT1, tmpr - solidus, 50.0) *
                                                      (s.pr(t, K_MANT1) + s.pr(t, K_MANT2) + s.pr(t, K_SERP));
                        cool(jj, i, tmpr - solidus);
                    }
                }
                break;
            }
        }
}

// change_phase (src/change_phase.f90:35-262), then melting when
// itype_melting = 1.
void change_phase(St &s) {
    const gf_params &p = *s.p;
    gf_layout &L = *s.L;
    int nx = p.nx, nz = p.nz;
    const double max_basalt_depth = 150e3, min_eclogite_temp = 400.0, min_eclogite_depth = 20e3,
                 mantle_density = 3000.0, max_melting_depth = 200e3, serpentine_temp = 550.0;
    std::vector<uint8_t> itmp(s.d.E, 0);
    int nmk = s.c->nmarkers;
#pragma omp parallel for schedule(guided) num_threads(g_threads) if (g_threads > 1)
    for (int kk = 0; kk < nmk; ++kk) {
        if (L.mark_dead[kk] == 0) continue;
        int n = L.mark_ntriag[kk];
        int k = (n - 1) % 2 + 1;
        int j = ((n - k) / 2) % (nz - 1);
        int i = (n - k) / 2 / (nz - 1);
        double a1 = L.mark_a1[kk], a2 = L.mark_a2[kk];
        double yy, tmpr;
        auto Tn = [&](int jj, int ii) { return L.temp[o_node(s.d, jj, ii)]; };
        if (k == 1) {
            yy = s.cord(j, i, 1) * a1 + s.cord(j + 1, i, 1) * a2 + s.cord(j, i + 1, 1) * (1 - a1 - a2);
            tmpr = Tn(j, i) * a1 + Tn(j + 1, i) * a2 + Tn(j, i + 1) * (1 - a1 - a2);
        } else {
            yy = s.cord(j, i + 1, 1) * a1 + s.cord(j + 1, i, 1) * a2 + s.cord(j + 1, i + 1, 1) * (1 - a1 - a2);
            tmpr = Tn(j, i + 1) * a1 + Tn(j + 1, i) * a2 + Tn(j + 1, i + 1) * (1 - a1 - a2);
        }
        double depth = 0.5 * (s.cord(0, i, 1) + s.cord(0, i + 1, 1)) - yy;
        if (depth > max_melting_depth) continue;
        int iph = L.mark_phase[kk];
        long long e = s.e(j, i);
        int newph = 0;
        switch (iph) {
        case 2: case 6:
            break;
        case 4: case 8: {
            if (depth > max_basalt_depth) break;
            double trpres = 2.1e9 + (7.5e9 - 2.1e9) * (tmpr - 730.0) / (500.0 - 730.0);
            double trpres2 = 2.1e9 + (0.6e9 - 2.1e9) * (tmpr - 730.0) / (670.0 - 730.0);
            double press = mantle_density * p.g * depth;
            double pg = std::fabs(press * 1e-9);
            double solidus = -5.02 * (pg * pg) + 1.32e2 * pg + 1.09e3 + 35.0;
            if (press < trpres && press > trpres2) {
                int jb0 = std::min(j + 2, nz - 1), jb1 = std::min(j + 1 + p.nelem_serp, nz - 1);
                for (int jb = jb0; jb <= jb1; ++jb) {
                    long long eb = s.e(jb - 1, i);
                    if (s.pr(eb, 3) > 0.8 || s.pr(eb, 7) > 0.8 || s.pr(eb, 1) > 0.8 || s.pr(eb, 11) > 0.8) {
                        newph = 9;
                        break;
                    }
                }
            } else if (tmpr >= solidus + 35.0) {
                newph = 18;
            }
            break;
        }
        case 10: case 3: case 7: {
            double press = mantle_density * p.g * depth;
            if (p.eclogite_rule == 1) {
                if (tmpr >= 600.0 && press >= 1.5e9) newph = 13;
            } else {
                double trpres = -0.3e9 + 2.2e6 * tmpr;
                double trpres2 = 20.1e9 - 0.0375e9 * tmpr;
                if (!(tmpr < min_eclogite_temp || depth < min_eclogite_depth || press < trpres || press < trpres2)) newph = 13;
            }
            break;
        }
        case 9: {
            double trpres = 2.1e9 + (7.5e9 - 2.1e9) * (tmpr - 730.0) / (500.0 - 730.0);
            double trpres2 = 2.1e9 + (0.2e9 - 2.1e9) * (tmpr - 730.0) / (650.0 - 730.0);
            double press = mantle_density * p.g * depth;
            if (!(tmpr < serpentine_temp || (press < trpres && press > trpres2))) newph = 4;
            break;
        }
        case 1:
            if (!(tmpr < 80.0 && depth < 2e3)) newph = 11;
            break;
        case 11:
            if (!(tmpr < 250.0 && depth < 7e3)) newph = 17;
            break;
        case 17: {
            double trpres = 0.88e9 - (0.88e9 - 0.704e9) * (710.8 - tmpr) / (710.8 - 662.3);
            double press = mantle_density * p.g * depth;
            if (!(press < trpres)) newph = 5;
            break;
        }
        case 5: {
            double trpres = 0.0e9 - (0.0e9 - 1.2e9) * (500.0 - tmpr) / (500.0 - 600.0);
            double press = mantle_density * p.g * depth;
            if (!(press > trpres)) newph = 19;
            break;
        }
        case 16: {
            double dd = depth - 62e3;
            double trtmpr = 880 - 35e-9 * (dd * dd);
            if (!(tmpr < trtmpr)) newph = 4;
            break;
        }
        default:
            break;
        }
        if (newph) {
            itmp[e] = 1;
            L.mark_phase[kk] = (int8_t)newph;
        }
    }
    int err = 0;
#pragma omp parallel for num_threads(g_threads) if (g_threads > 1)
    for (int i = 0; i < nx - 1; ++i)
        for (int j = 0; j < nz - 1; ++j) {
            long long e = s.e(j, i);
            if (!itmp[e]) continue;
            try {
                count_phase_ratio(s, j, i);
            } catch (const Stop &st) {
#pragma omp critical
                err = st.code;
            }
            int kinc = L.nmark_elem[e];
            double a0 = L.aps[e];
            L.aps[e] = std::max(a0 - a0 / (double)(float)kinc, 0.0);
        }
    if (err) throw Stop{err};
    if (p.itype_melting == 1) melting(s);
}

// --------------------------------------------------------------------------
// itest_mesh (src/rem_test.f90:70-136), angle criterion only

double min_angle(St &s) {
    int nx = s.p->nx, nz = s.p->nz;
    const double pi = 3.14159265358979323846, raddeg = 180.0 / pi;
    double anglemint = 180.0;
#pragma omp parallel for reduction(min : anglemint) num_threads(g_threads) if (g_threads > 1)
    for (int i = 0; i < nx - 1; ++i)
        for (int j = 0; j < nz - 1; ++j)
            for (int t = 0; t < 4; ++t) {
                int iv[4], jv[4];
                if (t == 0) { iv[0] = i; jv[0] = j; iv[1] = i; jv[1] = j + 1; iv[2] = i + 1; jv[2] = j; }
                else if (t == 1) { iv[0] = i; jv[0] = j + 1; iv[1] = i + 1; jv[1] = j + 1; iv[2] = i + 1; jv[2] = j; }
                else if (t == 2) { iv[0] = i; jv[0] = j; iv[1] = i; jv[1] = j + 1; iv[2] = i + 1; jv[2] = j + 1; }
                else { iv[0] = i; jv[0] = j; iv[1] = i + 1; jv[1] = j + 1; iv[2] = i + 1; jv[2] = j; }
                iv[3] = iv[0]; jv[3] = jv[0];
                double ang[3];
                for (int k = 1; k <= 2; ++k) {
                    double xa = s.cord(jv[k + 1], iv[k + 1], 0) - s.cord(jv[k], iv[k], 0);
                    double ya = s.cord(jv[k + 1], iv[k + 1], 1) - s.cord(jv[k], iv[k], 1);
                    double xxal = std::sqrt(xa * xa + ya * ya);
                    double xb = s.cord(jv[k - 1], iv[k - 1], 0) - s.cord(jv[k], iv[k], 0);
                    double yb = s.cord(jv[k - 1], iv[k - 1], 1) - s.cord(jv[k], iv[k], 1);
                    double xxbl = std::sqrt(xb * xb + yb * yb);
                    ang[k] = raddeg * std::acos((xa * xb + ya * yb) / (xxal * xxbl));
                }
                ang[0] = 180.0 - ang[1] - ang[2];
                double m = std::min(ang[0], std::min(ang[1], ang[2]));
                anglemint = std::min(anglemint, m);
            }
    return anglemint;
}

// --------------------------------------------------------------------------
// Remesh event (src/par.f90:94-110): bar2euler, remesh, lpeuler2bar,
// marker2elem.

double ipow(double x, int m) {
    unsigned n = m < 0 ? (unsigned)(-m) : (unsigned)m;
    double y = (n % 2) ? x : 1.0;
    while (n >>= 1) {
        x = x * x;
        if (n % 2) y = y * x;
    }
    return m < 0 ? 1.0 / y : y;
}

// mesh1 (init_cord.f90:141-179)
void mesh1(double x1, double x2, double *xmesh, int n, int nzon, const int *nelz, const double *sizez) {
    double all_ratio = 0.0;
    int nel = 0;
    xmesh[0] = 0.0;
    for (int k = 0; k < nzon - 1; k += 2) {
        all_ratio = all_ratio + nelz[k] * sizez[k];
        for (int i = 0; i < nelz[k]; ++i) {
            nel = nel + 1;
            xmesh[nel] = xmesh[nel - 1] + sizez[k];
        }
        double ratio = std::pow(sizez[k + 2] / sizez[k], 1.0 / (double)(nelz[k + 1] + 1));
        for (int i = 1; i <= nelz[k + 1]; ++i) {
            nel = nel + 1;
            xmesh[nel] = xmesh[nel - 1] + sizez[k] * ipow(ratio, i);
            all_ratio = all_ratio + sizez[k] * ipow(ratio, i);
        }
    }
    for (int k = 0; k < nelz[nzon - 1]; ++k) {
        nel = nel + 1;
        xmesh[nel] = xmesh[nel - 1] + sizez[nzon - 1];
    }
    all_ratio = all_ratio + nelz[nzon - 1] * sizez[nzon - 1];
    double magnification = (x2 - x1) / all_ratio;
    for (int k = 0; k < n; ++k) xmesh[k] = x1 + xmesh[k] * magnification;
}

// init_geotherm_profile (init_temp.f90:127-310) for node column i (0-based)
void geotherm_column(St &s, int n, int i, double age_1n, double tp1n, double tp2n) {
    const gf_params &p = *s.p;
    gf_layout &L = *s.L;
    int nz = p.nz, nx = p.nx;
    const double pi = 3.14159265358979323846;
    double t_top = p.t_top, t_bot = p.t_bot;
    auto T = [&](int j) -> double & { return L.temp[o_node(s.d, j, i)]; };
    auto Y = [&](int j) { return s.cord(j, i, 1); };
    int ic = p.ictherm[n];
    if (ic == 1) {
        for (int j = 0; j < nz; ++j) {
            double f = (Y(0) - Y(j)) / std::sqrt(4 * 1e-6 * age_1n * 1e6 * GF_SEC_YEAR);
            T(j) = t_top + (t_bot - t_top) * std::erf(f);
        }
    } else if (ic == 2 || ic == 12) {
        double yL0 = tp1n, age_init = age_1n * GF_SEC_YEAR * 1e6, tau_d = yL0 * yL0 * 1e6 / (pi * pi * 1e-6);
        double cond = 3.3, dens_c = 2700.0, ymoho = tp2n, tm = 0, qm = 0;
        if (ic == 12) {
            double rr = ymoho / (yL0 - ymoho);
            tm = (t_top + rr * t_bot + dens_c * p.hs * p.hr * p.hr * 1e6 / cond * (1.0 - std::exp(-ymoho / p.hr))) / (1 + rr);
            qm = cond * (t_bot - tm) / (yL0 - ymoho);
        }
        for (int j = 0; j < nz; ++j) {
            double y = (Y(0) - Y(j)) * 1e-3;
            double tss;
            if (ic == 2)
                tss = t_top + (t_bot - t_top) * y / yL0;
            else if (y <= ymoho)
                tss = t_top + qm / cond * y + (dens_c * p.hs * p.hr * p.hr * 1e6 / cond) * (1.0 - std::exp(-y / p.hr));
            else if (y <= yL0)
                tss = tm + qm / cond * (y - ymoho);
            else
                tss = t_bot;
            double tt = 0.0;
            for (int k = 1; k <= 100; ++k) tt = tt + 1.0 / k * std::exp(-k * k * age_init / tau_d) * std::sin(pi * k * y / yL0);
            T(j) = tss + 2.0 / pi * (t_bot - t_top) * tt;
            if (T(j) > t_bot || y > yL0) T(j) = t_bot;
        }
    } else if (ic == 21) {
        for (int j = 0; j < nz; ++j) {
            double y = (Y(0) - Y(j)) * 1e-3;
            T(j) = y * (t_bot - t_top) / age_1n;
            if (T(j) > t_bot) T(j) = t_bot;
        }
    } else if (ic == 22) {
        for (int j = 0; j < nz; ++j) {
            double y = (Y(0) - Y(j)) * 1e-3;
            if (y <= tp1n)
                T(j) = t_top + (age_1n - t_top) * y / tp1n;
            else
                T(j) = age_1n + (t_bot - age_1n) * (y - tp1n) / (tp2n - tp1n);
            if (T(j) > t_bot) T(j) = t_bot;
        }
    } else if (ic == 13) {
        double cond_c = 2.3, cond_m = 3.3, Fpart = 0.74, alc = 0.4e-6, am = 0.02e-6;
        double auc = (1.0 - Fpart) * age_1n * 1.0e-3 / (tp1n * 1000.0);
        double Q = age_1n * 1.0e-3;
        T(0) = t_top;
        int kl = 0;
        for (int j = 0; j < nz - 1; ++j) {
            double y = (Y(0) - Y(j)) * 1.0e-3, xdz = std::fabs(Y(j + 1) - Y(j));
            double *src = (i < nx - 1) ? &L.source[s.e(j, i)] : nullptr;
            double Qn = Q;
            if (y < tp1n) {
                T(j + 1) = T(j) + (Q / cond_c) * xdz - (auc) / (2.0 * cond_c) * (xdz * xdz);
                Qn = Q - auc * xdz;
                if (src) *src = auc * 1.0e-3;
            }
            if (y >= tp1n && y < (tp2n + tp1n)) {
                T(j + 1) = T(j) + (Q / cond_c) * xdz - (alc) / (2.0 * cond_c) * (xdz * xdz);
                Qn = Q - alc * xdz;
                if (src) *src = alc * 1.0e-3;
            }
            if (y >= (tp2n + tp1n) && kl == 0) {
                T(j + 1) = T(j) + (Q / cond_m) * xdz - (am) / (2.0 * cond_m) * (xdz * xdz);
                Qn = Q - am * xdz;
                if (src) *src = am * 1.0e-3;
                if (T(j + 1) >= t_bot) kl = 1;
            }
            if (kl == 1) {
                T(j + 1) = t_bot;
                if (src) *src = 0.0;
            }
            Q = Qn;
        }
    } else {
        throw Stop{1};
    }
}

// marker2xy (bar2euler.f90:73-117); bar2euler writes x,y into mark_a1/a2
void bar2euler(St &s) {
    gf_layout &L = *s.L;
    int nz = s.p->nz;
    for (int m = 0; m < s.c->nmarkers; ++m) {
        if (L.mark_dead[m] == 0) continue;
        int n = L.mark_ntriag[m];
        int k = (n - 1) % 2 + 1;
        int jj = ((n - k) / 2) % (nz - 1);
        int ii = (n - k) / 2 / (nz - 1);
        double ba1 = L.mark_a1[m], ba2 = L.mark_a2[m];
        double ba3 = 1.0 - ba1 - ba2;
        int i1, i2, i3, j1, j2, j3;
        if (k == 1) {
            i1 = ii; i2 = ii; i3 = ii + 1; j1 = jj; j2 = jj + 1; j3 = jj;
        } else {
            i1 = ii + 1; i2 = ii; i3 = ii + 1; j1 = jj; j2 = jj + 1; j3 = jj + 1;
        }
        double x = s.cord(j1, i1, 0) * ba1 + s.cord(j2, i2, 0) * ba2 + s.cord(j3, i3, 0) * ba3;
        double y = s.cord(j1, i1, 1) * ba1 + s.cord(j2, i2, 1) * ba2 + s.cord(j3, i3, 1) * ba3;
        if (L.dhacc_correction) {
            if (j1 == 0) y = y - L.dhacc_correction[i1] * ba1;
            if (j2 == 0) y = y - L.dhacc_correction[i2] * ba2;
            if (j3 == 0) y = y - L.dhacc_correction[i3] * ba3;
        }
        L.mark_a1[m] = x;
        L.mark_a2[m] = y;
    }
}

// euler2bar (euler2bar.f90:1-98): the element itself, then rings of 2, 6, 12
int euler2bar(St &s, double x, double y, double &b1, double &b2, int &ntr, int &ii, int &jj) {
    int nx = s.p->nx, nz = s.p->nz;
    if (check_inside(s, x, y, b1, b2, ntr, ii, jj)) return 1;
    const int rings[3] = {2, 6, 12};
    for (int r = 0; r < 3; ++r) {
        int n = rings[r], prev = r == 0 ? 0 : rings[r - 1];
        for (int j = std::max(0, jj - n); j <= std::min(nz - 2, jj + n); ++j)
            for (int i = std::max(0, ii - n); i <= std::min(nx - 2, ii + n); ++i) {
                if (r == 0) {
                    if (i == ii && j == jj) continue;
                } else if (std::abs(i - ii) <= prev && std::abs(j - jj) <= prev) {
                    continue;
                }
                if (check_inside(s, x, y, b1, b2, ntr, i, j)) {
                    ii = i;
                    jj = j;
                    return 1;
                }
            }
    }
    return 0;
}

// lpeuler2bar (lpeuler2bar.f90:1-62), serial marker order
void lpeuler2bar(St &s) {
    gf_layout &L = *s.L;
    int nz = s.p->nz;
    std::memset(L.mark_id_elem, 0, sizeof(int) * (size_t)s.d.E * GF_MAX_MARKERS_PER_ELEM);
    std::memset(L.nmark_elem, 0, sizeof(int) * (size_t)s.d.E);
    for (int m = 0; m < s.c->nmarkers; ++m) {
        if (L.mark_dead[m] == 0) continue;
        int nt = L.mark_ntriag[m];
        int k = (nt - 1) % 2 + 1;
        int j = ((nt - k) / 2) % (nz - 1);
        int i = (nt - k) / 2 / (nz - 1);
        double xx = L.mark_a1[m], yy = L.mark_a2[m], b1, b2;
        int ntr;
        if (!euler2bar(s, xx, yy, b1, b2, ntr, i, j)) {
            L.mark_dead[m] = 0;
            continue;
        }
        L.mark_a1[m] = b1;
        L.mark_a2[m] = b2;
        L.mark_ntriag[m] = ntr;
        long long e = s.e(j, i);
        if (L.nmark_elem[e] == GF_MAX_MARKERS_PER_ELEM) {
            L.mark_dead[m] = 0;
            continue;
        }
        L.nmark_elem[e] += 1;
        L.mark_id_elem[e * GF_MAX_MARKERS_PER_ELEM + L.nmark_elem[e] - 1] = m + 1;
    }
}

// rem_cord (rem_cord.f90:1-81)
void rem_cord(St &s, const std::vector<double> &cordo) {
    const gf_params &p = *s.p;
    int nx = p.nx, nz = p.nz;
    std::vector<double> st(std::max(nx, nz) + 2);
    auto CO = [&](int j, int i, int k) { return cordo[o_n2(s.d, j, i, k)]; };
    for (int j = 0; j < nz; ++j) {
        double xl = 0, xr = 0;
        if (p.mode_rem == 1) {
            xl = s.cord(j, 0, 0);
            xr = s.cord(j, nx - 1, 0);
        } else if (p.mode_rem == 11 || p.mode_rem == 3) {
            xl = p.x0;
            xr = p.x0 + p.rxbo;
        } else if (p.mode_rem == 4) {
            xl = s.cord(0, 0, 0);
            xr = s.cord(0, nx - 1, 0);
        }
        mesh1(xl, xr, st.data(), nx, p.nzonx, p.nelz_x, p.sizez_x);
        for (int i = 0; i < nx; ++i) s.cordr(j, i, 0) = st[i];
    }
    bool is_flex = false;
    for (int b = 0; b < p.nofbc; ++b)
        if (p.nbc[b] == 200 && p.nofside[b] == 2) is_flex = true;
    for (int i = 0; i < nx; ++i) {
        for (int j = 0; j < nz; j += nz - 1) {
            double xx = s.cord(j, i, 0);
            if (xx <= CO(j, 0, 0))
                s.cordr(j, i, 1) = CO(j, 0, 1);
            else if (xx >= CO(j, nx - 1, 0))
                s.cordr(j, i, 1) = CO(j, nx - 1, 1);
            else
                for (int ii = 0; ii < nx - 1; ++ii) {
                    double xl = CO(j, ii, 0), xr = CO(j, ii + 1, 0);
                    if (xx >= xl && xx <= xr) {
                        double zl = CO(j, ii, 1), zr = CO(j, ii + 1, 1);
                        s.cordr(j, i, 1) = zl + (xx - xl) * (zr - zl) / (xr - xl);
                        break;
                    }
                }
            if (nz == 1) break;
        }
        if (!is_flex && (p.mode_rem == 3 || p.mode_rem == 1)) s.cordr(nz - 1, i, 1) = p.z0 + p.rzbo;
        mesh1(s.cord(0, i, 1), s.cord(nz - 1, i, 1), st.data(), nz, p.nzony, p.nelz_y, p.sizez_y);
        for (int j = 0; j < nz; ++j) s.cordr(j, i, 1) = st[j];
    }
}

// rem_trpars / rem_barcord / rem_interpolate (remesh.f90:267-491) on a
// (nzt x nxt) point grid with old points `cold` and new points `cnew`
struct Interp {
    int nzt, nxt;
    std::vector<int> numtr;
    std::vector<double> bc; // 3 per point
};

Interp rem_barcord(const std::vector<double> &cold, const std::vector<double> &cnew, int nzt, int nxt) {
    auto OX = [&](int j, int i) { return cold[(size_t)2 * ((size_t)i * nzt + j)]; };
    auto OY = [&](int j, int i) { return cold[(size_t)2 * ((size_t)i * nzt + j) + 1]; };
    // rem_trpars
    size_t ntri = (size_t)2 * (nzt - 1) * (nxt - 1);
    std::vector<double> pt(ntri * 6);
    for (int i = 0; i < nxt - 1; ++i)
        for (int j = 0; j < nzt - 1; ++j)
            for (int k = 1; k <= 2; ++k) {
                double x1, x2, x3, y1, y2, y3;
                if (k == 1) {
                    x1 = OX(j, i); x2 = OX(j + 1, i); x3 = OX(j, i + 1);
                    y1 = OY(j, i); y2 = OY(j + 1, i); y3 = OY(j, i + 1);
                } else {
                    x1 = OX(j, i + 1); x2 = OX(j + 1, i); x3 = OX(j + 1, i + 1);
                    y1 = OY(j, i + 1); y2 = OY(j + 1, i); y3 = OY(j + 1, i + 1);
                }
                double det = ((x2 * y3 - y2 * x3) - (x1 * y3 - y1 * x3)) + (x1 * y2 - y1 * x2);
                size_t n = (size_t)2 * ((size_t)(nzt - 1) * i + j) + (k - 1);
                double *q = &pt[n * 6];
                q[0] = (x2 * y3 - y2 * x3) / det;
                q[1] = (y2 - y3) / det;
                q[2] = (x3 - x2) / det;
                q[3] = (x3 * y1 - y3 * x1) / det;
                q[4] = (y3 - y1) / det;
                q[5] = (x1 - x3) / det;
            }
    Interp r{nzt, nxt, std::vector<int>((size_t)nzt * nxt), std::vector<double>((size_t)3 * nzt * nxt)};
    const double perr = 1e-4;
    const int mm = 4;
    for (int i = 0; i < nxt; ++i)
        for (int j = 0; j < nzt; ++j) {
            size_t pidx = (size_t)i * nzt + j;
            double xx = cnew[2 * pidx], yy = cnew[2 * pidx + 1];
            double amodmin = 1e10;
            int nmin = 0, found = 0;
            for (int io = std::max(0, i - mm); io <= std::min(nxt - 2, i + mm) && !found; ++io)
                for (int jo = std::max(0, j - mm); jo <= std::min(nzt - 2, j + mm) && !found; ++jo)
                    for (int k = 1; k <= 2; ++k) {
                        int n1 = 2 * ((nzt - 1) * io + jo) + k; // 1-based triangle number
                        const double *q = &pt[(size_t)(n1 - 1) * 6];
                        double a1 = q[0] + xx * q[1] + yy * q[2];
                        double a2 = q[3] + xx * q[4] + yy * q[5];
                        double a3 = 1.0 - a1 - a2;
                        double amod = a1 * a1 + a2 * a2 + a3 * a3;
                        if (amod < amodmin) {
                            amodmin = amod;
                            nmin = n1;
                        }
                        if (a1 <= -perr || a1 >= (1.0 + perr)) continue;
                        if (a2 <= -perr || a2 >= (1.0 + perr)) continue;
                        if (a3 <= -perr || a3 >= (1.0 + perr)) continue;
                        r.numtr[pidx] = n1;
                        r.bc[3 * pidx] = a1;
                        r.bc[3 * pidx + 1] = a2;
                        r.bc[3 * pidx + 2] = a3;
                        found = 1;
                        break;
                    }
            if (!found) {
                r.numtr[pidx] = nmin;
                int numqu = (nmin + 1) / 2;
                int io = (numqu - 1) / (nzt - 1), jo = numqu - io * (nzt - 1) - 1; // 0-based
                double d1, d2, d3;
                auto dist = [&](int jj, int ii) {
                    double dx = xx - OX(jj, ii), dy = yy - OY(jj, ii);
                    return std::sqrt(dx * dx + dy * dy);
                };
                if (nmin % 2 == 0) {
                    d1 = dist(jo, io + 1); d2 = dist(jo + 1, io); d3 = dist(jo + 1, io + 1);
                } else {
                    d1 = dist(jo, io); d2 = dist(jo + 1, io); d3 = dist(jo, io + 1);
                }
                double *b = &r.bc[3 * pidx];
                auto w2 = [&](double da, double db, double &wa, double &wb) {
                    wa = 1.0 / da / (1.0 / da + 1.0 / db);
                    wb = 1.0 / db / (1.0 / da + 1.0 / db);
                };
                if (d1 > d2) {
                    if (d2 > d3) {
                        b[0] = 0.0; w2(d2, d3, b[1], b[2]);
                    } else if (d1 > d3) {
                        b[0] = 0.0; w2(d2, d3, b[1], b[2]);
                    } else {
                        w2(d1, d2, b[0], b[1]); b[2] = 0.0;
                    }
                } else {
                    if (d3 > d1) {
                        if (d2 > d3) {
                            w2(d1, d3, b[0], b[2]); b[1] = 0.0;
                        } else {
                            w2(d1, d2, b[0], b[1]); b[2] = 0.0;
                        }
                    } else {
                        w2(d1, d3, b[0], b[2]); b[1] = 0.0;
                    }
                }
            }
        }
    return r;
}

// rem_interpolate on a plane arr (nzt x nxt, j fastest)
void rem_interpolate(const Interp &r, double *arr) {
    int nzt = r.nzt, nxt = r.nxt;
    std::vector<double> dummy(arr, arr + (size_t)nzt * nxt);
    auto Dm = [&](int j, int i) { return dummy[(size_t)i * nzt + j]; };
    for (int i = 0; i < nxt; ++i)
        for (int j = 0; j < nzt; ++j) {
            size_t pidx = (size_t)i * nzt + j;
            int n = r.numtr[pidx];
            int numq = (n + 1) / 2;
            int io = (numq - 1) / (nzt - 1), jo = numq - io * (nzt - 1) - 1;
            double f1, f2, f3;
            if (n % 2 == 0) {
                f1 = Dm(jo, io + 1); f2 = Dm(jo + 1, io); f3 = Dm(jo + 1, io + 1);
            } else {
                f1 = Dm(jo, io); f2 = Dm(jo + 1, io); f3 = Dm(jo, io + 1);
            }
            const double *b = &r.bc[3 * pidx];
            arr[pidx] = b[0] * f1 + b[1] * f2 + b[2] * f3;
        }
}

void newphase2marker(St &s, int j1, int j2, int i1, int i2, int iph) {
    gf_layout &L = *s.L;
    for (int i = i1; i <= i2; ++i)
        for (int j = j1; j <= j2; ++j) {
            long long e = s.e(j - 1, i - 1);
            for (int n = 0; n < L.nmark_elem[e]; ++n) L.mark_phase[L.mark_id_elem[e * GF_MAX_MARKERS_PER_ELEM + n] - 1] = (int8_t)iph;
            L.iphase[e] = iph;
            for (int k = 0; k < s.p->nphase; ++k) L.phase_ratio[o_pr(s.d, e, k)] = 0.0;
            L.phase_ratio[o_pr(s.d, e, iph - 1)] = 1.0;
        }
}

void init_areas(St &s) {
    int nx = s.p->nx, nz = s.p->nz;
    for (int i = 0; i < nx - 1; ++i)
        for (int j = 0; j < nz - 1; ++j) {
            double x1 = s.cord(j, i, 0), y1 = s.cord(j, i, 1), x2 = s.cord(j + 1, i, 0), y2 = s.cord(j + 1, i, 1);
            double x3 = s.cord(j, i + 1, 0), y3 = s.cord(j, i + 1, 1), x4 = s.cord(j + 1, i + 1, 0), y4 = s.cord(j + 1, i + 1, 1);
            long long e = s.e(j, i);
            double *a = s.L->area;
            a[o_ek(s.d, e, 0)] = 1.0 / (((x2 * y3 - y2 * x3) - (x1 * y3 - y1 * x3)) + (x1 * y2 - y1 * x2));
            a[o_ek(s.d, e, 1)] = 1.0 / (((x2 * y4 - y2 * x4) - (x3 * y4 - y3 * x4)) + (x3 * y2 - y3 * x2));
            a[o_ek(s.d, e, 2)] = 1.0 / (((x2 * y4 - y2 * x4) - (x1 * y4 - y1 * x4)) + (x1 * y2 - y1 * x2));
            a[o_ek(s.d, e, 3)] = 1.0 / (((x4 * y3 - y4 * x3) - (x1 * y3 - y1 * x3)) + (x1 * y4 - y1 * x4));
            for (int k = 0; k < 4; ++k)
                if (a[o_ek(s.d, e, k)] < 0) throw Stop{41};
        }
}

// remesh (remesh.f90:1-259) without the surface accumulators dhacc/extr_acc
// and the magma fields, which belong to models this path does not run
void remesh(St &s) {
    const gf_params &p = *s.p;
    gf_layout &L = *s.L;
    int nx = p.nx, nz = p.nz;
    size_t N = (size_t)s.d.N, E = (size_t)s.d.E;
    std::vector<double> cordo(L.cord, L.cord + 2 * N);
    rem_cord(s, cordo);
    // surface accumulators, length-weighted onto the new surface elements
    // (remesh.f90:20-53)
    if (L.dhacc && L.extr_acc) {
        std::vector<double> dhnew(nx - 1, 0.0), extnew(nx - 1, 0.0);
        int i = 0, ii = 0;
        double xl = s.cord(0, i, 0), xr;
        while (std::max(i, ii) < nx - 1) {
            xr = std::min(cordo[o_n2(s.d, 0, ii + 1, 0)], s.cord(0, i + 1, 0));
            if (xl < xr) {
                dhnew[i] = dhnew[i] + L.dhacc[ii] * (xr - xl);
                extnew[i] = extnew[i] + L.extr_acc[ii] * (xr - xl);
            }
            if (xr == cordo[o_n2(s.d, 0, ii + 1, 0)])
                ii = ii + 1;
            else
                i = i + 1;
            if (std::max(i, ii) < nx - 1) xl = xr;
        }
        for (int k = 0; k < nx - 1; ++k) {
            L.dhacc[k] = dhnew[k] / (s.cord(0, k + 1, 0) - s.cord(0, k, 0));
            L.extr_acc[k] = extnew[k] / (s.cord(0, k + 1, 0) - s.cord(0, k, 0));
        }
    }
    // element fields: barycentric interpolation between element centres
    int nzt = nz - 1, nxt = nx - 1;
    std::vector<double> cold(2 * E), cnew(2 * E);
    auto CO = [&](int j, int i, int k) { return cordo[o_n2(s.d, j, i, k)]; };
    for (int i = 0; i < nxt; ++i)
        for (int j = 0; j < nzt; ++j) {
            size_t q = (size_t)i * nzt + j;
            for (int k = 0; k < 2; ++k) {
                cold[2 * q + k] = 0.25 * (CO(j, i, k) + CO(j + 1, i, k) + CO(j, i + 1, k) + CO(j + 1, i + 1, k));
                cnew[2 * q + k] = 0.25 * (s.cord(j, i, k) + s.cord(j + 1, i, k) + s.cord(j, i + 1, k) + s.cord(j + 1, i + 1, k));
            }
        }
    Interp r = rem_barcord(cold, cnew, nzt, nxt);
    for (int k = 0; k < 4; ++k)
        for (int c = 0; c < 4; ++c) rem_interpolate(r, L.stress0 + (size_t)(c + 4 * k) * E);
    for (int k = 0; k < 3; ++k) rem_interpolate(r, L.strain + (size_t)k * E);
    rem_interpolate(r, L.aps);
    for (size_t e = 0; e < E; ++e)
        if (L.aps[e] < 0.0) L.aps[e] = 0.0;
    if (p.itype_melting == 1) // remesh.f90:106-115
        for (double *f : {L.fmagma, L.fmagma2, L.dike_backlog, L.dike_marker_vol, L.mor_marker_vol}) rem_interpolate(r, f);
    // material entering through the side walls (remesh.f90:129-194)
    const int idist = 2;
    int ju = 1, jl = 1;
    if (p.incoming_left == 1) {
        for (int j = 0; j < nz - 1; ++j)
            for (int i = 0; i <= idist; ++i) L.aps[s.e(j, i)] = 0.0;
        int n = 0, i = 1;
        for (int m = 0; m < p.nph_layer[n] - 1; ++m) {
            ju = jl;
            for (int j = jl; j <= nz - 1; ++j)
                if ((s.cord(0, i - 1, 1) - 0.5 * (s.cord(j - 1, i - 1, 1) + s.cord(j, i - 1, 1))) > p.hc[n][m] * 1e3) {
                    jl = j;
                    break;
                }
            newphase2marker(s, ju, jl - 1, i, i + idist, p.iph_col[n][m]);
        }
        newphase2marker(s, jl, nz - 1, i, i + idist, p.iph_col[n][p.nph_layer[n] - 1]);
    }
    if (p.incoming_right == 1) {
        for (int j = 0; j < nz - 1; ++j)
            for (int i = nx - 2 - idist; i <= nx - 2; ++i) L.aps[s.e(j, i)] = 0.0;
        int n = p.nzone_age - 1, i = nx - 1;
        for (int m = 0; m < p.nph_layer[n] - 1; ++m) {
            ju = jl;
            for (int j = jl; j <= nz - 1; ++j)
                if ((s.cord(0, i, 1) - 0.5 * (s.cord(j - 1, i, 1) + s.cord(j, i, 1))) > p.hc[n][m] * 1e3) {
                    jl = j;
                    break;
                }
            newphase2marker(s, ju, jl - 1, i - idist, i, p.iph_col[n][m]);
        }
        newphase2marker(s, jl, nz - 1, i - idist, i, p.iph_col[n][p.nph_layer[n] - 1]);
    }
    rem_interpolate(r, L.source);
    // node fields: barycentric interpolation on the old node mesh
    std::vector<double> coldn(2 * N), cnewn(2 * N);
    for (size_t q = 0; q < N; ++q)
        for (int k = 0; k < 2; ++k) {
            coldn[2 * q + k] = cordo[k * N + q];
            cnewn[2 * q + k] = L.cord[k * N + q];
        }
    std::memcpy(L.temp0, L.temp, sizeof(double) * N);
    Interp rn = rem_barcord(coldn, cnewn, nz, nx);
    for (int k = 0; k < 2; ++k) rem_interpolate(rn, L.vel + (size_t)k * N);
    rem_interpolate(rn, L.temp);
    if (L.xoriginal) rem_interpolate(rn, L.xoriginal); // remesh.f90:242-243
    if (L.zoriginal) rem_interpolate(rn, L.zoriginal);
    // side-wall geotherms for incoming material (sidewalltemp, init_temp.f90:313-353)
    if (p.incoming_left == 1) {
        for (int i = 0; i <= idist; ++i) geotherm_column(s, 0, i, p.age_1[0], p.tp1[0], p.tp2[0]);
        for (int i = 0; i < idist; ++i)
            for (int j = 0; j < nz - 1; ++j) L.source[s.e(j, i)] = L.source[s.e(j, idist)];
    }
    if (p.incoming_right == 1) {
        int n = p.nzone_age - 1;
        for (int i = nx - 1 - idist; i <= nx - 1; ++i) geotherm_column(s, n, i, p.age_1[n], p.tp1[n], p.tp2[n]);
        for (int i = nx - 1 - idist; i < nx - 1; ++i)
            for (int j = 0; j < nz - 1; ++j) L.source[s.e(j, i)] = L.source[s.e(j, nx - 2 - idist)];
    }
    if (p.ivis_present == 1) init_visc(s);
    init_areas(s);
    rmasses(s);
    dt_mass(s);
}

void remesh_event(St &s) {
    bar2euler(s);
    remesh(s);
    lpeuler2bar(s);
    marker2elem(s);
    if (s.L->dhacc_correction)
        for (int i = 0; i < s.p->nx; ++i) s.L->dhacc_correction[i] = 0.0;
}

// --------------------------------------------------------------------------
// Start-up: read_params (src/read_params.f90:3-373) and the setflac chain
// (src/setflac.f90:4-89: init_cord, init_phase, init_marker,
// check_visc_rheol, init_areas, init_temp, init_stress, init_bc).  The
// oracle builds its own initial state from the .inp file with these, so
// that nothing of the product's host code enters a comparison.

// Fortran list-directed input over the lines of an .inp file.  A READ
// starts at the current record and takes values from as many records as it
// needs; what is left of its last record is dropped.  Values are separated
// by commas, blanks or the end of a record; two commas in a row give a null
// value (the item keeps its value), r*v repeats v r times, r* gives r nulls,
// a slash ends the READ.
struct ParseErr {
    int line;
};

class ListInput {
  public:
    explicit ListInput(std::vector<std::string> lines) : rec_(lines) {}
    // AdvanceToNextInputLine (read_params.f90:351-373): skip records whose
    // first character is ';'
    void advance() {
        while (cur_ < rec_.size() && !rec_[cur_].empty() && rec_[cur_][0] == ';') ++cur_;
        if (cur_ >= rec_.size()) throw ParseErr{(int)cur_ + 1};
    }
    void begin() {
        q_.clear();
        slash_ = false;
        used_ = false;
    }
    // end of a READ statement: continue after its last record
    void end() {
        if (used_ || q_.empty()) ++cur_;
        q_.clear();
    }
    // an empty READ: skips one record
    void skip() {
        if (cur_ >= rec_.size()) throw ParseErr{(int)cur_ + 1};
        ++cur_;
    }
    bool next(std::string &v) { // false: null value (item unchanged)
        if (slash_) return false;
        while (q_.empty()) {
            if (used_) ++cur_;
            if (cur_ >= rec_.size()) throw ParseErr{(int)cur_ + 1};
            split(rec_[cur_]);
            used_ = true;
        }
        Tok t = q_.front();
        q_.pop_front();
        if (t.kind == 2) {
            slash_ = true;
            q_.clear();
            return false;
        }
        if (t.kind == 1) return false;
        v = t.s;
        return true;
    }
    void i(int &x) {
        std::string v;
        if (!next(v)) return;
        char *e = nullptr;
        long r = std::strtol(v.c_str(), &e, 10);
        if (e == v.c_str() || *e) throw ParseErr{(int)cur_ + 1};
        x = (int)r;
    }
    void d(double &x) {
        std::string v;
        if (!next(v)) return;
        for (char &c : v)
            if (c == 'd' || c == 'D') c = 'e';
        char *e = nullptr;
        double r = std::strtod(v.c_str(), &e);
        if (e == v.c_str() || *e) throw ParseErr{(int)cur_ + 1};
        x = r;
    }
    void str(char *dst, size_t n) {
        std::string v;
        if (!next(v)) return;
        std::snprintf(dst, n, "%s", v.c_str());
    }
    int line() const { return (int)cur_ + 1; }

  private:
    struct Tok {
        int kind; // 0 value, 1 null, 2 slash
        std::string s;
    };
    void split(const std::string &r) {
        size_t k = 0, n = r.size();
        bool want = true; // a comma now gives a null value
        while (k < n) {
            char c = r[k];
            if (c == ' ' || c == '\t' || c == '\r') {
                ++k;
                continue;
            }
            if (c == ',') {
                if (want) q_.push_back({1, ""});
                want = true;
                ++k;
                continue;
            }
            if (c == '/') {
                q_.push_back({2, ""});
                return;
            }
            std::string t;
            if (c == '\'' || c == '"') {
                char qc = c;
                ++k;
                while (k < n && r[k] != qc) t += r[k++];
                ++k;
                q_.push_back({0, t});
                want = false;
                continue;
            }
            while (k < n && r[k] != ' ' && r[k] != '\t' && r[k] != ',' && r[k] != '/' && r[k] != '\r') t += r[k++];
            size_t star = t.find('*');
            if (star != std::string::npos && star > 0 &&
                t.find_first_not_of("0123456789") == star) { // r*v or r*
                int reps = std::atoi(t.substr(0, star).c_str());
                std::string v = t.substr(star + 1);
                for (int m = 0; m < reps; ++m) q_.push_back(v.empty() ? Tok{1, ""} : Tok{0, v});
            } else {
                q_.push_back({0, t});
            }
            want = false;
        }
    }
    std::vector<std::string> rec_;
    size_t cur_ = 0;
    std::deque<Tok> q_;
    bool slash_ = false, used_ = false;
};

const double O_SEC_YEAR = 3.1558e7; // src/params.f90 sec_year

// read_params (src/read_params.f90:3-348), in its order
int read_params(const char *path, gf_params *p) {
    std::FILE *f = std::fopen(path, "r");
    if (!f) return GF_ERR_IO;
    std::vector<std::string> lines;
    std::string cur;
    for (int ch; (ch = std::fgetc(f)) != EOF;) {
        if (ch == '\n') {
            lines.push_back(cur);
            cur.clear();
        } else {
            cur += (char)ch;
        }
    }
    if (!cur.empty()) lines.push_back(cur);
    std::fclose(f);
    // options with no .inp counterpart survive the read
    int mps = p->markers_per_side, ecl = p->eclogite_rule, tsw = p->therm_sweeps;
    std::memset(p, 0, sizeof *p);
    p->markers_per_side = mps;
    p->eclogite_rule = ecl;
    p->therm_sweeps = tsw;
    ListInput r(lines);
    auto rd = [&](auto &&body) {
        r.advance();
        r.begin();
        body();
        r.end();
    };
    try {
        rd([&] { r.i(p->nx); r.i(p->nz); });
        p->nx += 1;
        p->nz += 1;
        rd([&] { r.d(p->x0); r.d(p->z0); });
        rd([&] { r.d(p->rxbo); r.d(p->rzbo); });
        rd([&] { r.i(p->ircoord); r.str(p->coordfile, sizeof p->coordfile); });
        if (p->ircoord > 0) {
            rd([&] { r.i(p->nzonx); });
            if (p->nzonx != 0) return GF_ERR_PARSE;
            rd([&] { r.i(p->nzony); });
            if (p->nzony != 0) return GF_ERR_PARSE;
        } else {
            rd([&] { r.i(p->nzonx); });
            if (p->nzonx == 0) {
                p->nzonx = 1;
                p->nelz_x[0] = p->nx - 1;
                p->sizez_x[0] = 1.0;
            } else {
                if (p->nzonx < 0 || p->nzonx > GF_MAXZONE) return GF_ERR_PARSE;
                for (int k = 0; k < p->nzonx; ++k) rd([&] { r.i(p->nelz_x[k]); r.d(p->sizez_x[k]); });
            }
            rd([&] { r.i(p->nzony); });
            if (p->nzony == 0) {
                p->nzony = 1;
                p->nelz_y[0] = p->nz - 1;
                p->sizez_y[0] = 1.0;
            } else {
                if (p->nzony < 0 || p->nzony > GF_MAXZONE) return GF_ERR_PARSE;
                for (int k = 0; k < p->nzony; ++k) {
                    p->sizez_y[k] = 1.0;
                    rd([&] { r.i(p->nelz_y[k]); r.d(p->sizez_y[k]); });
                }
            }
        }
        // mechanical conditions
        rd([&] { r.i(p->nystressbc); r.i(p->nydrsides); });
        rd([&] { r.i(p->nofbc); });
        if (p->nofbc < 0 || p->nofbc > GF_MAXBC) return GF_ERR_PARSE;
        r.advance();
        for (int k = 0; k < p->nofbc; ++k) { // one READ per condition, no comment lines between
            r.begin();
            r.i(p->nofside[k]); r.i(p->nbc1[k]); r.i(p->nbc2[k]); r.i(p->nbc[k]);
            r.d(p->bca[k]); r.d(p->bcb[k]); r.d(p->bcc[k]); r.d(p->bcd[k]); r.d(p->bce[k]);
            r.d(p->bcf[k]); r.d(p->bcg[k]); r.d(p->bch[k]); r.d(p->bci[k]);
            r.end();
        }
        r.advance();
        rd([&] { r.i(p->nyhydro); r.d(p->pisos); r.i(p->iphsub); r.d(p->drosub); r.d(p->damp_vis); });
        rd([&] { r.d(p->g); });
        // thermal conditions
        rd([&] { r.i(p->i_prestress); });
        rd([&] { r.d(p->extra_pres); });
        rd([&] { r.i(p->itherm); });
        rd([&] { r.i(p->istress_therm); });
        rd([&] { r.i(p->ishearh); });
        rd([&] { r.d(p->t_top); });
        rd([&] { r.d(p->t_bot); });
        rd([&] { r.d(p->hs); r.d(p->hr); });
        rd([&] { r.i(p->itemp_bc); r.d(p->bot_bc); });
        if (p->itemp_bc == 2) p->bot_bc = p->bot_bc / 1000;
        rd([&] { r.i(p->irtemp); });
        r.advance();
        if (p->irtemp > 0) {
            r.begin();
            r.str(p->tempfile, sizeof p->tempfile);
            r.end();
        } else {
            r.skip();
        }
        rd([&] { r.i(p->nzone_age); });
        if (p->nzone_age < 0 || p->nzone_age > GF_MAXZONE_AGE) return GF_ERR_PARSE;
        r.advance();
        for (int n = 0; n < p->nzone_age; ++n) {
            r.begin();
            r.i(p->ictherm[n]); r.d(p->age_1[n]); r.d(p->tp1[n]); r.d(p->tp2[n]); r.i(p->ixtb1[n]); r.i(p->ixtb2[n]);
            r.end();
            r.advance();
            r.begin();
            r.i(p->nph_layer[n]);
            if (p->nph_layer[n] < 1 || p->nph_layer[n] > GF_MAXZONE_LAYER) return GF_ERR_PARSE;
            for (int m = 0; m < p->nph_layer[n] - 1; ++m) r.d(p->hc[n][m]);
            r.end();
            r.begin();
            for (int m = 0; m < p->nph_layer[n]; ++m) r.i(p->iph_col[n][m]);
            r.end();
        }
        // smooth transitions between age zones (read_params.f90:168-186)
        for (int n = 0; n < p->nzone_age - 1; ++n) {
            p->iph_col_trans[n] = 0;
            if (p->ixtb2[n] == -1) {
                p->iph_col_trans[n] = 1;
                p->ixtb2[n] = p->ixtb2[n + 1];
                p->ixtb1[n + 1] = p->ixtb1[n];
            }
        }
        // rheology
        rd([&] { r.i(p->nphase); });
        if (p->nphase < 1 || p->nphase > GF_MAXPH) return GF_ERR_PARSE;
        for (int k = 0; k < p->nphase; ++k)
            rd([&] {
                r.i(p->irheol[k]); r.d(p->visc[k]); r.d(p->den[k]); r.d(p->alfa[k]); r.d(p->beta[k]);
                r.d(p->pln[k]); r.d(p->acoef[k]); r.d(p->eactiv[k]); r.d(p->vactiv[k]); r.d(p->rl[k]);
                r.d(p->rm[k]); r.d(p->plstrain1[k]); r.d(p->plstrain2[k]); r.d(p->fric1[k]); r.d(p->fric2[k]);
                r.d(p->cohesion1[k]); r.d(p->cohesion2[k]); r.d(p->dilat1[k]); r.d(p->dilat2[k]);
                r.d(p->conduct[k]); r.d(p->cp[k]); r.d(p->ts[k]); r.d(p->tl[k]); r.d(p->tk[k]);
                r.d(p->erodibility[k]);
            });
        rd([&] { r.i(p->irphase); });
        r.advance();
        if (p->irphase > 0) {
            r.begin();
            r.str(p->phasefile, sizeof p->phasefile);
            r.end();
        } else {
            r.skip();
        }
        rd([&] { r.i(p->inhom); });
        if (p->inhom < 0 || p->inhom > GF_MAXINH) return GF_ERR_PARSE; // stop 26
        for (int k = 0; k < p->inhom; ++k)
            rd([&] {
                r.i(p->ix1[k]); r.i(p->ix2[k]); r.i(p->iy1[k]); r.i(p->iy2[k]); r.i(p->inphase[k]);
                r.i(p->igeom[k]); r.d(p->xinitaps[k]);
            });
        rd([&] { r.d(p->ten_off); });
        rd([&] { r.d(p->tau_heal); });
        rd([&] { r.d(p->v_min); r.d(p->v_max); r.i(p->ivis_shape); r.d(p->efoldc); });
        rd([&] {
            r.i(p->itype_melting); r.i(p->nelem_serp); r.i(p->nelem_dike); r.d(p->prod_magma); r.d(p->prod_magma2);
            r.d(p->rho_magma);
        });
        rd([&] { r.d(p->angle_mzone); r.d(p->fmagma_max); r.d(p->ratio_mantle_mzone); r.d(p->ratio_crust_mzone); });
        rd([&] { r.d(p->latent_heat_magma); r.d(p->lambda_freeze); r.d(p->lambda_freeze_tdep); });
        rd([&] { r.d(p->weaken_ratio_plastic); r.d(p->weaken_ratio_viscous); });
        p->weaken_ratio_viscous = std::log(p->weaken_ratio_viscous);
        // remeshing
        rd([&] { r.i(p->ny_rem); r.i(p->mode_rem); r.i(p->ntest_rem); r.d(p->angle_rem); });
        if (p->mode_rem != 1 && p->mode_rem != 11 && p->mode_rem != 3 && p->mode_rem != 4) return GF_ERR_PARSE;
        rd([&] { r.d(p->dx_rem); });
        rd([&] { r.d(p->topo_kappa); r.d(p->fac_kappa); });
        // process control
        rd([&] { r.i(p->idt_scale); });
        rd([&] { r.d(p->dt_scale); r.d(p->strain_inert); });
        rd([&] { r.i(p->i_rey); r.d(p->xReyn); });
        rd([&] { r.i(p->ifreq_rmasses); });
        rd([&] { r.i(p->ifreq_imasses); });
        rd([&] { r.i(p->ifreq_visc); });
        rd([&] { r.i(p->ifreq_avgsr); });
        if (p->ifreq_rmasses <= 0 || p->ifreq_imasses <= 0 || p->ifreq_visc <= 0 || p->ifreq_avgsr <= 0)
            return GF_ERR_PARSE;
        if (p->ntest_rem % p->ifreq_rmasses + p->ntest_rem % p->ifreq_imasses + p->ntest_rem % p->ifreq_visc +
                p->ntest_rem % p->ifreq_avgsr != 0)
            return GF_ERR_PARSE;
        rd([&] { r.d(p->frac); r.d(p->fracm); });
        rd([&] { r.i(p->movegrid); r.i(p->ndim); });
        rd([&] { r.d(p->demf); r.i(p->mix_strain); r.i(p->mix_stress); });
        // output
        rd([&] { r.d(p->time_max); });
        p->time_max = p->time_max * 1000 * O_SEC_YEAR;
        rd([&] { r.d(p->dtout_screen); });
        p->dtout_screen = p->dtout_screen * 1000 * O_SEC_YEAR;
        rd([&] { r.d(p->dtout_file); });
        p->dtout_file = p->dtout_file * 1000 * O_SEC_YEAR;
        rd([&] {
            for (int k = 0; k < 19; ++k) r.i(p->io_flags[k]);
        });
        rd([&] { r.i(p->lastout); });
        rd([&] { r.d(p->dtsave_file); });
        p->dtsave_file = p->dtsave_file * 1000 * O_SEC_YEAR;
        rd([&] { r.i(p->lastsave); });
    } catch (const ParseErr &) {
        return GF_ERR_PARSE;
    }
    if (p->nx < 2 || p->nz < 2) return GF_ERR_PARSE;
    return GF_OK;
}

// init_cord (src/init_cord.f90:5-93) for a mesh from the zone lists
void init_cord(St &s) {
    gf_params &p = *s.p;
    int nx = p.nx, nz = p.nz;
    if (p.ircoord > 0) throw Stop{GF_ERR_UNSUPPORTED};
    // test_grid (init_cord.f90:97-137)
    int sx = 0, sz = 0;
    for (int k = 0; k < p.nzonx; ++k) sx += p.nelz_x[k];
    for (int k = 0; k < p.nzony; ++k) sz += p.nelz_y[k];
    if (p.nzonx != 0 && p.nzonx % 2 == 0) throw Stop{16};
    if (sx != nx - 1) throw Stop{17};
    if (p.nzony != 0 && p.nzony % 2 == 0) throw Stop{18};
    if (sz != nz - 1) throw Stop{19};
    std::vector<double> rm(nx + nz);
    mesh1(p.x0, p.x0 + p.rxbo, rm.data(), nx, p.nzonx, p.nelz_x, p.sizez_x);
    for (int i = 0; i < nx; ++i)
        for (int j = 0; j < nz; ++j) s.cordr(j, i, 0) = rm[i];
    mesh1(p.z0, p.z0 + p.rzbo, rm.data(), nz, p.nzony, p.nelz_y, p.sizez_y);
    for (int j = 0; j < nz; ++j)
        for (int i = 0; i < nx; ++i) s.cordr(j, i, 1) = rm[j];
    // surface relief of igeom 20 (table) and 21 (trapezoid), 1-based columns
    for (int n = 0; n < p.inhom; ++n) {
        double amp = p.xinitaps[n];
        if (p.igeom[n] == 20) {
            for (int i = p.ix1[n]; i <= p.ix2[n]; ++i) s.cordr(0, i - 1, 1) += amp;
        } else if (p.igeom[n] == 21) {
            for (int i = p.ix1[n]; i <= p.ix2[n] - 1; ++i)
                s.cordr(0, i - 1, 1) += amp * (double)(float)(i - p.ix1[n]) / (p.ix2[n] - p.ix1[n]);
            for (int i = p.ix2[n]; i <= p.iy1[n]; ++i) s.cordr(0, i - 1, 1) += amp;
            for (int i = p.iy1[n] + 1; i <= p.iy2[n]; ++i)
                s.cordr(0, i - 1, 1) += amp * (double)(float)(p.iy2[n] - i) / (p.iy2[n] - p.iy1[n]);
        }
    }
    // every column re-spaced from its top to its bottom
    for (int i = 0; i < nx; ++i) {
        mesh1(s.cord(0, i, 1), s.cord(nz - 1, i, 1), rm.data(), nz, p.nzony, p.nelz_y, p.sizez_y);
        for (int j = 0; j < nz; ++j) s.cordr(j, i, 1) = rm[j];
    }
    double dxmin = 1e300, dzmin = 1e300;
    for (int i = 1; i < nx; ++i) dxmin = std::min(dxmin, s.cord(0, i, 0) - s.cord(0, i - 1, 0));
    for (int j = 0; j < nz - 1; ++j) dzmin = std::min(dzmin, s.cord(j, 0, 1) - s.cord(j + 1, 0, 1));
    p.dxmin = dxmin;
    p.dzmin = dzmin;
    gf_layout &L = *s.L;
    for (int i = 0; i < nx; ++i) {
        if (L.dhacc_correction) L.dhacc_correction[i] = 0.0;
        if (L.dhacc) L.dhacc[i] = 0.0;
        if (L.extr_acc) L.extr_acc[i] = 0.0;
    }
}

// real(4) arithmetic of the reference's inclined zones: nint / floor /
// ceiling of float(iy2-iy1)/float(ix2-ix1)*(j-ix1)
inline float o_slope(int ix1, int ix2, int iy1, int iy2, int j) {
    float a = (float)(iy2 - iy1) / (float)(ix2 - ix1);
    return a * (float)(j - ix1);
}
inline int o_nint(float v) { return (int)(v < 0 ? -std::floor(-v + 0.5f) : std::floor(v + 0.5f)); }

// init_phase (src/init_phase.f90:5-50): inclusions on the element phases
// and plastic strain (1-based element ranges)
void init_phase(St &s) {
    gf_params &p = *s.p;
    gf_layout &L = *s.L;
    if (p.irphase > 0) throw Stop{GF_ERR_UNSUPPORTED};
    auto E = [&](int j, int i) { return s.e(j - 1, i - 1); };
    for (int n = 0; n < p.inhom; ++n) {
        if (p.igeom[n] == 0)
            for (int i = p.ix1[n]; i <= p.ix2[n]; ++i)
                for (int j = p.iy1[n]; j <= p.iy2[n]; ++j) {
                    if (p.inphase[n] > 0) L.iphase[E(j, i)] = p.inphase[n];
                    L.aps[E(j, i)] = p.xinitaps[n];
                }
        if (p.igeom[n] == 3)
            for (int i = p.ix1[n]; i <= p.ix2[n]; ++i) {
                int j = o_nint(o_slope(p.ix1[n], p.ix2[n], p.iy1[n], p.iy2[n], i)) + p.iy1[n];
                if (p.inphase[n] > 0) L.iphase[E(j, i)] = p.inphase[n];
            }
        if (p.igeom[n] == 4)
            for (int i = p.ix1[n]; i <= p.ix2[n]; ++i) {
                float t = o_slope(p.ix1[n], p.ix2[n], p.iy1[n], p.iy2[n], i);
                int j1 = (int)std::floor(t) + p.iy1[n], j2 = (int)std::ceil(t) + p.iy1[n];
                for (int j = j1; j <= j2; ++j) {
                    L.aps[E(j, i)] = p.xinitaps[n];
                    if (p.inphase[n] > 0) L.iphase[E(j, i)] = p.inphase[n];
                }
            }
    }
}

// init_marker (src/init_marker.f90:1-164): ms x ms points per element on
// the reference's construction (3 x 3: the 1/6, 1/2, 5/6 weights along both
// edges), each moved by up to half a point spacing with two draws of the
// serial LCG chain, its phase from the age zone's layers at its depth; then
// the inclusions and marker2elem.  ms other than 3 has no reference
// counterpart; its points sit at (2m+1)/(2 ms) and move by up to half of
// their spacing dx/ms.
void init_marker(St &s) {
    gf_params &p = *s.p;
    gf_layout &L = *s.L;
    int nx = p.nx, nz = p.nz;
    const int ms = p.markers_per_side > 0 ? p.markers_per_side : 3;
    std::memset(L.mark_id_elem, 0, sizeof(int) * (size_t)s.d.E * GF_MAX_MARKERS_PER_ELEM);
    std::memset(L.nmark_elem, 0, sizeof(int) * (size_t)s.d.E);
    s.c->nmarkers = 0;
    std::vector<double> wa(ms), wb(ms); // weights of an edge's first and second node
    if (ms == 3) {
        const double half = 0.5, onesixth = 0.1666666666666666666666, fivesixth = 0.8333333333333333333333;
        wa[0] = fivesixth, wb[0] = onesixth;
        wa[1] = half, wb[1] = half;
        wa[2] = onesixth, wb[2] = fivesixth;
    } else {
        for (int m = 0; m < ms; ++m) {
            wb[m] = (2.0 * m + 1.0) / (2.0 * ms);
            wa[m] = 1.0 - wb[m];
        }
    }
    std::vector<double> ax(ms), az(ms), bx(ms), bz(ms), ptx(ms * ms), ptz(ms * ms);
    int iseed = 0;
    for (int i = 1; i <= nx - 1; ++i)
        for (int j = 1; j <= nz - 1; ++j) {
            // a: points along the element's left edge, b: its right edge
            for (int m = 0; m < ms; ++m) {
                ax[m] = s.cord(j - 1, i - 1, 0) * wa[m] + s.cord(j, i - 1, 0) * wb[m];
                az[m] = s.cord(j - 1, i - 1, 1) * wa[m] + s.cord(j, i - 1, 1) * wb[m];
                bx[m] = s.cord(j - 1, i, 0) * wa[m] + s.cord(j, i, 0) * wb[m];
                bz[m] = s.cord(j - 1, i, 1) * wa[m] + s.cord(j, i, 1) * wb[m];
            }
            for (int m = 0; m < ms; ++m)
                for (int q = 0; q < ms; ++q) {
                    ptx[m * ms + q] = ax[m] * wa[q] + bx[m] * wb[q];
                    ptz[m * ms + q] = az[m] * wa[q] + bz[m] * wb[q];
                }
            double dx = s.cord(j - 1, i, 0) - s.cord(j - 1, i - 1, 0);
            double dy = s.cord(j, i - 1, 1) - s.cord(j - 1, i - 1, 1);
            iseed = iseed + i + j;
            int l = 1, tries = 0;
            while (l <= ms * ms) {
                int kph = L.iphase[s.e(j - 1, i - 1)];
                double rx = o_myrandom(iseed);
                double ry = o_myrandom(iseed);
                rx = 0.5 - rx;
                ry = 0.5 - ry;
                double ddx = dx * rx / ms;
                double ddy = dy * ry / ms;
                double xx = ptx[l - 1] + ddx;
                double yy = ptz[l - 1] + ddy;
                for (int n = 1; n <= p.nzone_age; ++n) {
                    if (i < p.ixtb1[n - 1] || i > p.ixtb2[n - 1]) continue;
                    if (n != 1 && p.iph_col_trans[n - 2] == 1) continue;
                    int nl = p.nph_layer[n - 1];
                    double hhc[GF_MAXZONE_LAYER];
                    for (int m = 1; m <= nl - 1; ++m) hhc[m - 1] = p.hc[n - 1][m - 1];
                    if (p.iph_col_trans[n - 1] == 1) {
                        int i1 = p.ixtb1[n - 1], i2 = p.ixtb2[n - 1];
                        double rr = (s.cord(0, i - 1, 0) - s.cord(0, i1 - 1, 0)) / (s.cord(0, i2 - 1, 0) - s.cord(0, i1 - 1, 0));
                        for (int m = 1; m <= nl - 1; ++m)
                            hhc[m - 1] = p.hc[n - 1][m - 1] + (p.hc[n][m - 1] - p.hc[n - 1][m - 1]) * rr;
                    }
                    double yyy = yy * (-1e-3);
                    int m = 1;
                    while (m <= nl - 1 && !(yyy < hhc[m - 1])) ++m; // the Fortran DO leaves m = nl
                    kph = p.iph_col[n - 1][m - 1];
                }
                int inc = add_marker(s, xx, yy, kph, 0.0, j - 1, i - 1);
                if (++tries > 1000 * ms * ms) throw Stop{133};
                if (inc <= 0) continue;
                l = l + 1;
            }
        }
    for (int n = 0; n < p.inhom; ++n) {
        if (p.inphase[n] < 0) continue;
        if (p.igeom[n] == 0) newphase2marker(s, p.iy1[n], p.iy2[n], p.ix1[n], p.ix2[n], p.inphase[n]);
        if (p.igeom[n] == 3)
            for (int i = p.ix1[n]; i <= p.ix2[n]; ++i) {
                int k = o_nint(o_slope(p.ix1[n], p.ix2[n], p.iy1[n], p.iy2[n], i)) + p.iy1[n];
                newphase2marker(s, k, k, i, i, p.inphase[n]);
            }
        if (p.igeom[n] == 4)
            for (int i = p.ix1[n]; i <= p.ix2[n]; ++i) {
                float t = o_slope(p.ix1[n], p.ix2[n], p.iy1[n], p.iy2[n], i);
                newphase2marker(s, (int)std::floor(t) + p.iy1[n], (int)std::ceil(t) + p.iy1[n], i, i, p.inphase[n]);
            }
    }
    marker2elem(s);
}

// init_temp (src/init_temp.f90:3-124): the age zones' geotherms, radiogenic
// sources by depth, Gaussian perturbations (igeom 11, 13, 14)
void init_temp(St &s) {
    gf_params &p = *s.p;
    gf_layout &L = *s.L;
    int nx = p.nx, nz = p.nz;
    if (p.irtemp > 0) throw Stop{GF_ERR_UNSUPPORTED};
    for (int n = 1; n <= p.nzone_age; ++n) {
        if (n != 1 && p.iph_col_trans[n - 2] == 1) continue;
        for (int i = p.ixtb1[n - 1]; i <= p.ixtb2[n - 1]; ++i) {
            double age = p.age_1[n - 1], t1 = p.tp1[n - 1], t2 = p.tp2[n - 1];
            if (p.iph_col_trans[n - 1] == 1) {
                int i1 = p.ixtb1[n - 1], i2 = p.ixtb2[n - 1];
                double ratio = (s.cord(0, i - 1, 0) - s.cord(0, i1 - 1, 0)) / (s.cord(0, i2 - 1, 0) - s.cord(0, i1 - 1, 0));
                age = p.age_1[n - 1] + (p.age_1[n] - p.age_1[n - 1]) * ratio;
                t1 = p.tp1[n - 1] + (p.tp1[n] - p.tp1[n - 1]) * ratio;
                t2 = p.tp2[n - 1] + (p.tp2[n] - p.tp2[n - 1]) * ratio;
            }
            geotherm_column(s, n - 1, i - 1, age, t1, t2);
        }
    }
    for (int j = 0; j < nz - 1; ++j) {
        double y = -(s.cord(j + 1, 0, 1) + s.cord(j, 0, 1)) / 2 / 1000;
        double v = p.hs * std::exp(-y / p.hr);
        for (int i = 0; i < nx - 1; ++i) L.source[s.e(j, i)] = v;
    }
    auto T = [&](int j, int i) -> double & { return L.temp[o_node(s.d, j - 1, i - 1)]; };
    for (int n = 0; n < p.inhom; ++n) {
        int g = p.igeom[n];
        if (g != 11 && g != 13 && g != 14) continue;
        int ixc = (p.ix1[n] + p.ix2[n]) / 2, iwidth = p.ix2[n] - p.ix1[n];
        double amp = p.xinitaps[n];
        auto pert_of = [&](int i) {
            double t = (double)(float)(i - ixc) / (0.25 * (double)(float)iwidth);
            return amp * std::exp(-(t * t));
        };
        if (g == 11)
            for (int i = p.ix1[n]; i <= p.ix2[n]; ++i) {
                double pert = pert_of(i);
                for (int k = p.iy1[n]; k <= p.iy2[n]; ++k) {
                    double pert2 = 1.0 * (k - p.iy1[n]) / (p.iy2[n] - p.iy1[n]);
                    T(k, i) = std::min(p.t_bot, T(k, i) + pert * pert2);
                }
            }
        else
            for (int k = p.iy1[n]; k <= p.iy2[n]; ++k) {
                int kk = k - p.iy1[n];
                for (int i = p.ix1[n]; i <= p.ix2[n]; ++i) {
                    int ic = g == 13 ? i + kk : i - kk;
                    T(k, ic) = std::max(p.t_top, std::min(p.t_bot, T(k, ic) + pert_of(i)));
                }
            }
    }
}

// init_stress (src/init_stress.f90:5-60): hydrostatic prestress per column
// (oceanic columns under 8 km of water), pisos for the Winkler foundation
void init_stress(St &s) {
    gf_params &p = *s.p;
    gf_layout &L = *s.L;
    int nx = p.nx, nz = p.nz;
    p.pisos = 0.0;
    for (int i = 1; i <= nx - 1; ++i) {
        int top = L.iphase[s.e(0, i - 1)];
        double rogh = (top == 3 || top == 7) ? -1030.0 * p.g * 8.0e3 : 0.0; // kocean1, kocean2
        for (int j = 1; j <= nz - 1; ++j) {
            long long e = s.e(j - 1, i - 1);
            int iph = L.iphase[e] - 1;
            double tmpr = 0.25 * (s.temp(j - 1, i - 1) + s.temp(j, i - 1) + s.temp(j - 1, i) + s.temp(j, i));
            double densT = p.den[iph] * (1 - p.alfa[iph] * tmpr);
            double dh1 = s.cord(j - 1, i - 1, 1) - s.cord(j, i - 1, 1);
            double dh2 = s.cord(j - 1, i, 1) - s.cord(j, i, 1);
            double dh = 0.5 * (dh1 + dh2);
            double dPT = densT * p.g * dh;
            double dP = dPT * (1 - p.beta[iph] * rogh) / (1 + p.beta[iph] / 2 * dPT);
            double press = rogh + 0.5 * dP;
            for (int k = 0; k < 4; ++k) {
                s.st(e, 0, k) = -press;
                s.st(e, 1, k) = -press;
                s.st(e, 2, k) = 0.0;
                s.st(e, 3, k) = -press;
            }
            rogh = rogh + dP;
        }
        if (i == nx - 1 && p.nyhydro == 2) p.pisos = rogh + p.extra_pres;
    }
}

// velbc (src/init_bc.f90:284-339) at node (j,i) (0-based) for condition n
void velbc(St &s, int n, int j, int i, double x) {
    gf_params &p = *s.p;
    gf_layout &L = *s.L;
    const double pi2 = 2.0 * 3.14159;
    double fun = p.bca[n] + p.bcb[n] * x + p.bcc[n] * x * x +
                 (p.bcd[n] * std::cos(pi2 * p.bce[n] * x) + p.bcf[n] * std::sin(pi2 * p.bcg[n] * x)) *
                     std::exp(-((x - p.bci[n]) * p.bch[n]) * ((x - p.bci[n]) * p.bch[n]));
    long long kx = o_n2(s.d, j, i, 0), kz = o_n2(s.d, j, i, 1);
    if (p.nbc[n] == 10) {
        L.ncod[kx] = 1;
        if (std::fabs(L.bc[kx]) > 0.0) fun = L.bc[kx];
        L.bc[kx] = fun;
    }
    if (p.nbc[n] == 1 || p.nbc[n] == 200) {
        L.ncod[kz] = 1;
        L.bc[kz] = p.nbc[n] == 200 ? 0.0 : fun;
    }
}

// init_bc (src/init_bc.f90:4-221) for velocity conditions on the four
// sides (stress conditions and the mid-domain side 5 are not restated) and
// vbcal (:385-409)
void init_bc(St &s) {
    gf_params &p = *s.p;
    gf_layout &L = *s.L;
    int nx = p.nx, nz = p.nz;
    std::memset(L.bc, 0, sizeof(double) * 2 * (size_t)s.d.N);
    std::memset(L.ncod, 0, sizeof(int) * 2 * (size_t)s.d.N);
    p.incoming_left = 0;
    p.incoming_right = 0;
    for (int n = 0; n < p.nofbc; ++n) {
        int t = p.nbc[n], side = p.nofside[n];
        if (t == 2 || t == 20 || t == 40 || side == 5) throw Stop{GF_ERR_UNSUPPORTED};
        int ndbc = p.nbc2[n] - p.nbc1[n] + 1;
        bool vel = t == 1 || t == 10 || t == 30 || (side == 2 && t == 200);
        // coordinate along the side, scaled to [0,1] over the condition's range
        auto along = [&](int k) -> double { // k: 1-based node along the side
            if (side == 1) return s.cord(k - 1, 0, 1);
            if (side == 3) return s.cord(k - 1, nx - 1, 1);
            if (side == 2) return s.cord(nz - 1, k - 1, 0);
            return s.cord(0, k - 1, 0);
        };
        double x1 = along(p.nbc1[n]), x2 = along(p.nbc2[n]);
        for (int m = 1; m <= ndbc; ++m) {
            int numbp = m + p.nbc1[n] - 1;
            double x = (along(numbp) - x1) / (x2 - x1);
            if (vel) {
                if (side == 1) velbc(s, n, numbp - 1, 0, x);
                if (side == 2) velbc(s, n, nz - 1, numbp - 1, x);
                if (side == 3) velbc(s, n, numbp - 1, nx - 1, x);
                if (side == 4) velbc(s, n, 0, numbp - 1, x);
            }
            if (side == 1 && (t == 1 || t == 10) && p.bca[n] > 0) p.incoming_left = 1;
            if (side == 3 && (t == 1 || t == 10) && p.bca[n] < 0) p.incoming_right = 1;
        }
    }
    p.nopbmax = 0;
    double vbc = 0.0;
    for (int i = 0; i < nx; ++i)
        for (int j = 0; j < nz; ++j)
            for (int k = 0; k < 2; ++k) {
                int c = L.ncod[o_n2(s.d, j, i, k)];
                if (c == 1 || c == 10 || c == 30) vbc = std::max(vbc, std::fabs(L.bc[o_n2(s.d, j, i, k)]));
            }
    if (vbc == 0.0) vbc = 1.0e-10;
    p.vbc = vbc;
}

// setflac (src/setflac.f90:4-66): the start-up state up to (not including)
// rmasses / init_visc / dt_mass, which or_finish_setflac runs
void setflac(St &s) {
    gf_params &p = *s.p;
    gf_clock &c = *s.c;
    gf_layout &L = *s.L;
    size_t N = (size_t)s.d.N, E = (size_t)s.d.E;
    std::memset(&c, 0, sizeof c);
    c.nloop = 0;
    c.time = 0.0;
    c.frac = p.frac;
    init_cord(s);
    std::fill(L.aps, L.aps + E, 0.0);
    std::fill(L.vel, L.vel + 2 * N, 0.0);
    std::fill(L.dvol, L.dvol + 4 * E, 0.0);
    std::fill(L.strain, L.strain + 3 * E, 0.0);
    init_phase(s);
    init_marker(s);
    // check_visc_rheol (src/init_phase.f90:56-72)
    p.ivis_present = 0;
    for (size_t e = 0; e < E; ++e) {
        int irh = p.irheol[L.iphase[e] - 1];
        if (irh == 3 || irh >= 11) p.ivis_present = 1;
    }
    init_areas(s);
    double amin = 1e300;
    for (size_t e = 0; e < E; ++e) amin = std::min(amin, 0.5 / L.area[e] + 0.5 / L.area[E + e]);
    p.Amin = amin;
    init_temp(s);
    init_stress(s);
    init_bc(s);
    std::copy(L.temp, L.temp + N, L.temp0);
    if (L.xoriginal) std::copy(L.cord, L.cord + N, L.xoriginal);
    if (L.zoriginal) std::copy(L.cord + N, L.cord + 2 * N, L.zoriginal);
    for (double *f : {L.shrheat, L.sshrheat, L.fmagma, L.fmagma2, L.dike_released, L.fmelt, L.fmelt2, L.dike_backlog,
                      L.dike_marker_vol, L.mor_marker_vol, L.visn})
        if (f) std::fill(f, f + E, 0.0);
    std::fill(L.e2sr, L.e2sr + E, 1e-16);
    std::fill(L.se2sr, L.se2sr + 3 * E, 1e-16);
    if (L.dtopo) std::fill(L.dtopo, L.dtopo + p.nx, 0.0);
    if (L.extrusion) std::fill(L.extrusion, L.extrusion + p.nx, 0.0);
    if (L.q_init) std::fill(L.q_init, L.q_init + p.nx, 0.0);
    std::fill(L.amass, L.amass + N, 0.0);
    std::fill(L.rmass, L.rmass + N, 0.0);
    c.dtavg = 0.0;
    c.nsrate = -1;
}

template <class F> int guard(F &&f) {
    try {
        f();
    } catch (const Stop &st) {
        return st.code;
    }
    return 0;
}

} // namespace

extern "C" {

// 1: the oracle's exp/pow/sin/tan from the C library; 0: from gf_math.h
void or_set_libm(int on) { g_libm = on != 0; }

// Batch evaluation of gf_math.h's functions (fn 0 exp, 1 log, 2 pow, 3 sin,
// 4 cos, 5 tan) for the accuracy test against the C library; y only for pow
void or_gfm(int fn, const double *x, const double *y, double *out, long long n) {
    for (long long k = 0; k < n; ++k) {
        double v = x[k];
        switch (fn) {
        case 0: out[k] = gfm::exp(v); break;
        case 1: out[k] = gfm::log(v); break;
        case 2: out[k] = gfm::pow(v, y[k]); break;
        case 3: out[k] = gfm::sin(v); break;
        case 4: out[k] = gfm::cos(v); break;
        default: out[k] = gfm::tan(v); break;
        }
    }
}

void or_set_threads(int n) { g_threads = n > 0 ? n : 1; }
int or_get_threads(void) { return g_threads; }

#define OR_ENTRY(name, body)                                                                                           \
    int or_##name(gf_params *p, gf_clock *c, gf_layout *L) {                                                             \
        St s = make(p, c, L);                                                                                          \
        return guard([&] { body; });                                                                                   \
    }

OR_ENTRY(fl_therm, fl_therm(s))
OR_ENTRY(change_phase, change_phase(s))
OR_ENTRY(fl_rheol, fl_rheol(s))
OR_ENTRY(fl_node, fl_node(s))
OR_ENTRY(fl_move, fl_move(s))
OR_ENTRY(rmasses, rmasses(s))
OR_ENTRY(dt_mass, dt_mass(s))
OR_ENTRY(init_visc, init_visc(s))
OR_ENTRY(marker2elem, marker2elem(s))
OR_ENTRY(bar2euler, bar2euler(s))
OR_ENTRY(lpeuler2bar, lpeuler2bar(s))
OR_ENTRY(remesh, remesh(s))
OR_ENTRY(remesh_event, remesh_event(s))

// read_params (src/read_params.f90:3-348) into *p; markers_per_side,
// eclogite_rule and therm_sweeps keep the caller's values
int or_read_params(const char *path, gf_params *p) {
    if (!path || !p) return GF_ERR_ARG;
    return read_params(path, p);
}

// setflac (src/setflac.f90:4-66) on the caller's host arrays
int or_setflac(gf_params *p, gf_clock *c, gf_layout *L) {
    if (!p || !c || !L || L->nx != p->nx || L->nz != p->nz || L->nphase != p->nphase) return GF_ERR_ARG;
    St s = make(p, c, L);
    return guard([&] { setflac(s); });
}

// rmasses, init_visc, dt_mass and the averaging reset of setflac.f90:71-81
int or_finish_setflac(gf_params *p, gf_clock *c, gf_layout *L) {
    St s = make(p, c, L);
    return guard([&] {
        rmasses(s);
        if (p->ivis_present == 1) init_visc(s);
        dt_mass(s);
        c->dtavg = 0;
        c->nsrate = -1;
    });
}

// The tail of rsflac (src/rsflac.f90:197-236) after marker2elem and init_bc:
// init_areas, temp0 = temp, heating and strain-rate accumulators reset, dvol
// cleared, rmasses, init_visc, dt_mass, averaging reset
int or_restart_tail(gf_params *p, gf_clock *c, gf_layout *L) {
    St s = make(p, c, L);
    return guard([&] {
        const long long E = s.d.E, N = s.d.N;
        init_areas(s);
        std::memcpy(L->temp0, L->temp, sizeof(double) * (size_t)N);
        for (long long e = 0; e < E; ++e) {
            L->shrheat[e] = 0.0;
            L->sshrheat[e] = 0.0;
            L->e2sr[e] = 1e-16;
        }
        for (long long e = 0; e < 3 * E; ++e) L->se2sr[e] = 1e-16;
        for (long long e = 0; e < 4 * E; ++e) L->dvol[e] = 0.0;
        rmasses(s);
        if (p->ivis_present == 1) init_visc(s);
        dt_mass(s);
        c->dtavg = 0;
        c->nsrate = -1;
    });
}

// flac (src/flac.f90:5-91) followed by par.f90:84-87
int or_flac(gf_params *p, gf_clock *c, gf_layout *L) {
    St s = make(p, c, L);
    return guard([&] {
        fl_therm(s);
        if (p->itherm != 2) {
            if (c->nloop % p->ifreq_rmasses == 0) change_phase(s);
            fl_rheol(s);
            fl_node(s);
            fl_move(s);
            if (c->nloop % p->ifreq_rmasses == 0) rmasses(s);
            if (c->nloop % p->ifreq_imasses == 0) dt_mass(s);
        }
        c->nloop = c->nloop + 1;
        c->time = c->time + c->dt;
    });
}

int or_step(gf_params *p, gf_clock *c, gf_layout *L, int nsteps) {
    for (int k = 0; k < nsteps; ++k) {
        int rc = or_flac(p, c, L);
        if (rc) return rc;
    }
    return 0;
}

// itest_mesh (rem_test.f90:9-139): shortening (mode_rem 3 / 11, code 2),
// surface topography change (code 3), then the smallest angle (code 1); the
// angle is returned in every case
int or_itest_mesh(gf_params *p, gf_clock *c, gf_layout *L, double *angle) {
    St s = make(p, c, L);
    int need = 0;
    const int nx = p->nx;
    if (p->mode_rem == 11 || p->mode_rem == 3) {
        double testcr = p->dx_rem * p->rxbo / (nx - 1);
        double shortening = std::fabs(s.cord(0, nx - 1, 0) - s.cord(0, 0, 0) - p->rxbo);
        if (shortening > testcr) need = 2;
    }
    const double arc_extrusion_rate = 1.0 - p->ratio_mantle_mzone;
    if (need == 0 && (p->topo_kappa > 0 || arc_extrusion_rate > 0) && L->dhacc && L->extr_acc)
        for (int i = 0; i < nx - 1; ++i) {
            double testcr = (s.cord(0, 0, 1) - s.cord(1, 0, 1)) * 0.3333;
            double topochanges = std::fabs(L->dhacc[i]) + L->extr_acc[i];
            if (topochanges > testcr) need = 3;
        }
    double a = min_angle(s);
    if (angle) *angle = a;
    if (need == 0 && a <= p->angle_rem) need = 1;
    c->need_remeshing = need;
    return 0;
}

} // extern "C"
