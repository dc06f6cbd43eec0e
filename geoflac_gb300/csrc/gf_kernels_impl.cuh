// Kernel bodies and launchers of the FLAC step; included once per precision.
#pragma once

#include "gf_kernels.cuh"

// resident CTAs per SM the register allocation of k_rheol is sized for:
// 2 for FP64 (128 registers; its spills cost less than the latency that 16
// warps per SM hide: 0.703 -> 0.678 ms against 255 registers and 8 warps),
// 3 for the mixed path (80 registers; its few spills cost less than the
// occupancy they buy)
#ifndef GF_RHEOL_MINB
#define GF_RHEOL_MINB (sizeof(R) == sizeof(float) ? 3 : 2)
#endif

// internal linkage: each precision's translation unit has its own copy
namespace {
namespace gfk {

__device__ __forceinline__ void elem_ji(const GfDims &d, GF_IDX e, int &j, int &i) {
    i = (int)(e / (d.nz - 1));
    j = (int)(e - (GF_IDX)i * (d.nz - 1));
}
__device__ __forceinline__ void node_ji(const GfDims &d, GF_IDX n, int &j, int &i) {
    i = (int)(n / d.nz);
    j = (int)(n - (GF_IDX)i * d.nz);
}

inline unsigned grid_for(GF_IDX n) { return (unsigned)((n + GF_THREADS - 1) / GF_THREADS); }

// ======================================================================
// Mixed path: the element's share of the node forces of fl_node.f90.  For
// corner c (node 1..4 = (j,i), (j+1,i), (j,i+1), (j+1,i+1)) the three
// triangles that contain it contribute -0.25/ar * (s . grad N); written as
//   F_c = -sum_t 0.25/ar_t * ((s_t - s_ref) . grad N_c,t)   (small: stress
//         variation inside the element, s_ref = triangle 1's stored stress)
//   G_c =  sum_t 0.25/ar_t * grad N_c,t
// so that a node sums F_c - (s_ref,e - s_ref,n) . G_c over its elements
// (sum_e G_c = 0 around an interior node): every FP32 term is a difference.
// The triangle/vertex tables are fl_node.f90:7-8 for quad 4 - c.
__device__ __forceinline__ void elem_corner_forces(const float dx[3][4], const float dz[3][4], const float ar[4],
                                                   const float sn[4][4], float *__restrict__ frc, GF_IDX E,
                                                   GF_IDX e) {
    const int kk[4][3] = {{1, 2, 3}, {0, 1, 2}, {0, 1, 3}, {0, 2, 3}};
    const int mm[4][3] = {{2, 2, 1}, {1, 1, 1}, {2, 0, 2}, {0, 0, 0}};
#pragma unroll
    for (int c = 0; c < 4; ++c) {
        const int qd = 3 - c;
        float fx = 0.0f, fy = 0.0f, gx = 0.0f, gz = 0.0f;
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            const int t = kk[qd][k], m = mm[qd][k];
            const float factor = 0.25f / ar[t];
            const float ax = factor * dx[m][t], az = factor * dz[m][t];
            const float sxx = sn[0][t] - sn[0][1], szz = sn[1][t] - sn[1][1], sxz = sn[2][t] - sn[2][1];
            fx -= sxx * ax + sxz * az;
            fy -= sxz * ax + szz * az;
            gx += ax;
            gz += az;
        }
        frc[(4 * c + 0) * E + e] = fx;
        frc[(4 * c + 1) * E + e] = fy;
        frc[(4 * c + 2) * E + e] = gx;
        frc[(4 * c + 3) * E + e] = gz;
    }
}

// ======================================================================
// fl_rheol (fl_rheol.f90:4-389): one thread per element.
template <class R> __device__ __forceinline__ void b_k_rheol(const DevParams *__restrict__ Pp, DevClock *__restrict__ C, DevArrays A, GfDims d, int update_visc, int nloop, GF_IDX e) {
    if (e >= d.E) return;
    const DevParams &P = *Pp;
    int j, i;
    elem_ji(d, e, j, i);
    const double dtd = C->dt;
    if (e == 0) C->dtavg = C->dtavg + dtd; // fl_rheol.f90:43 (no thread reads dtavg here)
    const R dt = gf_to<R>(dtd);
    R *st = (R *)A.stress0;
    const R *area = (const R *)A.area;

    GF_IDX n1 = gf_node(d, j, i), n3 = gf_node(d, j, i + 1);
    R vx[4], vy[4];
    R ar[4];
    for (int k = 0; k < 4; ++k) ar[k] = area[gf_ek(d, e, k)];
    R dx[3][4], dz[3][4], sr[3][4];
    if constexpr (sizeof(R) == sizeof(float)) {
        // FP32 from the hi/lo splits: coordinates and velocities relative to
        // the quad's node 1 (each triangle's shape derivatives sum to zero,
        // so a common velocity offset drops out of the strain rates)
        QuadF qf;
        load_vel_rel(A, d, j, i, vx, vy);
        load_quad_rel(A, d, j, i, qf);
        shape_derivs_f(qf, ar, dx, dz);
    } else {
        const double *vel = A.vel;
        vx[0] = R(vel[n1]); vx[1] = R(vel[n1 + 1]); vx[2] = R(vel[n3]); vx[3] = R(vel[n3 + 1]);
        vy[0] = R(vel[d.N + n1]); vy[1] = R(vel[d.N + n1 + 1]); vy[2] = R(vel[d.N + n3]); vy[3] = R(vel[d.N + n3 + 1]);
        Quad q;
        load_quad(A.cord, d, j, i, q);
        shape_derivs<R>(q, ar, dx, dz);
    }
    // node triplets of triangles A,B,C,D: (1,2,3), (3,2,4), (1,2,4), (1,4,3)
    const int tn[4][3] = {{0, 1, 2}, {2, 1, 3}, {0, 1, 3}, {0, 3, 2}};
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        R a0 = vx[tn[k][0]], a1 = vx[tn[k][1]], a2 = vx[tn[k][2]];
        R b0 = vy[tn[k][0]], b1 = vy[tn[k][1]], b2 = vy[tn[k][2]];
        sr[0][k] = a0 * dx[0][k] + a1 * dx[1][k] + a2 * dx[2][k];
        sr[1][k] = b0 * dz[0][k] + b1 * dz[1][k] + b2 * dz[2][k];
        sr[2][k] = gf_scale<-1>(a0 * dz[0][k] + a1 * dz[1][k] + a2 * dz[2][k] +
                                b0 * dx[0][k] + b1 * dx[1][k] + b2 * dx[2][k]);
    }
    if (P.mix_strain == 1) {
#pragma unroll
        for (int k = 0; k < 4; k += 2) {
            R em = R(0.5) * (sr[0][k] + sr[1][k] + sr[0][k + 1] + sr[1][k + 1]);
            R eda = sr[0][k] - sr[1][k];
            R edb = sr[0][k + 1] - sr[1][k + 1];
            sr[0][k] = R(0.5) * (em + eda);
            sr[1][k] = R(0.5) * (em - eda);
            sr[0][k + 1] = R(0.5) * (em + edb);
            sr[1][k + 1] = R(0.5) * (em - edb);
        }
    }
    R *se2sr = (R *)A.se2sr;
    R *sshrheat = (R *)A.sshrheat;
    R s11 = gf_scale<-2>(sr[0][0] + sr[0][1] + sr[0][2] + sr[0][3]);
    R s22 = gf_scale<-2>(sr[1][0] + sr[1][1] + sr[1][2] + sr[1][3]);
    R s12 = gf_scale<-2>(sr[2][0] + sr[2][1] + sr[2][2] + sr[2][3]);
    R srII = gf_scale<-1>(m_sqrt((s11 - s22) * (s11 - s22) + gf_scale<2>(s12) * s12));
    R srI = gf_scale<-1>(s11 + s22);
    R srs2 = (s11 - srI) * (s11 - srI) + (s22 - srI) * (s22 - srI) + gf_scale<1>(s12) * s12;
    se2sr[gf_ek(d, e, 0)] = se2sr[gf_ek(d, e, 0)] + s11 * dt;
    se2sr[gf_ek(d, e, 1)] = se2sr[gf_ek(d, e, 1)] + s22 * dt;
    se2sr[gf_ek(d, e, 2)] = se2sr[gf_ek(d, e, 2)] + s12 * dt;
    R s0v[4][4]; // start-of-step stresses [comp][tri]
#pragma unroll
    for (int k = 0; k < 4; ++k)
#pragma unroll
        for (int c = 0; c < 4; ++c) s0v[c][k] = st[gf_s(d, e, c, k)];
    s11 = gf_scale<-2>(s0v[0][0] + s0v[0][1] + s0v[0][2] + s0v[0][3]);
    s22 = gf_scale<-2>(s0v[1][0] + s0v[1][1] + s0v[1][2] + s0v[1][3]);
    s12 = gf_scale<-2>(s0v[2][0] + s0v[2][1] + s0v[2][2] + s0v[2][3]);
    R stII = gf_scale<-1>(m_sqrt((s11 - s22) * (s11 - s22) + gf_scale<2>(s12) * s12));
    R shr = sshrheat[e];
    if (srII != R(0.0)) shr = shr + gf_ddiv(stII, srII) * srs2 * dt;

    int iph = A.iphase[e] - 1;
    int irh = P.irheol[iph];
    R bulkm, rmu;
    if constexpr (sizeof(R) == sizeof(float)) {
        bulkm = P.f_bulkm[iph];
        rmu = P.f_rm[iph];
    } else {
        bulkm = R(P.bulkm[iph]);
        rmu = R(P.rm[iph]);
    }
    R stherm = R(0.0);
    if (P.istress_therm > 0)
        stherm = R(-P.alfa[iph] * P.bulkm[iph] * (A.temp[n1] - A.temp0[n1]));
    R *aps = (R *)A.aps;
    R aps_e = aps[e];
    // mixed path: stored normal stresses are deviations from -pref
    R pref = R(0);
    if constexpr (sizeof(R) == sizeof(float)) pref = A.pr_hi[e]; // == float(p_ref)
    R hardn = 0;
    PlasticConsts<R> pc;
    if (irh == 6 || irh >= 11) {
        // single-phase elements outside the softening interval read the
        // per-phase table
        const int pst = A.plast_tab ? plastic_table_state<R>(P, A, d, e, iph, aps_e) : -1;
        if (pst >= 0) {
            const R *t = (const R *)A.plast_tab + (GF_IDX)(pst * GF_MAXPH + iph) * GF_PT_W;
            pc.anphi = t[0]; pc.anpsi = t[1]; pc.amc = t[2]; pc.e1 = t[3];
            pc.e2 = t[4]; pc.x1 = t[5]; pc.ten_max = t[6]; hardn = t[7];
            plastic_consts_f32(pc);
        } else {
            R coh = 0, phi = 0, psi = 0;
            pre_plast<R>(P, A, d, e, aps_e, coh, phi, psi, hardn);
            pc = plastic_consts<R>(bulkm, rmu, coh, phi, psi,
                                   sizeof(R) == sizeof(float) ? R(P.f_ten_off) : R(P.ten_off));
        }
    }
    R *visn = (R *)A.visn;
    R vis;
    if ((irh == 3 || irh >= 11) && update_visc) {
        vis = R(visc_of<R>(P, A, d, j, i, e, st));
        visn[e] = vis;
    } else {
        vis = visn[e];
    }
    R dike = A.dike_released ? gf_to<R>(A.dike_released[e]) : R(0);
    const R *dvol = (const R *)A.dvol;
    R sp[4][4], sv[4][4], depl[4] = {0, 0, 0, 0};
    bool plas_mod = false;
    MaxwellConsts<R> mc;
    if (irh == 3 || irh >= 11) mc = maxwell_consts<R>(rmu, vis, dt);
    const bool ok = !(irh == 3 || irh >= 11) || mc.ok;
    R sumD = 0, sumD12 = 0; // strain-increment sums for the FP32 selection
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        R de11 = sr[0][k] * dt, de22 = sr[1][k] * dt, de12 = sr[2][k] * dt, de33 = R(0.0);
        // (dike and stherm are +0 without dikes and thermal stress:
        // gf_sub_z / gf_add_z take them on the integer pipes)
        R dv = gf_sub_z(dvol[gf_ek(d, e, k)], dike);
        sp[0][k] = gf_add_z(s0v[0][k], stherm);
        sp[1][k] = gf_add_z(s0v[1][k], stherm);
        sp[2][k] = s0v[2][k];
        sp[3][k] = gf_add_z(s0v[3][k], stherm);
        sv[0][k] = sp[0][k]; sv[1][k] = sp[1][k]; sv[2][k] = sp[2][k]; sv[3][k] = sp[3][k];
        if (irh == 1) {
            elastic<R>(bulkm, rmu, sp[0][k], sp[1][k], sp[3][k], sp[2][k], de11, de22, de12);
        } else if (irh == 3) {
            maxwell<R>(bulkm, mc, sv[0][k], sv[1][k], sv[3][k], sv[2][k], de11, de22, de33, de12, dv, P.ndim);
        } else if (irh == 6) {
            bool m;
            plastic_sel(pc, rmu, depl[k], hardn, sp[0][k], sp[1][k], sp[3][k], sp[2][k], de11, de22, de33, de12, pref,
                        m);
        } else if (irh >= 11) {
            bool m;
            plastic_sel(pc, rmu, depl[k], hardn, sp[0][k], sp[1][k], sp[3][k], sp[2][k], de11, de22, de33, de12, pref,
                        m);
            plas_mod = plas_mod || m;
            maxwell<R>(bulkm, mc, sv[0][k], sv[1][k], sv[3][k], sv[2][k], de11, de22, de33, de12, dv, P.ndim);
            if (sizeof(R) == sizeof(float)) {
                sumD = sumD + (de11 - de22);
                sumD12 = sumD12 + de12;
            }
        }
    }
    if (!ok) set_status(C, 22, (int)e);
    R sn[4][4]; // new stresses [comp][tri]
    bool use_visc = (irh == 3);
    if (irh >= 11) {
        R a = sp[0][0] + sp[0][1] + sp[0][2] + sp[0][3] - sp[1][0] - sp[1][1] - sp[1][2] - sp[1][3];
        R b = sp[2][0] + sp[2][1] + sp[2][2] + sp[2][3];
        R sII_plas = a * a + gf_scale<2>(b * b);
        a = sv[0][0] + sv[0][1] + sv[0][2] + sv[0][3] - sv[1][0] - sv[1][1] - sv[1][2] - sv[1][3];
        b = sv[2][0] + sv[2][1] + sv[2][2] + sv[2][3];
        R sII_visc = a * a + gf_scale<2>(b * b);
        use_visc = !(sII_plas < sII_visc);
        if (sizeof(R) == sizeof(float) && !plas_mod) {
            R pa = sp[0][0] + sp[0][1] + sp[0][2] + sp[0][3] - sp[1][0] - sp[1][1] - sp[1][2] - sp[1][3];
            R pb = sp[2][0] + sp[2][1] + sp[2][2] + sp[2][3];
            R S = s0v[0][0] + s0v[0][1] + s0v[0][2] + s0v[0][3] - s0v[1][0] - s0v[1][1] - s0v[1][2] - s0v[1][3];
            R B = s0v[2][0] + s0v[2][1] + s0v[2][2] + s0v[2][3];
            use_visc = maxwell_wins_unyielded(float(pa), float(pb), float(S), float(B), float(sumD), float(sumD12),
                                              float(rmu), float(vis), float(dt));
        }
    }
#pragma unroll
    for (int k = 0; k < 4; ++k)
#pragma unroll
        for (int c = 0; c < 4; ++c) sn[c][k] = use_visc ? sv[c][k] : sp[c][k];
    // FP64: the reciprocals 1/ar of the stress mixing and the node-force
    // factors 0.25/ar, one IEEE division per triangle
    R rar[4];
    if constexpr (sizeof(R) == sizeof(double)) {
        if (P.mix_stress == 1 || A.n_frc) {
#pragma unroll
            for (int t = 0; t < 4; ++t) rar[t] = gf_rcp(ar[t]); // RN(1/ar) off the FP64 pipe
        }
    }
    if (P.mix_stress == 1) {
#pragma unroll
        for (int h = 0; h < 4; h += 2) {
            R ra = ar[h], rb = ar[h + 1];
            R s0a = gf_scale<-1>(sn[0][h] + sn[1][h]);
            R s0b = gf_scale<-1>(sn[0][h + 1] + sn[1][h + 1]);
            R s0;
            if constexpr (sizeof(R) == sizeof(double)) {
                const GfRecip qa = gf_recip_y(ra, rar[h]), qb = gf_recip_y(rb, rar[h + 1]);
                R quad_area = qa.y + qb.y;
                s0 = gf_ddiv(gf_div(s0a, qb) + gf_div(s0b, qa), quad_area);
            } else {
                R quad_area = R(1.0) / ra + R(1.0) / rb;
                s0 = (s0a / rb + s0b / ra) / quad_area;
            }
            sn[0][h] = sn[0][h] - s0a + s0;
            sn[1][h] = sn[1][h] - s0a + s0;
            sn[0][h + 1] = sn[0][h + 1] - s0b + s0;
            sn[1][h + 1] = sn[1][h + 1] - s0b + s0;
        }
    }
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        sn[0][k] = gf_sub_z(sn[0][k], stherm);
        sn[1][k] = gf_sub_z(sn[1][k], stherm);
        sn[3][k] = gf_sub_z(sn[3][k], stherm);
    }
#pragma unroll
    for (int k = 0; k < 4; ++k)
#pragma unroll
        for (int c = 0; c < 4; ++c) st[gf_s(d, e, c, k)] = sn[c][k];
    if constexpr (sizeof(R) == sizeof(double)) {
        // fl_node's force terms of this element (fl_node.f90:50-254), each
        // the expression the node gather evaluates, from the stresses just
        // stored: the node kernel then sums them in the reference's order
        // instead of recomputing four elements' shape derivatives and twelve
        // divisions per node (the mesh does not move before fl_node)
        if (A.n_frc) {
            const int kk[4][3] = {{1, 2, 3}, {0, 1, 2}, {0, 1, 3}, {0, 2, 3}};
            const int mm[4][3] = {{2, 2, 1}, {1, 1, 1}, {2, 0, 2}, {0, 0, 0}};
            double *nf = A.n_frc;
#pragma unroll
            for (int c = 0; c < 4; ++c) {
                const int qd = 3 - c;
#pragma unroll
                for (int k = 0; k < 3; ++k) {
                    const int t = kk[qd][k], m = mm[qd][k];
                    // 0.25 * RN(1/ar) == RN(0.25/ar) while both are normal
                    R factor = gf_dmid(ar[t]) ? gf_scale<-2>(rar[t]) : R(0.25) / ar[t];
                    R fx = factor * (sn[0][t] * dx[m][t] + sn[2][t] * dz[m][t]);
                    R fy = factor * (sn[2][t] * dx[m][t] + sn[1][t] * dz[m][t]);
                    nf[(GF_IDX)(6 * c + 2 * k) * d.E + e] = fx;
                    nf[(GF_IDX)(6 * c + 2 * k + 1) * d.E + e] = fy;
                }
            }
        }
    }
    if constexpr (sizeof(R) == sizeof(float)) {
        // the node gather's corner forces of the new stresses (the mesh does
        // not move before fl_node); shape derivatives taken again rather than
        // kept live through the stress update
        QuadF q2;
        load_quad_rel(A, d, j, i, q2);
        float dx2[3][4], dz2[3][4];
        shape_derivs_f(q2, ar, dx2, dz2);
        elem_corner_forces(dx2, dz2, ar, sn, A.e_frc, d.E, e);
    }
    if (irh == 6 || irh >= 11) {
        R quad_area = ar[0] + ar[1] + ar[2] + ar[3];
        aps_e = aps_e + gf_ddiv(depl[0] * ar[0] + depl[1] * ar[1] + depl[2] * ar[2] + depl[3] * ar[3], quad_area);
        if (aps_e < R(0.0)) aps_e = R(0.0);
        if constexpr (sizeof(R) == sizeof(float)) {
            if (P.f_tau_heal != 0.0f) aps_e = aps_e / (1.0f + dt / P.f_tau_heal);
        } else {
            if (P.tau_heal != 0.0) aps_e = aps_e / (R(1.0) + dt / R(P.tau_heal));
        }
        aps[e] = aps_e;
    }
    // accumulates the element-averaged start-of-step stress (s11/s22/s12 are
    // reassigned before this point in fl_rheol.f90:181-183)
    R *strain = (R *)A.strain;
    if (sizeof(R) == sizeof(float)) { // total stress, not the stored deviation
        s11 = s11 - pref;
        s22 = s22 - pref;
    }
    strain[gf_ek(d, e, 0)] = strain[gf_ek(d, e, 0)] + s11 * dt;
    strain[gf_ek(d, e, 1)] = strain[gf_ek(d, e, 1)] + s22 * dt;
    strain[gf_ek(d, e, 2)] = strain[gf_ek(d, e, 2)] + s12 * dt;
    if (P.ishearh == 1) {
        R qsum = R(0.0);
        if constexpr (sizeof(R) == sizeof(float)) {
            R lambda = bulkm - R(2.0 / 3.0) * rmu, mu = rmu;
            R den_el = R(3.0) * lambda + R(2.0) * mu;
            if (m_abs(den_el) < R(1e-30)) den_el = den_el < R(0) ? R(-1e-30) : R(1e-30);
            // the same elastic-strain differences with one reciprocal and the
            // stress changes taken first
            const float lamr = lambda / den_el, inv2mu = 1.0f / (2.0f * mu);
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                float f11 = sn[0][k], f22 = sn[1][k], f12 = sn[2][k], f33 = sn[3][k];
                float dtr = ((f11 - s0v[0][k]) + (f22 - s0v[1][k])) + (f33 - s0v[3][k]);
                float d11 = sr[0][k] * dt - ((f11 - s0v[0][k]) - lamr * dtr) * inv2mu;
                float d22 = sr[1][k] * dt - ((f22 - s0v[1][k]) - lamr * dtr) * inv2mu;
                float d12 = sr[2][k] * dt - (f12 - s0v[2][k]) * inv2mu;
                float d33 = -(((f33 - s0v[3][k]) - lamr * dtr) * inv2mu);
                float a11 = 0.5f * (s0v[0][k] + f11), a22 = 0.5f * (s0v[1][k] + f22),
                      a12 = 0.5f * (s0v[2][k] + f12), a33 = 0.5f * (s0v[3][k] + f33);
                float qk = a11 * d11 + a22 * d22 + 2.0f * a12 * d12 + a33 * d33;
                qk -= pref * (d11 + d22 + d33); // isotropic reference part
                qsum = qsum + 0.25f * qk;
            }
        } else {
            // the 32 quotients by 2 mu (fl_rheol.f90:352-362) share one
            // reciprocal; gf_div gives each the bits of the division.  The
            // phase's lambda / den_el and reciprocal pair of 2 mu are the
            // same expressions evaluated once per phase at set-up.
            const GfRecip r2mu = gf_recip_pre(R(2.0) * rmu, P.sh_r2mu_y[iph], P.sh_r2mu_yl[iph]);
            auto by2mu = [&](R a) { return gf_div(a, r2mu); };
            const R lam_den = P.sh_lam_den[iph];
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                R f11 = sn[0][k], f22 = sn[1][k], f12 = sn[2][k], f33 = sn[3][k];
                R tr0 = s0v[0][k] + s0v[1][k] + s0v[3][k];
                R lt0 = lam_den * tr0;
                R e11a = by2mu(s0v[0][k] - lt0);
                R e22a = by2mu(s0v[1][k] - lt0);
                R e33a = by2mu(s0v[3][k] - lt0);
                R e12a = by2mu(s0v[2][k]);
                R tr1 = f11 + f22 + f33;
                R lt1 = lam_den * tr1;
                R e11b = by2mu(f11 - lt1);
                R e22b = by2mu(f22 - lt1);
                R e33b = by2mu(f33 - lt1);
                R e12b = by2mu(f12);
                R d11 = sr[0][k] * dt - (e11b - e11a);
                R d22 = sr[1][k] * dt - (e22b - e22a);
                R d12 = sr[2][k] * dt - (e12b - e12a);
                R d33 = gf_zero_minus(e33b - e33a);
                R a11 = gf_scale<-1>(s0v[0][k] + f11), a22 = gf_scale<-1>(s0v[1][k] + f22),
                  a12 = gf_scale<-1>(s0v[2][k] + f12), a33 = gf_scale<-1>(s0v[3][k] + f33);
                R qk = a11 * d11 + a22 * d22 + gf_scale<1>(a12) * d12 + a33 * d33;
                qsum = qsum + gf_scale<-2>(qk);
            }
        }
        shr = shr + qsum;
    }
    sshrheat[e] = shr;
    (void)nloop;
}
template <class R> __global__ void __launch_bounds__(GF_THREADS, GF_RHEOL_MINB) k_rheol(const DevParams *__restrict__ Pp, DevClock *__restrict__ C, DevArrays A, GfDims d, int update_visc, int nloop) {
    gf_pdl_entry();
    b_k_rheol<R>(Pp, C, A, d, update_visc, nloop, (GF_IDX)blockIdx.x * blockDim.x + threadIdx.x);
}

template <class R> __device__ __forceinline__ void b_k_rheol_avg(DevClock *__restrict__ C, DevArrays A, GfDims d, int reset, GF_IDX e) {
    if (e >= d.E) return;
    R *se2sr = (R *)A.se2sr;
    R *e2sr = (R *)A.e2sr;
    R *shrheat = (R *)A.shrheat;
    R *sshrheat = (R *)A.sshrheat;
    R dtavg = R(C->dtavg);
    R a = se2sr[gf_ek(d, e, 0)], b = se2sr[gf_ek(d, e, 1)], q = se2sr[gf_ek(d, e, 2)];
    e2sr[e] = (R(0.5) * m_sqrt((a - b) * (a - b) + R(4.0) * q * q)) / dtavg;
    shrheat[e] = sshrheat[e] / dtavg;
    if (reset) {
        se2sr[gf_ek(d, e, 0)] = R(0.0);
        se2sr[gf_ek(d, e, 1)] = R(0.0);
        se2sr[gf_ek(d, e, 2)] = R(0.0);
        sshrheat[e] = R(0.0);
    }
}
template <class R> __global__ void __launch_bounds__(GF_THREADS) k_rheol_avg(DevClock *__restrict__ C, DevArrays A, GfDims d, int reset) {
    gf_pdl_entry();
    b_k_rheol_avg<R>(C, A, d, reset, (GF_IDX)blockIdx.x * blockDim.x + threadIdx.x);
}

// scalar bookkeeping of fl_rheol: dtavg += dt at entry; dtavg = 0 at a reset
__device__ __forceinline__ void b_k_rheol_clock(DevClock *C, int phase) {
    if (phase == 0)
        C->dtavg = C->dtavg + C->dt;
    else
        C->dtavg = 0.0;
}
__global__ void k_rheol_clock(DevClock *C, int phase) {
    b_k_rheol_clock(C, phase);
}

// ======================================================================
// fl_node (fl_node.f90:3-393): one thread per node, forces gathered from
// the 4 adjacent quads in the reference's order, no atomics.
//
// Threads are numbered boundary ring first (top row, bottom row, left and
// right columns), then the interior nodes (column by column, j fastest), so
// that the boundary nodes, which take the FP64 path with water load and
// Winkler foundation, run in warps of their own and start first.
__device__ __forceinline__ GF_IDX node_of_slot(const GfDims &d, GF_IDX t) {
    const int nzi = d.nz - 2;
    if (t < d.nx) return gf_node(d, 0, (int)t);
    t -= d.nx;
    if (t < d.nx) return gf_node(d, d.nz - 1, (int)t);
    t -= d.nx;
    if (t < nzi) return gf_node(d, 1 + (int)t, 0);
    t -= nzi;
    if (t < nzi) return gf_node(d, 1 + (int)t, d.nx - 1);
    t -= nzi;
    const int i = (int)(t / nzi);
    return gf_node(d, 1 + (int)(t - (GF_IDX)i * nzi), 1 + i);
}

// (hi, lo) + b in FP32 pairs: two-sum of hi and b, then renormalised
__device__ __forceinline__ void ff_add(float &hi, float &lo, float b) {
    const float s = hi + b;
    const float bb = s - hi;
    const float err = (hi - (s - bb)) + (b - bb);
    const float l = lo + err;
    hi = s + l;
    lo = l - (hi - s);
}

// Mixed path, interior node.  Stored normal stresses are deviations from
// the element's reference pressure p_ref.  The node sums its four elements'
// corner forces (elem_corner_forces, written by fl_rheol) with the
// reference-stress differences to one neighbouring triangle (sigma_n) and the
// p_ref differences, all small, so FP32 resolves the net force.  Damping and
// the velocity increment are FP32; the velocity is carried as its hi/lo FP32
// pair and written back to the FP64 array as hi + lo.
__device__ __forceinline__ void node_interior_f(const DevParams &P, const DevClock *__restrict__ C, DevArrays &A,
                                                const GfDims &d, GF_IDX n, int j, int i) {
    const float *st = (const float *)A.stress0;
    const float *frc = A.e_frc;
    const GF_IDX E = d.E;
    const GF_IDX en = gf_elem(d, j - 1, i - 1);
    const float nxx = st[gf_s(d, en, 0, 1)], nzz = st[gf_s(d, en, 1, 1)], nxz = st[gf_s(d, en, 2, 1)];
    float fx0 = 0.0f, fy0 = 0.0f;
#pragma unroll
    for (int qd = 0; qd < 4; ++qd) {
        const int je = j + (qd < 2 ? -1 : 0), ie = i + ((qd & 1) ? 0 : -1);
        const GF_IDX e = gf_elem(d, je, ie);
        const int c = 3 - qd; // this node's corner of element e
        const float dp = hl_diff(A.pr_hi, A.pr_lo, e, en);
        const float rxx = (st[gf_s(d, e, 0, 1)] - nxx) - dp;
        const float rzz = (st[gf_s(d, e, 1, 1)] - nzz) - dp;
        const float rxz = st[gf_s(d, e, 2, 1)] - nxz;
        const float gx = frc[(4 * c + 2) * E + e], gz = frc[(4 * c + 3) * E + e];
        fx0 += frc[(4 * c + 0) * E + e] - (rxx * gx + rxz * gz);
        fy0 += frc[(4 * c + 1) * E + e] - (rxz * gx + rzz * gz);
    }
    float f0 = fx0;
    float f1 = fy0 - gf_d2f(A.rmass[n]) * P.f_g;
    const float dtf = gf_d2f(C->dt);
    float drat = dtf / gf_d2f(C->dt_elastic);
    if (drat < 1.0f) drat = 1.0f;
    float h0 = A.vel_hi[n], l0 = A.vel_lo[n], h1 = A.vel_hi[d.N + n], l1 = A.vel_lo[d.N + n];
    const int c0 = A.ncod[n], c1 = A.ncod[d.N + n];
    if ((c0 & 1) != 1 && fabsf(h0) > 1.0e-13f) f0 = f0 - P.f_demf * copysignf(fabsf(f0), h0);
    if ((c1 & 2) != 2 && fabsf(h1) > 1.0e-13f) f1 = f1 - P.f_demf * copysignf(fabsf(f1), h1);
    const float s = dtf / (gf_d2f(A.amass[n]) * drat * drat);
    double v0, v1;
    if (c0 == 1) {
        v0 = A.bc[n];
        gf_split(v0, h0, l0);
    } else {
        ff_add(h0, l0, s * f0);
        v0 = gf_f2d(h0) + gf_f2d(l0);
    }
    if (c1 == 1) {
        v1 = A.bc[d.N + n];
        gf_split(v1, h1, l1);
    } else {
        ff_add(h1, l1, s * f1);
        v1 = gf_f2d(h1) + gf_f2d(l1);
    }
    A.vel[n] = v0;
    A.vel[d.N + n] = v1;
    A.vel_hi[n] = h0;
    A.vel_lo[n] = l0;
    A.vel_hi[d.N + n] = h1;
    A.vel_lo[d.N + n] = l1;
}

template <class R> __device__ __forceinline__ void b_k_node(const DevParams *__restrict__ Pp, DevClock *__restrict__ C, DevArrays A, GfDims d, GF_IDX slot, int terms = 0) {
    if (slot >= d.N) return;
    const GF_IDX n = node_of_slot(d, slot);
    const DevParams &P = *Pp;
    int j, i;
    node_ji(d, n, j, i);
    const int nx = d.nx, nz = d.nz;
    const R *st = (const R *)A.stress0;
    const R *area = (const R *)A.area;
    // kk/mm tables of fl_node.f90:7-8 (0-based)
    const int kk[4][3] = {{1, 2, 3}, {0, 1, 2}, {0, 1, 3}, {0, 2, 3}};
    const int mm[4][3] = {{2, 2, 1}, {1, 1, 1}, {2, 0, 2}, {0, 0, 0}};
    double f0, f1;
    const bool interior = j > 0 && j < nz - 1 && i > 0 && i < nx - 1;
    if constexpr (sizeof(R) == sizeof(float)) {
        if (interior) {
            node_interior_f(P, C, A, d, n, j, i);
            return;
        }
    }
    if constexpr (sizeof(R) == sizeof(float)) {
        // Mixed path, boundary node: the elements' corner forces plus their
        // total reference stress (triangle-1 stress less p_ref) against the
        // corner geometry G_c, in FP64 from the node coordinates:
        // 0.25/ar * grad N = 0.25 * (y_u - y_v, x_v - x_u) for the edge (u, v)
        // that shape_derivs uses for vertex m of triangle t.
        const int uv[4][3][2] = {{{1, 2}, {2, 0}, {0, 1}}, {{1, 3}, {3, 2}, {2, 1}},
                                 {{1, 3}, {3, 0}, {0, 1}}, {{3, 2}, {2, 0}, {0, 3}}};
        const float *frc = A.e_frc;
        const double *cx = A.cord, *cy = A.cord + d.N;
        double gx = 0.0, gy = 0.0;
#pragma unroll
        for (int qd = 0; qd < 4; ++qd) {
            int je = j + (qd < 2 ? -1 : 0), ie = i + ((qd & 1) ? 0 : -1);
            if (je < 0 || ie < 0 || je > nz - 2 || ie > nx - 2) continue;
            const GF_IDX e = gf_elem(d, je, ie);
            const int c = 3 - qd;
            GF_IDX nn[4];
            quad_nodes(d, je, ie, nn);
            double Gx = 0.0, Gz = 0.0;
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                const int t = kk[qd][k], m = mm[qd][k];
                const GF_IDX u = nn[uv[t][m][0]], v = nn[uv[t][m][1]];
                Gx += cy[u] - cy[v];
                Gz += cx[v] - cx[u];
            }
            Gx *= 0.25;
            Gz *= 0.25;
            const double pe = A.p_ref[e];
            const double rxx = (double)st[gf_s(d, e, 0, 1)] - pe, rzz = (double)st[gf_s(d, e, 1, 1)] - pe,
                         rxz = (double)st[gf_s(d, e, 2, 1)];
            gx += (double)frc[(4 * c + 0) * d.E + e] - (rxx * Gx + rxz * Gz);
            gy += (double)frc[(4 * c + 1) * d.E + e] - (rxz * Gx + rzz * Gz);
        }
        f0 = gx;
        f1 = gy - A.rmass[n] * P.g;
    } else if (terms) {
        // FP64 path, terms written by fl_rheol: the reference's sum order
        R fx0 = R(0.0), fy0 = R(0.0);
#pragma unroll
        for (int qd = 0; qd < 4; ++qd) {
            int je = j + (qd < 2 ? -1 : 0), ie = i + ((qd & 1) ? 0 : -1);
            if (je < 0 || ie < 0 || je > nz - 2 || ie > nx - 2) continue;
            const GF_IDX e = gf_elem(d, je, ie);
            const int c = 3 - qd;
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                fx0 = fx0 - A.n_frc[(GF_IDX)(6 * c + 2 * k) * d.E + e];
                fy0 = fy0 - A.n_frc[(GF_IDX)(6 * c + 2 * k + 1) * d.E + e];
            }
        }
        f0 = (double)fx0;
        f1 = (double)fy0 - gf_mul(A.rmass[n], P.g);
    } else {
        // FP64 path: the reference's gather from the four quads
        R fx0 = R(0.0), fy0 = R(0.0);
#pragma unroll
        for (int qd = 0; qd < 4; ++qd) {
            int je = j + (qd < 2 ? -1 : 0), ie = i + ((qd & 1) ? 0 : -1);
            if (je < 0 || ie < 0 || je > nz - 2 || ie > nx - 2) continue;
            GF_IDX e = gf_elem(d, je, ie);
            Quad q;
            load_quad(A.cord, d, je, ie, q);
            R ar[4];
#pragma unroll
            for (int k = 0; k < 4; ++k) ar[k] = area[gf_ek(d, e, k)];
            R dx[3][4], dz[3][4];
            shape_derivs<R>(q, ar, dx, dz);
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                int t = kk[qd][k], m = mm[qd][k];
                R factor = R(0.25) / ar[t];
                R sxx = st[gf_s(d, e, 0, t)], szz = st[gf_s(d, e, 1, t)], sxz = st[gf_s(d, e, 2, t)];
                R fx = factor * (sxx * dx[m][t] + sxz * dz[m][t]);
                R fy = factor * (sxz * dx[m][t] + szz * dz[m][t]);
                fx0 = fx0 - fx;
                fy0 = fy0 - fy;
            }
        }
        f0 = (double)fx0;
        f1 = (double)fy0 - A.rmass[n] * P.g;
    }
    const double *cord = A.cord;
    if (P.nyhydro > 0 && j == 0) { // water load on the surface
        double rho_water_g = 1030.0 * P.g;
        double water_depth = (i < nx - 1) ? 0.5 * (cord[d.N + gf_node(d, 0, i + 1)] + cord[d.N + gf_node(d, 0, i)])
                                          : 0.5 * (cord[d.N + gf_node(d, 0, i - 1)] + cord[d.N + gf_node(d, 0, i)]);
        if (water_depth < 0.0) {
            double pl = 0, dlxl = 0, dlyl = 0, pr = 0, dlxr = 0, dlyr = 0;
            if (i > 0) {
                pl = rho_water_g * ((cord[d.N + gf_node(d, 0, i - 1)] + cord[d.N + gf_node(d, 0, i)]) / 2.0);
                dlxl = cord[gf_node(d, 0, i)] - cord[gf_node(d, 0, i - 1)];
                dlyl = cord[d.N + gf_node(d, 0, i)] - cord[d.N + gf_node(d, 0, i - 1)];
            }
            if (i < nx - 1) {
                pr = rho_water_g * ((cord[d.N + gf_node(d, 0, i + 1)] + cord[d.N + gf_node(d, 0, i)]) / 2.0);
                dlxr = cord[gf_node(d, 0, i + 1)] - cord[gf_node(d, 0, i)];
                dlyr = cord[d.N + gf_node(d, 0, i + 1)] - cord[d.N + gf_node(d, 0, i)];
            }
            f0 = f0 - 0.5 * pl * dlyl - 0.5 * pr * dlyr;
            f1 = f1 + 0.5 * pl * dlxl + 0.5 * pr * dlxr;
        }
    }
    if (P.nyhydro > 0 && j == nz - 1) { // Winkler foundation
        int ips = P.iphsub - 1;
        double zb = cord[d.N + n];
        double p_est = P.pisos + 0.5 * (P.den[ips] + P.drosub) * P.g * (zb - P.rzbo);
        double rosubg = P.g * (P.den[ips] + P.drosub) * (1 - P.alfa[ips] * A.temp[n] + P.beta[ips] * p_est);
        double pl = 0, dlxl = 0, dlyl = 0, pr = 0, dlxr = 0, dlyr = 0;
        if (i > 0) {
            GF_IDX m = gf_node(d, nz - 1, i - 1);
            pl = P.pisos - rosubg * ((cord[d.N + m] + zb) / 2.0 - P.rzbo);
            dlxl = cord[n] - cord[m];
            dlyl = zb - cord[d.N + m];
        }
        if (i < nx - 1) {
            GF_IDX m = gf_node(d, nz - 1, i + 1);
            pr = P.pisos - rosubg * ((cord[d.N + m] + zb) / 2.0 - P.rzbo);
            dlxr = cord[m] - cord[n];
            dlyr = cord[d.N + m] - zb;
        }
        f0 = f0 - 0.5 * pl * dlyl - 0.5 * pr * dlyr;
        f1 = f1 + 0.5 * pl * dlxl + 0.5 * pr * dlxr;
    }
    double dt = C->dt;
    double drat = gf_ddiv(dt, C->dt_elastic); // (divisions off the FP64 pipe: gf_ddiv)
    if (drat < 1.0) drat = 1.0;
    double *vel = A.vel;
    double v0 = vel[n], v1 = vel[d.N + n];
    int c0 = A.ncod[n], c1 = A.ncod[d.N + n];
    // (the products and the |v| > 1e-13 tests on the integer pipes: gf_mul,
    // gf_abs_gt)
    if ((c0 & 1) != 1 && gf_abs_gt(v0, 1.0e-13)) f0 = f0 - gf_mul(P.demf, copysign(fabs(f0), v0));
    if ((c1 & 2) != 2 && gf_abs_gt(v1, 1.0e-13)) f1 = f1 - gf_mul(P.demf, copysign(fabs(f1), v1));
    double am = A.amass[n];
    if (sizeof(R) == sizeof(float)) {
        // FP32 increment on the FP64 velocity
        float s = gf_d2f(dt) / (gf_d2f(am) * gf_d2f(drat) * gf_d2f(drat));
        v0 = (c0 == 1) ? A.bc[n] : v0 + gf_f2d(s * gf_d2f(f0));
        v1 = (c1 == 1) ? A.bc[d.N + n] : v1 + gf_f2d(s * gf_d2f(f1));
    } else {
        const double den = gf_mul(gf_mul(am, drat), drat);
        v0 = (c0 == 1) ? A.bc[n] : v0 + gf_ddiv(gf_mul(dt, f0), den);
        v1 = (c1 == 1) ? A.bc[d.N + n] : v1 + gf_ddiv(gf_mul(dt, f1), den);
    }
    if (P.i_prestress == 1 && C->time < 600e3 * GF_SEC_YEAR) {
        if (j == nz - 1 || i == 0 || i == nx - 1) {
            v0 = 0.0;
            v1 = 0.0;
        }
    }
    vel[n] = v0;
    vel[d.N + n] = v1;
    if (sizeof(R) == sizeof(float)) {
        float h0, l0, h1, l1;
        gf_split(v0, h0, l0);
        gf_split(v1, h1, l1);
        A.vel_hi[n] = h0;
        A.vel_lo[n] = l0;
        A.vel_hi[d.N + n] = h1;
        A.vel_lo[d.N + n] = l1;
    }
}
template <class R> __global__ void __launch_bounds__(GF_THREADS) k_node(const DevParams *__restrict__ Pp, DevClock *__restrict__ C, DevArrays A, GfDims d, int terms) {
    gf_pdl_entry();
    b_k_node<R>(Pp, C, A, d, (GF_IDX)blockIdx.x * blockDim.x + threadIdx.x, terms);
}

// ======================================================================
// fl_move (fl_move.f90:3-132)
__device__ __forceinline__ void b_k_move_cord(DevClock *__restrict__ C, DevArrays A, GfDims d, GF_IDX n) {
    if (n >= 2 * d.N) return;
    const double c = A.cord[n] + A.vel[n] * C->dt;
    A.cord[n] = c;
    if (A.cord_hi) {
        float h, l;
        gf_split(c, h, l);
        A.cord_hi[n] = h;
        A.cord_lo[n] = l;
    }
}
__global__ void __launch_bounds__(GF_THREADS) k_move_cord(DevClock *__restrict__ C, DevArrays A, GfDims d) {
    gf_pdl_entry();
    b_k_move_cord(C, A, d, (GF_IDX)blockIdx.x * blockDim.x + threadIdx.x);
}

template <class R> __device__ __forceinline__ void b_k_move_elem(DevClock *__restrict__ C, DevArrays A, GfDims d, int advance_time, GF_IDX e) {
    if (e >= d.E) return;
    int j, i;
    elem_ji(d, e, j, i);
    const double dtd = C->dt;
    if (advance_time && e == 0) C->time = C->time + dtd; // par.f90:86, after every reader of time
    const bool fp32_path = sizeof(R) == sizeof(float);
    Quad q;
    QuadF qf;
    double xv[4], yv[4];
    float rvx[4], rvy[4];
    if (fp32_path) {
        load_quad_rel(A, d, j, i, qf);
        load_vel_rel(A, d, j, i, rvx, rvy);
    } else {
        load_quad(A.cord, d, j, i, q);
        GF_IDX n1 = gf_node(d, j, i), n3 = gf_node(d, j, i + 1);
        const double *vel = A.vel;
        xv[0] = vel[n1]; xv[1] = vel[n1 + 1]; xv[2] = vel[n3]; xv[3] = vel[n3 + 1];
        yv[0] = vel[d.N + n1]; yv[1] = vel[d.N + n1 + 1]; yv[2] = vel[d.N + n3]; yv[3] = vel[d.N + n3 + 1];
    }
    R *area = (R *)A.area;
    R *dvol = (R *)A.dvol;
    R *st = (R *)A.stress0;
    R *strain = (R *)A.strain;
    const int nd1[4] = {0, 2, 0, 0}, nd2[4] = {1, 1, 1, 3}, nd3[4] = {2, 3, 3, 2};
    bool neg = false;
    const bool fp32 = sizeof(R) == sizeof(float);
    // the surface nodes also moved by diff_topo's dtopo (zero without it)
    float tz[4] = {0.0f, 0.0f, 0.0f, 0.0f};
    if (fp32 && j == 0) {
        tz[0] = gf_d2f(A.dtopo[i]);
        tz[2] = gf_d2f(A.dtopo[i + 1]);
    }
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        int a = nd1[k], b = nd2[k], c = nd3[k];
        const double *xc = q.x, *yc = q.y;
        R ar_old = area[gf_ek(d, e, k)];
        R dw12, ar_new;
        if (!fp32) {
            // fl_move.f90:70-90 with the reference's operations
            // (products on the integer pipes: gf_mul, the bits of the FP64
            // multiply, which this FP64-bound kernel has few enough of)
            double det = ((gf_mul(xc[b], yc[c]) - gf_mul(yc[b], xc[c])) - (gf_mul(xc[a], yc[c]) - gf_mul(yc[a], xc[c]))) +
                         (gf_mul(xc[a], yc[b]) - gf_mul(yc[a], xc[b]));
            dvol[gf_ek(d, e, k)] = R(gf_mul(det, (double)ar_old) - 1.0);
            const double rdet = gf_rcp(det); // RN(1/det) off the FP64 pipe
            ar_new = R(rdet);
            // the rotation's quotient by det (gf_ddiv: the bits of the division)
            double dw = gf_mul(gf_ddiv(gf_scale<-1>(gf_mul(xv[a], xc[c] - xc[b]) + gf_mul(xv[b], xc[a] - xc[c]) +
                                                    gf_mul(xv[c], xc[b] - xc[a]) + gf_mul(yv[a], yc[c] - yc[b]) +
                                                    gf_mul(yv[b], yc[a] - yc[c]) + gf_mul(yv[c], yc[b] - yc[a])),
                                       det),
                               dtd);
            dw12 = R(dw);
        } else {
            // FP32 from edge vectors of the relative coordinates: det = B x C
            // with B = b - a, C = c - a.  dvol = det_new*area_old - 1 is taken
            // as (det_new - det_old)*area_old with the change of det expanded
            // in this step's displacements u = vel*dt, which FP32 resolves.
            const float *x = qf.x, *y = qf.y;
            const float dtf = gf_d2f(dtd);
            float Bx = x[b] - x[a], By = y[b] - y[a];
            float Cx = x[c] - x[a], Cy = y[c] - y[a];
            float dBx = (rvx[b] - rvx[a]) * dtf, dBy = (rvy[b] - rvy[a]) * dtf + (tz[b] - tz[a]);
            float dCx = (rvx[c] - rvx[a]) * dtf, dCy = (rvy[c] - rvy[a]) * dtf + (tz[c] - tz[a]);
            float Box = Bx - dBx, Boy = By - dBy, Cox = Cx - dCx, Coy = Cy - dCy;
            float ddet = (Box * dCy - Boy * dCx) + (dBx * Coy - dBy * Cox) + (dBx * dCy - dBy * dCx);
            float det = Bx * Cy - By * Cx;
            dvol[gf_ek(d, e, k)] = R(ddet * (float)ar_old);
            ar_new = R(1.0f / det);
            // 0.5 * curl of the velocity over the triangle, times dt
            float wx = rvx[a] * (x[c] - x[b]) + rvx[b] * (x[a] - x[c]) + rvx[c] * (x[b] - x[a]);
            float wy = rvy[a] * (y[c] - y[b]) + rvy[b] * (y[a] - y[c]) + rvy[c] * (y[b] - y[a]);
            dw12 = R(0.5f * (wx + wy) / det * dtf);
        }
        area[gf_ek(d, e, k)] = ar_new;
        neg |= !(ar_new > R(0));
        R s11 = st[gf_s(d, e, 0, k)], s22 = st[gf_s(d, e, 1, k)], s12 = st[gf_s(d, e, 2, k)];
        st[gf_s(d, e, 0, k)] = s11 + gf_mul(gf_scale<1>(s12), dw12);
        st[gf_s(d, e, 1, k)] = s22 - gf_mul(gf_scale<1>(s12), dw12);
        st[gf_s(d, e, 2, k)] = s12 + gf_mul(dw12, s22 - s11);
        if (k == 0) {
            R e11 = strain[gf_ek(d, e, 0)], e22 = strain[gf_ek(d, e, 1)], e12 = strain[gf_ek(d, e, 2)];
            strain[gf_ek(d, e, 0)] = e11 + gf_mul(gf_scale<1>(e12), dw12);
            strain[gf_ek(d, e, 1)] = e22 - gf_mul(gf_scale<1>(e12), dw12);
            strain[gf_ek(d, e, 2)] = e12 + gf_mul(dw12, e22 - e11);
        }
    }
    if (neg) set_status(C, 40, (int)e);
}
template <class R> __global__ void __launch_bounds__(GF_THREADS) k_move_elem(DevClock *__restrict__ C, DevArrays A, GfDims d, int advance_time) {
    gf_pdl_entry();
    b_k_move_elem<R>(C, A, d, advance_time, (GF_IDX)blockIdx.x * blockDim.x + threadIdx.x);
}

// ======================================================================
// fl_therm (fl_therm.f90:393-598).
//
// The reference updates temp in place, i outer and j inner: node (j,i) reads
// new values at its upstream neighbours (j-1,i), (j,i-1), (j+1,i-1) and old
// values at itself and downstream.  Its result is the unique fixed point of
//   Tnew(n) = f_n(Tnew(upstream), Told(rest))
// with f_n the reference's floating-point expression.  The system is lower
// triangular, so iterating Jacobi-style sweeps of f_n from Told reaches that
// fixed point exactly (bit for bit) after finitely many sweeps; each sweep
// contracts the distance by ~kappa*dt/h^2, so a handful of sweeps suffice.
// A sweep that changes no value proves convergence; later sweeps exit at once.
//
// k_therm_prep computes, per element, everything of the triangles A and B that
// does not depend on temperature (fl_therm.f90:424-567): the shape-derivative
// products K_ab, real_area13 = (1/area)/6, 0.5*diff/area and
// src*real_area13, each with the reference's operations.

#define GF_TC 18 // doubles per element: KA[6], KB[6], raA, raB, preA, preB, srA, srB
// K index of (a,b), a,b in 0..2 (symmetric)
__device__ __forceinline__ int kidx(int a, int b) {
    int lo = a < b ? a : b, hi = a < b ? b : a;
    return lo == 0 ? hi : (lo == 1 ? 2 + hi : 5);
}

template <class R> __device__ __forceinline__ void b_k_therm_prep(const DevParams *__restrict__ Pp, DevClock *__restrict__ C, DevArrays A, GfDims d, double *__restrict__ tc, GF_IDX e) {
    if (e == 0)
        for (int k = 0; k < GF_THERM_KMAX; ++k) C->therm_flags[k] = 0; // before any sweep runs
    if (e >= d.E) return;
    const DevParams &P = *Pp;
    int j, i;
    elem_ji(d, e, j, i);
    int iph = A.iphase[e] - 1;
    double cp_eff = P.cp[iph];
    double dissip = (P.ishearh == 1 && P.itherm != 2) ? (double)((const R *)A.shrheat)[e] : 0.0;
    // conduct / den / cp of the phase: the same two IEEE divisions as the
    // reference's cond_eff / dens / cp_eff, taken once per phase at set-up
    double diff = P.diffu[iph];
    // the source's quotients by den and cp (gf_ddiv: the bits of the IEEE
    // divisions, off the FP64 pipe)
    double src = gf_ddiv(A.source[e] + gf_ddiv(dissip, P.den[iph]), cp_eff);
    Quad q;
    load_quad(A.cord, d, j, i, q);
    const R *area = (const R *)A.area;
    const GF_IDX E = d.E;
    // triangle A: local vertices (q1,q2,q3); triangle B: (q3,q2,q4)
    const int tv[2][3] = {{0, 1, 2}, {2, 1, 3}};
#pragma unroll
    for (int t = 0; t < 2; ++t) {
        double a = (double)area[gf_ek(d, e, t)];
        double y1 = q.y[tv[t][0]], y2 = q.y[tv[t][1]], y3 = q.y[tv[t][2]];
        double x1 = q.x[tv[t][0]], x2 = q.x[tv[t][1]], x3 = q.x[tv[t][2]];
        // (products on the integer pipes: gf_mul, the bits of the FP64
        // multiply, which this FP64-bound kernel has few enough of)
        double dd[3] = {gf_mul(y2 - y3, a), gf_mul(y3 - y1, a), gf_mul(y1 - y2, a)};
        double zz[3] = {gf_mul(x3 - x2, a), gf_mul(x1 - x3, a), gf_mul(x2 - x1, a)};
#pragma unroll
        for (int m = 0; m < 3; ++m)
#pragma unroll
            for (int n = m; n < 3; ++n) tc[(t * 6 + kidx(m, n)) * E + e] = gf_mul(dd[m], dd[n]) + gf_mul(zz[m], zz[n]);
        double inv_area = gf_rcp(a); // RN(1/a) off the FP64 pipe
        double ra = gf_ddiv(inv_area, 6.0);
        tc[(12 + t) * E + e] = ra;
        tc[(14 + t) * E + e] = gf_mul(gf_scale<-1>(diff), inv_area);
        tc[(16 + t) * E + e] = gf_mul(src, ra);
    }
}
template <class R> __global__ void __launch_bounds__(GF_THREADS) k_therm_prep(const DevParams *__restrict__ Pp, DevClock *__restrict__ C, DevArrays A, GfDims d, double *__restrict__ tc) {
    gf_pdl_entry();
    b_k_therm_prep<R>(Pp, C, A, d, tc, (GF_IDX)blockIdx.x * blockDim.x + threadIdx.x);
}

// Temperature after the boundary conditions of fl_therm.f90:573-598 (top
// row t_top, bottom row bot_bc or the flux condition, then the side columns
// copied from their inner neighbours), read from the swept values `src`.
template <class Src>
__device__ __forceinline__ double therm_bc_value(const DevParams &P, const DevArrays &A, const GfDims &d, Src src, int j,
                                                 int i) {
    const int nx = d.nx, nz = d.nz;
    int ii = (i == 0 || nx == 2) ? 1 : (i == nx - 1 ? nx - 2 : i);
    if (j == 0) return P.t_top;
    if (j == nz - 1) {
        if (P.itemp_bc == 1) return P.bot_bc;
        if (P.itemp_bc == 2) {
            int ie = ii < nx - 2 ? ii : nx - 2;
            double cond_eff = P.conduct[A.iphase[gf_elem(d, nz - 2, ie)] - 1];
            return src(gf_node(d, nz - 2, ii)) +
                   P.bot_bc * (A.cord[d.N + gf_node(d, nz - 2, ii)] - A.cord[d.N + gf_node(d, nz - 1, ii)]) / cond_eff;
        }
    }
    return src(gf_node(d, j, ii));
}

// One node of sweep k.  Tup holds the current iterate; the start (the
// iterate before sweep 0) is Told + the previous step's increment
// (A.t_pred), a guess: the fixed point does not depend on it, only how many
// nodes the sweeps recompute before they reach it (on the 1000x300 model
// sweep 2 recomputes 16 % of the nodes instead of 82 %).  Self and
// downstream values always come from Told (A.temp).  Returns whether the
// node's value changed.  The iterates and the change flags are written by
// other CTAs of the same (persistent) launch, so their loads bypass L1
// (__ldcg).
__device__ __forceinline__ bool therm_sweep_node(DevArrays A, GfDims d, double dt, const double *__restrict__ tc,
                                                 const double *Tup, double *Tout, int k, GF_IDX n) {
    int j, i;
    node_ji(d, n, j, i);
    // A node's sweep-k value depends on sweep k-1 only through its upstream
    // neighbours (j-1,i), (j,i-1), (j+1,i-1); if none of them changed in
    // sweep k-1 its value is the one it had (the same inputs give the same
    // result), and the FP64 evaluation is skipped.
    if (k > 0) {
        const uint8_t *prev = A.t_chg + (GF_IDX)((k - 1) & 1) * d.N;
        bool recompute = (j != 0 && __ldcg(prev + gf_node(d, j - 1, i))) ||
                         (i != 0 && __ldcg(prev + gf_node(d, j, i - 1))) ||
                         (i != 0 && j != d.nz - 1 && __ldcg(prev + gf_node(d, j + 1, i - 1)));
        if (!recompute) {
            Tout[n] = __ldcg(Tup + n);
            return false;
        }
    }
    const int nx = d.nx, nz = d.nz;
    const GF_IDX E = d.E;
    const double *T = A.temp;
    double rhs = 0.0, area_n = 0.0;
    auto Nd = [&](int jj, int ii) { return gf_node(d, jj, ii); };
    const double *pred = A.t_pred;
    auto start = [&](GF_IDX m) { return T[m] + pred[m]; };
    auto U = [&](int jj, int ii) { return k == 0 ? start(Nd(jj, ii)) : __ldcg(Tup + Nd(jj, ii)); };
    // triangle t of element e; vs = local index of the updated node; the
    // three (local vertex, temperature) terms in the reference's order
    // (products on the integer pipes: gf_mul, the bits of the FP64 multiply;
    // the first sweeps are bound by the FP64 pipe)
    auto tri = [&](GF_IDX e, int t, int vs, int v0, double T0, int v1, double T1, int v2, double T2) {
        double ra = tc[(12 + t) * E + e];
        area_n = area_n + ra;
        const double *K = tc + (GF_IDX)t * 6 * E + e;
        rhs = rhs + tc[(16 + t) * E + e] -
              gf_mul(tc[(14 + t) * E + e], gf_mul(T0, K[kidx(v0, vs) * E]) + gf_mul(T1, K[kidx(v1, vs) * E]) +
                                               gf_mul(T2, K[kidx(v2, vs) * E]));
    };
    double Ts = T[n];
    if (j != 0 && i != 0) // element (j-1,i-1), triangle B: vertices (j-1,i), (j,i-1), node
        tri(gf_elem(d, j - 1, i - 1), 1, 2, 0, U(j - 1, i), 1, U(j, i - 1), 2, Ts);
    if (j != 0 && i != nx - 1) { // element (j-1,i), triangles A and B
        GF_IDX e = gf_elem(d, j - 1, i);
        tri(e, 0, 1, 0, U(j - 1, i), 1, Ts, 2, T[Nd(j - 1, i + 1)]);
        tri(e, 1, 1, 0, T[Nd(j - 1, i + 1)], 1, Ts, 2, T[Nd(j, i + 1)]);
    }
    if (j != nz - 1 && i != 0) { // element (j,i-1), triangles A and B
        GF_IDX e = gf_elem(d, j, i - 1);
        tri(e, 0, 2, 0, U(j, i - 1), 1, U(j + 1, i - 1), 2, Ts);
        tri(e, 1, 0, 0, Ts, 1, U(j + 1, i - 1), 2, T[Nd(j + 1, i)]);
    }
    if (j != nz - 1 && i != nx - 1) // element (j,i), triangle A
        tri(gf_elem(d, j, i), 0, 0, 0, Ts, 1, T[Nd(j + 1, i)], 2, T[Nd(j, i + 1)]);
    double tn = Ts + gf_ddiv(gf_mul(rhs, dt), area_n);
    Tout[n] = tn;
    return !gf_deq(tn, k == 0 ? start(n) : __ldcg(Tup + n));
}

// Bounded grid barrier of a co-resident (cooperative) launch: generation
// counter in bar[1], arrivals in bar[0], error flag in bar[2].  A CTA that
// waits longer than `limit` polls sets the flag; every CTA returns false
// once the flag is set.
__device__ bool gf_grid_barrier(unsigned *bar, GF_IDX limit) {
    __shared__ int bad;
    __syncthreads();
    if (threadIdx.x == 0) {
        volatile unsigned *vgen = bar + 1;
        unsigned g0 = *vgen;
        __threadfence();
        unsigned arrived = atomicAdd(bar, 1u);
        if (arrived == gridDim.x - 1) {
            atomicExch(bar, 0u);
            __threadfence();
            atomicAdd(bar + 1, 1u);
        } else {
            GF_IDX it = 0;
            while (*vgen == g0) {
                if (++it > limit) {
                    atomicExch(bar + 2, 1u);
                    break;
                }
                __nanosleep(64);
            }
        }
        __threadfence();
        bad = *(volatile unsigned *)(bar + 2) != 0u;
    }
    __syncthreads();
    return !bad;
}

// The FP64 thermal update after k_therm_prep, in one co-resident launch:
// sweeps until one changes nothing (at most kmax; grid barrier between
// sweeps, every CTA reads the same flag after it), then the boundary
// conditions and temp0 = temp (fl_therm.f90:53, 577-598) from the last
// sweep's buffer.  Node n is always handled by the same thread.
__global__ void __launch_bounds__(GF_THREADS) k_therm_sweeps(const DevParams *__restrict__ Pp, DevClock *__restrict__ C,
                                                            DevArrays A, GfDims d, const double *__restrict__ tc,
                                                            double *b0, double *b1, int kmax, int keep_temp0,
                                                            unsigned *bar) {
    const GF_IDX stride = (GF_IDX)gridDim.x * blockDim.x; // a multiple of 32
    const GF_IDX gt = (GF_IDX)blockIdx.x * blockDim.x + threadIdx.x;
    const GF_IDX npad = (d.N + 31) / 32 * 32; // equal trip counts within a warp (the vote)
    const double dt = C->dt;
    int kc = kmax; // the first sweep that changed nothing
    for (int k = 0; k < kmax; ++k) {
        const double *up = k == 0 ? A.temp : ((k - 1) & 1 ? b1 : b0);
        double *out = (k & 1) ? b1 : b0;
        bool any = false;
        for (GF_IDX n = gt; n < npad; n += stride) {
            bool changed = n < d.N && therm_sweep_node(A, d, dt, tc, up, out, k, n);
            if (n < d.N) A.t_chg[(GF_IDX)(k & 1) * d.N + n] = changed ? 1 : 0;
            any = any || changed;
        }
        if (__any_sync(0xffffffffu, any) && (threadIdx.x & 31) == 0) C->therm_flags[k] = 1;
        if (!gf_grid_barrier(bar, 1LL << 24)) {
            if (gt == 0) set_status(C, GF_ERR_TIMEOUT, k);
            return;
        }
        if (*(volatile int *)&C->therm_flags[k] == 0) {
            kc = k;
            break;
        }
    }
    if (gt == 0) {
        C->therm_sweeps_used = kc + 1;
        if (kc == kmax) C->therm_unconverged += 1;
    }
    const double *src = ((kc < kmax ? kc : kmax - 1) & 1) ? b1 : b0;
    for (GF_IDX n = gt; n < d.N; n += stride) {
        int j, i;
        node_ji(d, n, j, i);
        double t = therm_bc_value(*Pp, A, d, [src](GF_IDX m) { return __ldcg(src + m); }, j, i);
        const double told = A.temp[n];
        if (!keep_temp0) A.temp0[n] = told;
        A.temp[n] = t;
        A.t_pred[n] = t - told; // the next step's start: its Told + this increment
    }
}

// ---- mixed precision: FP32 coefficients, two sweeps.
// The diffusion sum is taken over temperature differences to the updated
// node (the rows of the triangle stiffness sum to zero), so FP32 keeps the
// accuracy that a sum of ~1000 C values would lose.  Sweep 0 is the all-old
// (Jacobi) update, sweep 1 reuses the upstream increments of sweep 0, which
// leaves an error of order (kappa dt/h^2)^2 relative to the increment.
__device__ __forceinline__ void b_k_therm_prep32(const DevParams *__restrict__ Pp, DevArrays A, GfDims d, float *__restrict__ tc, GF_IDX e) {
    if (e >= d.E) return;
    const DevParams &P = *Pp;
    int j, i;
    elem_ji(d, e, j, i);
    int iph = A.iphase[e] - 1;
    float cp_eff = P.f_cp[iph], cond_eff = P.f_cond[iph], den = P.f_den[iph];
    float dissip = (P.ishearh == 1 && P.itherm != 2) ? ((const float *)A.shrheat)[e] : 0.0f;
    float diff = cond_eff / den / cp_eff;
    float src = (gf_d2f(A.source[e]) + dissip / den) / cp_eff;
    QuadF q;
    load_quad_rel(A, d, j, i, q);
    const float *area = (const float *)A.area;
    const GF_IDX E = d.E;
    const int tv[2][3] = {{0, 1, 2}, {2, 1, 3}};
#pragma unroll
    for (int t = 0; t < 2; ++t) {
        float a = area[gf_ek(d, e, t)];
        const int v1 = tv[t][0], v2 = tv[t][1], v3 = tv[t][2];
        float dd[3] = {(q.y[v2] - q.y[v3]) * a, (q.y[v3] - q.y[v1]) * a, (q.y[v1] - q.y[v2]) * a};
        float zz[3] = {(q.x[v3] - q.x[v2]) * a, (q.x[v1] - q.x[v3]) * a, (q.x[v2] - q.x[v1]) * a};
#pragma unroll
        for (int m = 0; m < 3; ++m)
#pragma unroll
            for (int n = m; n < 3; ++n) tc[(t * 6 + kidx(m, n)) * E + e] = dd[m] * dd[n] + zz[m] * zz[n];
        float inv_area = 1.0f / a;
        float ra = inv_area / 6.0f;
        tc[(12 + t) * E + e] = ra;
        tc[(14 + t) * E + e] = 0.5f * diff * inv_area;
        tc[(16 + t) * E + e] = src * ra;
    }
}
__global__ void __launch_bounds__(GF_THREADS) k_therm_prep32(const DevParams *__restrict__ Pp, DevArrays A, GfDims d, float *__restrict__ tc) {
    gf_pdl_entry();
    b_k_therm_prep32(Pp, A, d, tc, (GF_IDX)blockIdx.x * blockDim.x + threadIdx.x);
}

// sweep 0 (final = 0): dT0 = increment with old values; sweep 1 (final = 1):
// upstream neighbours use T + dT0, and tnew = T + dT1 (FP64) is written.
// The temperature differences come from the hi/lo FP32 split of T.
__device__ __forceinline__ void b_k_therm_sweep32(const DevParams *__restrict__ Pp, DevClock *__restrict__ C, DevArrays A, GfDims d, const float *__restrict__ tc, float *__restrict__ d0, double *__restrict__ tnew, int final_sweep, GF_IDX n) {
    if (n >= d.N) return;
    int j, i;
    node_ji(d, n, j, i);
    const int nx = d.nx, nz = d.nz;
    const GF_IDX E = d.E;
    const float *th = A.temp_hi, *tl = A.temp_lo;
    float rhs = 0.0f, area_n = 0.0f;
    auto Nd = [&](int jj, int ii) { return gf_node(d, jj, ii); };
    // temperature difference to the updated node; upstream nodes carry the
    // increment of sweep 0 in the final sweep
    auto dT = [&](GF_IDX m, bool up) {
        float v = hl_diff(th, tl, m, n);
        if (up && final_sweep) v += d0[m];
        return v;
    };
    auto tri = [&](GF_IDX e, int t, int vs, int v0, float D0, int v1, float D1, int v2, float D2) {
        float ra = tc[(12 + t) * E + e];
        area_n += ra;
        const float *K = tc + (GF_IDX)t * 6 * E + e;
        rhs += tc[(16 + t) * E + e] - tc[(14 + t) * E + e] * (D0 * K[kidx(v0, vs) * E] + D1 * K[kidx(v1, vs) * E] +
                                                           D2 * K[kidx(v2, vs) * E]);
    };
    if (j != 0 && i != 0)
        tri(gf_elem(d, j - 1, i - 1), 1, 2, 0, dT(Nd(j - 1, i), true), 1, dT(Nd(j, i - 1), true), 2, 0.0f);
    if (j != 0 && i != nx - 1) {
        GF_IDX e = gf_elem(d, j - 1, i);
        tri(e, 0, 1, 0, dT(Nd(j - 1, i), true), 1, 0.0f, 2, dT(Nd(j - 1, i + 1), false));
        tri(e, 1, 1, 0, dT(Nd(j - 1, i + 1), false), 1, 0.0f, 2, dT(Nd(j, i + 1), false));
    }
    if (j != nz - 1 && i != 0) {
        GF_IDX e = gf_elem(d, j, i - 1);
        tri(e, 0, 2, 0, dT(Nd(j, i - 1), true), 1, dT(Nd(j + 1, i - 1), true), 2, 0.0f);
        tri(e, 1, 0, 0, 0.0f, 1, dT(Nd(j + 1, i - 1), true), 2, dT(Nd(j + 1, i), false));
    }
    if (j != nz - 1 && i != nx - 1)
        tri(gf_elem(d, j, i), 0, 0, 0, 0.0f, 1, dT(Nd(j + 1, i), false), 2, dT(Nd(j, i + 1), false));
    float inc = rhs * gf_d2f(C->dt) / area_n;
    if (!final_sweep)
        d0[n] = inc;
    else
        tnew[n] = A.temp[n] + gf_f2d(inc);
}
__global__ void __launch_bounds__(GF_THREADS) k_therm_sweep32(const DevParams *__restrict__ Pp, DevClock *__restrict__ C, DevArrays A, GfDims d, const float *__restrict__ tc, float *__restrict__ d0, double *__restrict__ tnew, int final_sweep) {
    gf_pdl_entry();
    b_k_therm_sweep32(Pp, C, A, d, tc, d0, tnew, final_sweep, (GF_IDX)blockIdx.x * blockDim.x + threadIdx.x);
}

// temp0 = temp; temp = tnew with the boundary conditions (which read tnew
// at neighbours, never the temp being overwritten), and its split
__device__ __forceinline__ void b_k_therm_apply32(const DevParams *__restrict__ Pp, DevArrays A, GfDims d, const double *__restrict__ tnew, GF_IDX n) {
    if (n >= d.N) return;
    int j, i;
    node_ji(d, n, j, i);
    const double t = therm_bc_value(*Pp, A, d, [tnew](GF_IDX m) { return tnew[m]; }, j, i);
    A.temp0[n] = A.temp[n];
    A.temp[n] = t;
    float h, l;
    gf_split(t, h, l);
    A.temp_hi[n] = h;
    A.temp_lo[n] = l;
}
__global__ void __launch_bounds__(GF_THREADS) k_therm_apply32(const DevParams *__restrict__ Pp, DevArrays A, GfDims d, const double *__restrict__ tnew) {
    gf_pdl_entry();
    b_k_therm_apply32(Pp, A, d, tnew, (GF_IDX)blockIdx.x * blockDim.x + threadIdx.x);
}

// ======================================================================
// rmasses (rmasses.f90:4-63): per-element density, then a node gather in
// the reference's colour order with each element's triangles in order.
template <class R> __device__ __forceinline__ void b_k_elem_dens(const DevParams *__restrict__ Pp, DevClock *__restrict__ C, DevArrays A, GfDims d, GF_IDX e) {
    if (e >= d.E) return;
    int j, i;
    elem_ji(d, e, j, i);
    int wrote = 0;
    const R *area = (const R *)A.area;
    if constexpr (sizeof(R) == sizeof(float)) {
        // mixed: FP32 density and FP32 triangle shares
        float fval = 0.0f;
        const float dens = eff_dens_f32(*Pp, A, d, j, i, e, &wrote, &fval);
        A.e_dens[e] = gf_f2d(dens);
        float *tri = (float *)A.e_tri;
#pragma unroll
        for (int k = 0; k < 4; ++k) tri[k * d.E + e] = (1.0f / 12.0f) / area[gf_ek(d, e, k)] * dens;
    } else {
        double fval = 0.0;
        double dens = eff_dens<R>(*Pp, A, d, j, i, e, &wrote, &fval);
        A.e_dens[e] = dens;
        // each triangle's share c1d12/area*dens (rmasses.f90:35-57),
        // computed once here with the reference's operations and gathered
        // per node
        const double c1d12 = 1.0 / 12.0;
#pragma unroll
        for (int k = 0; k < 4; ++k) A.e_tri[k * d.E + e] = c1d12 / (double)area[gf_ek(d, e, k)] * dens;
    }
    if (wrote) {
        // serial position of this element in the coloured sweep
        int ib = i & 1, jb = j & 1;
        GF_IDX ci = (GF_IDX)(d.nx - 1 - ib + 1) / 2; // columns of this colour
        GF_IDX cj = (GF_IDX)(d.nz - 1 - jb + 1) / 2;
        GF_IDX before = 0;
        for (int b = 0; b < ib * 2 + jb; ++b) {
            int bi = b >> 1, bj = b & 1;
            before += (GF_IDX)((d.nx - 1 - bi + 1) / 2) * ((d.nz - 1 - bj + 1) / 2);
        }
        GF_IDX pos = before + (GF_IDX)(i >> 1) * cj + (j >> 1);
        (void)ci;
        atomicMax((unsigned long long *)&C->frac_writer, (unsigned long long)(pos + 1));
    }
}
template <class R> __global__ void __launch_bounds__(GF_THREADS) k_elem_dens(const DevParams *__restrict__ Pp, DevClock *__restrict__ C, DevArrays A, GfDims d) {
    gf_pdl_entry();
    b_k_elem_dens<R>(Pp, C, A, d, (GF_IDX)blockIdx.x * blockDim.x + threadIdx.x);
}

template <class R> __device__ __forceinline__ void b_k_frac_fix(const DevParams *__restrict__ Pp, DevClock *__restrict__ C, DevArrays A, GfDims d) {
    long long w = C->frac_writer;
    if (w <= 0) return;
    GF_IDX pos = w - 1;
    for (int b = 0; b < 4; ++b) {
        int bi = b >> 1, bj = b & 1;
        GF_IDX ci = (d.nx - 1 - bi + 1) / 2, cj = (d.nz - 1 - bj + 1) / 2;
        if (pos < ci * cj) {
            int i = (int)(pos / cj) * 2 + bi, j = (int)(pos % cj) * 2 + bj;
            int wrote = 0;
            double f = 0.0;
            eff_dens<R>(*Pp, A, d, j, i, gf_elem(d, j, i), &wrote, &f);
            if (wrote) C->frac = f;
            break;
        }
        pos -= ci * cj;
    }
    C->frac_writer = 0;
}
template <class R> __global__ void k_frac_fix(const DevParams *__restrict__ Pp, DevClock *__restrict__ C, DevArrays A, GfDims d) {
    b_k_frac_fix<R>(Pp, C, A, d);
}

// Contribution lists: for local vertex v of a quad (1:(j,i) 2:(j+1,i)
// 3:(j,i+1) 4:(j+1,i+1)), the triangles that contain it, in order.
__device__ __constant__ int c_vtx_tris[4][3] = {{0, 2, 3}, {0, 1, 2}, {0, 1, 3}, {1, 2, 3}};

// Node gather of per-triangle shares tri[k*E + e] in the reference's order:
// adjacent elements by colour ((ie&1)*2 + (je&1), rmasses.f90:25-30,
// dt_mass.f90:74-81), then each element's triangles containing the node in
// the order A, B, C, D.  Every element in a node's neighbourhood has a
// different colour, so this is the serial order of the coloured scatter.
// T = double: FP64 shares summed in the reference's order; T = float: the
// mixed path's FP32 shares
template <class T>
__device__ __forceinline__ void b_k_node_gather_tri(const T *__restrict__ tri, double *__restrict__ out, GfDims d, GF_IDX n) {
    if (n >= d.N) return;
    int j, i;
    node_ji(d, n, j, i);
    T acc = T(0);
    int ord[4];
    // the node is vertex 4 of quad (j-1,i-1), 2 of (j-1,i), 3 of (j,i-1), 1 of (j,i)
    int je_[4] = {j - 1, j - 1, j, j}, ie_[4] = {i - 1, i, i - 1, i}, lv[4] = {3, 1, 2, 0};
#pragma unroll
    for (int q = 0; q < 4; ++q) ord[q] = ((ie_[q] & 1) << 1) | (je_[q] & 1);
#pragma unroll
    for (int c = 0; c < 4; ++c)
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            if (ord[q] != c) continue;
            int je = je_[q], ie = ie_[q];
            if (je < 0 || ie < 0 || je > d.nz - 2 || ie > d.nx - 2) continue;
            GF_IDX e = gf_elem(d, je, ie);
#pragma unroll
            for (int t = 0; t < 3; ++t) acc = acc + tri[c_vtx_tris[lv[q]][t] * d.E + e];
        }
    if constexpr (sizeof(T) == sizeof(float)) out[n] = gf_f2d(acc);
    else out[n] = acc;
}
template <class T>
__global__ void __launch_bounds__(GF_THREADS) k_node_gather_tri(const T *__restrict__ tri, double *__restrict__ out, GfDims d) {
    gf_pdl_entry();
    b_k_node_gather_tri<T>(tri, out, d, (GF_IDX)blockIdx.x * blockDim.x + threadIdx.x);
}

// ======================================================================
// dt_mass (dt_mass.f90:16-232)
// The CTA's minimum edge measure, maximum |velocity|, maximum diffusivity
// and phase mask (each warp's already reduced in its lane 0) combined in
// shared memory, then one atomic per quantity and CTA (per-warp atomics on
// the same four words serialise).  min / max are exact in any order.  Every
// thread of the CTA calls it; `diffu` (mixed path) turns the phase mask into
// the maximum diffusivity, otherwise dmax is used.
__device__ __forceinline__ void dt_block_commit(DevClock *__restrict__ C, double dl, double vmax, double dmax,
                                                unsigned pm, const double *diffu, int nphase) {
    __shared__ unsigned long long s_dl[GF_THREADS_MAX / 32], s_v[GF_THREADS_MAX / 32], s_d[GF_THREADS_MAX / 32];
    __shared__ unsigned s_pm[GF_THREADS_MAX / 32];
    const int w = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
    if ((threadIdx.x & 31) == 0) {
        s_dl[w] = (unsigned long long)__double_as_longlong(dl);
        s_v[w] = (unsigned long long)__double_as_longlong(vmax);
        s_d[w] = (unsigned long long)__double_as_longlong(dmax);
        s_pm[w] = pm;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned long long a = s_dl[0], b = s_v[0], c = s_d[0];
        unsigned m = s_pm[0];
        for (int k = 1; k < nw; ++k) {
            a = min(a, s_dl[k]);
            b = max(b, s_v[k]);
            c = max(c, s_d[k]);
            m |= s_pm[k];
        }
        if (diffu) { // the largest diffusivity of the phases present (dt_mass.f90:130)
            double dm = 0.0;
            for (int k = 0; k < nphase; ++k)
                if (m & (1u << k)) dm = fmax(dm, diffu[k]);
            c = (unsigned long long)__double_as_longlong(dm);
        }
        atomicMin(&C->r_dlmin, a);
        atomicMax(&C->r_velmax, b);
        atomicMax(&C->r_diffmax, c);
        atomicOr(&C->phase_mask, m);
    }
    __syncthreads(); // the shared slots are free for the CTA's next item
}

template <class R> __device__ __forceinline__ void b_k_dt_reduce(const DevParams *__restrict__ Pp, DevClock *__restrict__ C, DevArrays A, GfDims d, GF_IDX t) {
    const DevParams &P = *Pp;
    double dl = 1e300, vmax = 0.0, dmax = 0.0;
    unsigned pm = 0;
    if constexpr (sizeof(R) == sizeof(float)) {
        // mixed: edge lengths and 1/(area*length) in FP32 from the hi/lo
        // coordinates, |vel| from the hi parts; the warp minima and maxima of
        // these FP32 values convert to FP64 exactly, and the minimum over
        // elements is taken on their FP64 values
        float df = 1e30f, vf = 0.0f;
        if (t < d.E) {
            GF_IDX e = t;
            int j, i;
            elem_ji(d, e, j, i);
            const float *area = (const float *)A.area;
            QuadF q;
            load_quad_rel(A, d, j, i, q);
            auto len = [&](int a, int b) {
                float ddx = q.x[a] - q.x[b], ddy = q.y[a] - q.y[b];
                return sqrtf(ddx * ddx + ddy * ddy);
            };
            float a0 = area[gf_ek(d, e, 0)], a1 = area[gf_ek(d, e, 1)], a2 = area[gf_ek(d, e, 2)],
                  a3 = area[gf_ek(d, e, 3)];
            float l;
            l = len(1, 0); df = fminf(df, 1.0f / (a0 * l)); df = fminf(df, 1.0f / (a2 * l));
            l = len(3, 1); df = fminf(df, 1.0f / (a1 * l)); df = fminf(df, 1.0f / (a2 * l));
            l = len(3, 2); df = fminf(df, 1.0f / (a1 * l)); df = fminf(df, 1.0f / (a3 * l));
            l = len(2, 0); df = fminf(df, 1.0f / (a0 * l)); df = fminf(df, 1.0f / (a3 * l));
            l = len(3, 0); df = fminf(df, 1.0f / (a2 * l)); df = fminf(df, 1.0f / (a3 * l));
            l = len(1, 2); df = fminf(df, 1.0f / (a0 * l)); df = fminf(df, 1.0f / (a1 * l));
            pm = 1u << (A.iphase[e] - 1);
        }
        if (t < d.N) vf = fmaxf(fabsf(A.vel_hi[t]), fabsf(A.vel_hi[d.N + t]));
        df = warp_min(df);
        vf = warp_max(vf);
        for (int o = 16; o > 0; o >>= 1) pm |= __shfl_xor_sync(0xffffffffu, pm, o);
        dt_block_commit(C, df < 1e30f ? gf_f2d(df) : 1e300, gf_f2d(vf), 0.0, pm, P.diffu, P.nphase);
        return;
    } else {
        if (t < d.E) {
            GF_IDX e = t;
            int j, i;
            elem_ji(d, e, j, i);
            const R *area = (const R *)A.area;
            Quad q;
            load_quad(A.cord, d, j, i, q);
            auto len = [&](int a, int b) {
                double ddx = q.x[a] - q.x[b], ddy = q.y[a] - q.y[b];
                return sqrt(ddx * ddx + ddy * ddy);
            };
            double a0 = (double)area[gf_ek(d, e, 0)], a1 = (double)area[gf_ek(d, e, 1)],
                   a2 = (double)area[gf_ek(d, e, 2)], a3 = (double)area[gf_ek(d, e, 3)];
            // the smallest of the twelve quotients 1/(area*length) of
            // dlmin_prop (dt_mass.f90:174-231) is the quotient of the largest
            // product: correctly rounded division is monotone, so
            // min fl(1/x_k) = fl(1/max x_k) exactly, for one division
            double l, xm = 0.0;
            l = len(1, 0); xm = fmax(xm, a0 * l); xm = fmax(xm, a2 * l);
            l = len(3, 1); xm = fmax(xm, a1 * l); xm = fmax(xm, a2 * l);
            l = len(3, 2); xm = fmax(xm, a1 * l); xm = fmax(xm, a3 * l);
            l = len(2, 0); xm = fmax(xm, a0 * l); xm = fmax(xm, a3 * l);
            l = len(3, 0); xm = fmax(xm, a2 * l); xm = fmax(xm, a3 * l);
            l = len(1, 2); xm = fmax(xm, a0 * l); xm = fmax(xm, a1 * l);
            dl = fmin(dl, 1.0 / xm);
            int iph = A.iphase[e] - 1;
            dmax = P.conduct[iph] / P.den[iph] / P.cp[iph];
            pm = 1u << iph;
        }
        if (t < d.N) vmax = fmax(fabs(A.vel[t]), fabs(A.vel[d.N + t]));
        dl = warp_min(dl);
        vmax = warp_max(vmax);
        dmax = warp_max(dmax);
        for (int o = 16; o > 0; o >>= 1) pm |= __shfl_xor_sync(0xffffffffu, pm, o);
        dt_block_commit(C, dl, vmax, dmax, pm, nullptr, 0);
    }
}
template <class R> __global__ void __launch_bounds__(GF_THREADS) k_dt_reduce(const DevParams *__restrict__ Pp, DevClock *__restrict__ C, DevArrays A, GfDims d) {
    gf_pdl_entry();
    b_k_dt_reduce<R>(Pp, C, A, d, (GF_IDX)blockIdx.x * blockDim.x + threadIdx.x);
}

__device__ __forceinline__ void b_k_dt_scalars(const DevParams *__restrict__ Pp, DevClock *__restrict__ C) {
    const DevParams &P = *Pp;
    double dlmin = fmin(1e28, __longlong_as_double((long long)C->r_dlmin));
    double vel_max = __longlong_as_double((long long)C->r_velmax);
    double diffmax = __longlong_as_double((long long)C->r_diffmax);
    C->dlmin = dlmin;
    C->vel_max = vel_max;
    if (P.idt_scale == 1)
        C->dt_elastic = P.dt_scale;
    else if (P.idt_scale == 2) {
        if (P.vbc == 0)
            C->dt_elastic = dlmin * C->frac * P.strain_inert / (1.0 / GF_SEC_YEAR / 100);
        else
            C->dt_elastic = dlmin * C->frac * P.strain_inert / P.vbc;
    }
    // min over elements of dlmin^2/diff == dlmin^2 / max(diff) (rounded
    // division is monotone in the divisor)
    double dtmax_therm = 1e28;
    if (diffmax > 0.0) dtmax_therm = fmin(dtmax_therm, dlmin * dlmin / diffmax);
    double dt_maxwell = 1e28;
    double dt_elastic = C->dt_elastic;
    unsigned pm = C->phase_mask;
    for (int k = 0; k < P.nphase; ++k) {
        if (!(pm & (1u << k))) continue;
        if (P.idt_scale == 0) {
            // dt_mass.f90:122-126: a running minimum that starts from the
            // previous dt_elastic
            double pwave = P.rl[k] + 0.6666 * P.rm[k];
            double dte = C->frac * dlmin * sqrt(P.den[k] / pwave);
            dt_elastic = fmin(dt_elastic, dte);
        }
        if (P.ivis_present == 1 && (P.irheol[k] == 3 || P.irheol[k] == 12) && P.rm[k] < 1e11) {
            double visc_cut = 1e10;
            double rmu = (P.v_min < visc_cut) ? P.rm[k] * P.v_min / visc_cut : P.rm[k];
            double dt_m = P.v_min / rmu * P.fracm;
            dt_maxwell = fmin(dt_m, dt_maxwell);
        }
    }
    C->dt_elastic = dt_elastic;
    C->dt_maxwell = dt_maxwell;
    C->dtmax_therm = dtmax_therm;
    C->dt = fmin(fmin(dt_elastic, dt_maxwell), dtmax_therm);
}
__global__ void k_dt_scalars(const DevParams *__restrict__ Pp, DevClock *__restrict__ C) {
    b_k_dt_scalars(Pp, C);
}

// inertial mass share of each triangle c1d12*rho_inert/area
// (dt_mass.f90:83-120), one element per thread
template <class R> __device__ __forceinline__ void b_k_elem_am3(const DevParams *__restrict__ Pp, DevClock *__restrict__ C, DevArrays A, GfDims d, GF_IDX e) {
    if (e >= d.E) return;
    const DevParams &P = *Pp;
    const R *area = (const R *)A.area;
    if constexpr (sizeof(R) == sizeof(float)) {
        // mixed: the inertial density in FP32 (pwave / vel_sound^2 ~ 1e21,
        // well inside the FP32 range), from FP32 copies of the inputs
        const int iph = A.iphase[e] - 1;
        const float pwave = gf_d2f(P.rl[iph]) + 0.6666f * P.f_rm[iph];
        const float vel_sound = gf_d2f(C->dlmin) * gf_d2f(C->frac) / gf_d2f(C->dt_elastic);
        float rho_inert = pwave / (vel_sound * vel_sound);
        const float vel_max = gf_d2f(C->vel_max);
        if (P.i_rey == 1 && vel_max > 0.0f) {
            const float rho_inert2 = (gf_d2f(P.xReyn) * gf_d2f(P.v_min)) / (vel_max * fabsf(gf_d2f(P.rzbo)));
            if (rho_inert > rho_inert2) rho_inert = rho_inert2;
        }
        const float r = rho_inert / 12.0f;
        float *tri = (float *)A.e_tri;
#pragma unroll
        for (int k = 0; k < 4; ++k) tri[k * d.E + e] = r / area[gf_ek(d, e, k)];
        return;
    }
    const double c1d12 = 1.0 / 12.0;
    double dlmin = C->dlmin, frac = C->frac, dt_elastic = C->dt_elastic, vel_max = C->vel_max;
    int iph = A.iphase[e] - 1;
    double pwave = P.rl[iph] + 0.6666 * P.rm[iph];
    double vel_sound = dlmin * frac / dt_elastic;
    double rho_inert = pwave / (vel_sound * vel_sound);
    if (P.i_rey == 1 && vel_max > 0.0) {
        double rho_inert2 = (P.xReyn * P.v_min) / (vel_max * fabs(P.rzbo));
        if (rho_inert > rho_inert2) rho_inert = rho_inert2;
    }
#pragma unroll
    for (int k = 0; k < 4; ++k) A.e_tri[k * d.E + e] = c1d12 * rho_inert / (double)area[gf_ek(d, e, k)];
}
template <class R> __global__ void __launch_bounds__(GF_THREADS) k_elem_am3(const DevParams *__restrict__ Pp, DevClock *__restrict__ C, DevArrays A, GfDims d) {
    gf_pdl_entry();
    b_k_elem_am3<R>(Pp, C, A, d, (GF_IDX)blockIdx.x * blockDim.x + threadIdx.x);
}

__device__ __forceinline__ void b_k_dt_reset(DevClock *C) {
    C->r_dlmin = (unsigned long long)__double_as_longlong(1e300);
    C->r_velmax = 0ull;
    C->r_diffmax = 0ull;
    C->phase_mask = 0u;
}
__global__ void k_dt_reset(DevClock *C) {
    b_k_dt_reset(C);
}

// ======================================================================
// init_visc
template <class R> __device__ __forceinline__ void b_k_init_visc(const DevParams *__restrict__ Pp, DevArrays A, GfDims d, GF_IDX e) {
    if (e >= d.E) return;
    int j, i;
    elem_ji(d, e, j, i);
    ((R *)A.visn)[e] = R(visc_of<R>(*Pp, A, d, j, i, e, (const R *)A.stress0));
}
template <class R> __global__ void __launch_bounds__(GF_THREADS) k_init_visc(const DevParams *__restrict__ Pp, DevArrays A, GfDims d) {
    gf_pdl_entry();
    b_k_init_visc<R>(Pp, A, d, (GF_IDX)blockIdx.x * blockDim.x + threadIdx.x);
}

// ======================================================================
// change_phase (change_phase.f90:35-262)
__device__ __forceinline__ void b_k_phase_markers(const DevParams *__restrict__ Pp, DevArrays A, GfDims d, int nmarkers, GF_IDX kk) {
    if (kk >= nmarkers) return;
    if (A.mark_dead[kk] == 0) return;
    const DevParams &P = *Pp;
    const int nz = d.nz;
    int n = A.mark_ntriag[kk];
    int k = (n - 1) % 2 + 1;
    int j = ((n - k) / 2) % (nz - 1);
    int i = (n - k) / 2 / (nz - 1);
    // Exclusions that change no output, ahead of the FP64 evaluation: a
    // phase without a rule, and a marker certainly deeper than its rule
    // reaches (below 200 km; 150 km for mantle phases 4 and 8).  The marker
    // lies in its triangle, so its depth is at least the surface height less
    // the highest corner; FP32 copies of those heights err by under 0.1 m
    // and the test keeps a 10 m margin.
    {
        const int ph = A.mark_phase[kk];
        if (!(ph == 4 || ph == 8 || ph == 10 || ph == 3 || ph == 7 || ph == 9 || ph == 1 || ph == 11 || ph == 17 ||
              ph == 5 || ph == 16))
            return;
        const double *zc = A.cord + d.N;
        const GF_IDX q1 = gf_node(d, j, i), q3 = gf_node(d, j, i + 1);
        float zmax = fmaxf(fmaxf(gf_d2f(zc[q1]), gf_d2f(zc[q1 + 1])), fmaxf(gf_d2f(zc[q3]), gf_d2f(zc[q3 + 1])));
        const float surf = 0.5f * (gf_d2f(zc[gf_node(d, 0, i)]) + gf_d2f(zc[gf_node(d, 0, i + 1)]));
        const float lim = (ph == 4 || ph == 8) ? 150e3f : 200e3f;
        if (surf - zmax > lim + 10.0f) return;
    }
    double a1 = A.mark_a1[kk], a2 = A.mark_a2[kk];
    const double *cord = A.cord, *T = A.temp;
    double yy, tmpr;
    GF_IDX p1, p2, p3;
    if (k == 1) {
        p1 = gf_node(d, j, i); p2 = gf_node(d, j + 1, i); p3 = gf_node(d, j, i + 1);
    } else {
        p1 = gf_node(d, j, i + 1); p2 = gf_node(d, j + 1, i); p3 = gf_node(d, j + 1, i + 1);
    }
    yy = cord[d.N + p1] * a1 + cord[d.N + p2] * a2 + cord[d.N + p3] * (1 - a1 - a2);
    tmpr = T[p1] * a1 + T[p2] * a2 + T[p3] * (1 - a1 - a2);
    double depth = 0.5 * (cord[d.N + gf_node(d, 0, i)] + cord[d.N + gf_node(d, 0, i + 1)]) - yy;
    if (depth > 200e3) return;
    int iph = A.mark_phase[kk];
    GF_IDX e = gf_elem(d, j, i);
    const double mantle_density = 3000.0;
    GF_IDX total = (GF_IDX)P.nphase * d.E;
    auto pr = [&](GF_IDX eb, int ph1) {
        GF_IDX off = (GF_IDX)(ph1 - 1) + (GF_IDX)P.nphase * eb;
        return (off < 0 || off >= total) ? 0.0 : A.phase_ratio[off];
    };
    int newph = 0;
    switch (iph) {
    case 4: case 8: {
        if (depth > 150e3) break;
        // the reference's expressions, each evaluated only when its branch
        // needs it (the second pressure only below the first, the solidus
        // only outside the serpentine window)
        double press = mantle_density * P.g * depth;
        double trpres = 2.1e9 + (7.5e9 - 2.1e9) * (tmpr - 730.0) / (500.0 - 730.0);
        bool serp_window = false;
        if (press < trpres) {
            double trpres2 = 2.1e9 + (0.6e9 - 2.1e9) * (tmpr - 730.0) / (670.0 - 730.0);
            serp_window = press > trpres2;
        }
        if (serp_window) {
            int jb0 = min(j + 2, nz - 1), jb1 = min(j + 1 + P.nelem_serp, nz - 1);
            for (int jb = jb0; jb <= jb1; ++jb) {
                GF_IDX eb = gf_elem(d, jb - 1, i);
                if (pr(eb, 3) > 0.8 || pr(eb, 7) > 0.8 || pr(eb, 1) > 0.8 || pr(eb, 11) > 0.8) {
                    newph = 9;
                    break;
                }
            }
        } else {
            double pg = fabs(press * 1e-9);
            double solidus = -5.02 * (pg * pg) + 1.32e2 * pg + 1.09e3 + 35.0;
            if (tmpr >= solidus + 35.0) newph = 18;
        }
        break;
    }
    case 10: case 3: case 7: {
        double press = mantle_density * P.g * depth;
        if (P.eclogite_rule == 1) {
            if (tmpr >= 600.0 && press >= 1.5e9) newph = 13;
        } else {
            double trpres = -0.3e9 + 2.2e6 * tmpr;
            double trpres2 = 20.1e9 - 0.0375e9 * tmpr;
            if (!(tmpr < 400.0 || depth < 20e3 || press < trpres || press < trpres2)) newph = 13;
        }
        break;
    }
    case 9: {
        double trpres = 2.1e9 + (7.5e9 - 2.1e9) * (tmpr - 730.0) / (500.0 - 730.0);
        double trpres2 = 2.1e9 + (0.2e9 - 2.1e9) * (tmpr - 730.0) / (650.0 - 730.0);
        double press = mantle_density * P.g * depth;
        if (!(tmpr < 550.0 || (press < trpres && press > trpres2))) newph = 4;
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
        double press = mantle_density * P.g * depth;
        if (!(press < trpres)) newph = 5;
        break;
    }
    case 5: {
        double trpres = 0.0e9 - (0.0e9 - 1.2e9) * (500.0 - tmpr) / (500.0 - 600.0);
        double press = mantle_density * P.g * depth;
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
        A.e_flag[e] = 1;
        A.mark_phase[kk] = (int8_t)newph;
    }
}
__global__ void __launch_bounds__(GF_THREADS) k_phase_markers(const DevParams *__restrict__ Pp, DevArrays A, GfDims d, int nmarkers) {
    gf_pdl_entry();
    b_k_phase_markers(Pp, A, d, nmarkers, (GF_IDX)blockIdx.x * blockDim.x + threadIdx.x);
}

// The same rules in FP32 for the mixed path: the marker's depth below the
// surface from coordinate differences of the hi/lo splits, its temperature
// from the hi parts.  Decisions within FP32 rounding of a threshold may
// differ from the FP64 path.
__device__ __forceinline__ void b_k_phase_markers32(const DevParams *__restrict__ Pp, DevArrays A, GfDims d, int nmarkers, GF_IDX kk) {
    if (kk >= nmarkers) return;
    if (A.mark_dead[kk] == 0) return;
    const DevParams &P = *Pp;
    const int nz = d.nz;
    int n = A.mark_ntriag[kk];
    int k = (n - 1) % 2 + 1;
    int j = ((n - k) / 2) % (nz - 1);
    int i = (n - k) / 2 / (nz - 1);
    // the exclusions of the FP64 kernel (a phase without a rule; a marker
    // certainly deeper than its rule reaches, from the hi parts of the
    // corner and surface heights with a 10 m margin), before the marker's
    // own coordinates are read
    {
        const int ph = A.mark_phase[kk];
        if (!(ph == 4 || ph == 8 || ph == 10 || ph == 3 || ph == 7 || ph == 9 || ph == 1 || ph == 11 || ph == 17 ||
              ph == 5 || ph == 16))
            return;
        const float *zc = A.cord_hi + d.N;
        const GF_IDX q1 = gf_node(d, j, i), q3 = gf_node(d, j, i + 1);
        const float zmax = fmaxf(fmaxf(zc[q1], zc[q1 + 1]), fmaxf(zc[q3], zc[q3 + 1]));
        const float surf = 0.5f * (zc[gf_node(d, 0, i)] + zc[gf_node(d, 0, i + 1)]);
        const float lim = (ph == 4 || ph == 8) ? 150e3f : 200e3f;
        if (surf - zmax > lim + 10.0f) return;
    }
    const float a1 = gf_d2f(A.mark_a1[kk]), a2 = gf_d2f(A.mark_a2[kk]), a3 = 1.0f - a1 - a2;
    GF_IDX p1, p2, p3;
    if (k == 1) {
        p1 = gf_node(d, j, i); p2 = gf_node(d, j + 1, i); p3 = gf_node(d, j, i + 1);
    } else {
        p1 = gf_node(d, j, i + 1); p2 = gf_node(d, j + 1, i); p3 = gf_node(d, j + 1, i + 1);
    }
    const float *zh = A.cord_hi + d.N, *zl = A.cord_lo + d.N, *th = A.temp_hi;
    const GF_IDX s0 = gf_node(d, 0, i), s1 = gf_node(d, 0, i + 1);
    // depth = 0.5 * (z_s0 + z_s1) - sum a_k z_pk, as differences to z_s0
    const float ds1 = hl_diff(zh, zl, s1, s0);
    const float y1 = hl_diff(zh, zl, p1, s0), y2 = hl_diff(zh, zl, p2, s0), y3 = hl_diff(zh, zl, p3, s0);
    const float depth = 0.5f * ds1 - (y1 * a1 + y2 * a2 + y3 * a3);
    if (depth > 200e3f) return;
    const float tmpr = th[p1] * a1 + th[p2] * a2 + th[p3] * a3;
    int iph = A.mark_phase[kk];
    GF_IDX e = gf_elem(d, j, i);
    const float rho_g = 3000.0f * P.f_g;
    GF_IDX total = (GF_IDX)P.nphase * d.E;
    auto pr = [&](GF_IDX eb, int ph1) {
        GF_IDX off = (GF_IDX)(ph1 - 1) + (GF_IDX)P.nphase * eb;
        return (off < 0 || off >= total) ? 0.0 : A.phase_ratio[off];
    };
    int newph = 0;
    switch (iph) {
    case 4: case 8: {
        if (depth > 150e3f) break;
        float trpres = 2.1e9f + (7.5e9f - 2.1e9f) * (tmpr - 730.0f) / (500.0f - 730.0f);
        float trpres2 = 2.1e9f + (0.6e9f - 2.1e9f) * (tmpr - 730.0f) / (670.0f - 730.0f);
        float press = rho_g * depth;
        float pg = fabsf(press * 1e-9f);
        float solidus = -5.02f * (pg * pg) + 1.32e2f * pg + 1.09e3f + 35.0f;
        if (press < trpres && press > trpres2) {
            int jb0 = min(j + 2, nz - 1), jb1 = min(j + 1 + P.nelem_serp, nz - 1);
            for (int jb = jb0; jb <= jb1; ++jb) {
                GF_IDX eb = gf_elem(d, jb - 1, i);
                if (pr(eb, 3) > 0.8 || pr(eb, 7) > 0.8 || pr(eb, 1) > 0.8 || pr(eb, 11) > 0.8) {
                    newph = 9;
                    break;
                }
            }
        } else if (tmpr >= solidus + 35.0f) {
            newph = 18;
        }
        break;
    }
    case 10: case 3: case 7: {
        float press = rho_g * depth;
        if (P.eclogite_rule == 1) {
            if (tmpr >= 600.0f && press >= 1.5e9f) newph = 13;
        } else {
            float trpres = -0.3e9f + 2.2e6f * tmpr;
            float trpres2 = 20.1e9f - 0.0375e9f * tmpr;
            if (!(tmpr < 400.0f || depth < 20e3f || press < trpres || press < trpres2)) newph = 13;
        }
        break;
    }
    case 9: {
        float trpres = 2.1e9f + (7.5e9f - 2.1e9f) * (tmpr - 730.0f) / (500.0f - 730.0f);
        float trpres2 = 2.1e9f + (0.2e9f - 2.1e9f) * (tmpr - 730.0f) / (650.0f - 730.0f);
        float press = rho_g * depth;
        if (!(tmpr < 550.0f || (press < trpres && press > trpres2))) newph = 4;
        break;
    }
    case 1:
        if (!(tmpr < 80.0f && depth < 2e3f)) newph = 11;
        break;
    case 11:
        if (!(tmpr < 250.0f && depth < 7e3f)) newph = 17;
        break;
    case 17: {
        float trpres = 0.88e9f - (0.88e9f - 0.704e9f) * (710.8f - tmpr) / (710.8f - 662.3f);
        if (!(rho_g * depth < trpres)) newph = 5;
        break;
    }
    case 5: {
        float trpres = 0.0f - (0.0f - 1.2e9f) * (500.0f - tmpr) / (500.0f - 600.0f);
        if (!(rho_g * depth > trpres)) newph = 19;
        break;
    }
    case 16: {
        float dd = depth - 62e3f;
        float trtmpr = 880.0f - 35e-9f * (dd * dd);
        if (!(tmpr < trtmpr)) newph = 4;
        break;
    }
    default:
        break;
    }
    if (newph) {
        A.e_flag[e] = 1;
        A.mark_phase[kk] = (int8_t)newph;
    }
}
__global__ void __launch_bounds__(GF_THREADS) k_phase_markers32(const DevParams *__restrict__ Pp, DevArrays A, GfDims d, int nmarkers) {
    gf_pdl_entry();
    b_k_phase_markers32(Pp, A, d, nmarkers, (GF_IDX)blockIdx.x * blockDim.x + threadIdx.x);
}

// count_phase_ratio (marker_data.f90:140-172) for flagged elements + aps
template <class R> __device__ __forceinline__ void b_k_phase_recount(const DevParams *__restrict__ Pp, DevClock *__restrict__ C, DevArrays A, GfDims d, int all, GF_IDX e) {
    if (e >= d.E) return;
    if (!all && !A.e_flag[e]) return;
    const DevParams &P = *Pp;
    int nm = A.nmark_elem[e];
    if (nm == 0) {
        set_status(C, 134, (int)e);
        return;
    }
    int cnt[GF_MAXPH + 1];
#pragma unroll
    for (int k = 0; k <= GF_MAXPH; ++k) cnt[k] = 0;
    for (int m = 0; m < nm; ++m) {
        int kk = A.mark_id_elem[e * GF_MAX_MARKERS_PER_ELEM + m];
        int iph = A.mark_phase[kk - 1];
        if (iph >= 1 && iph <= GF_MAXPH) cnt[iph] += 1;
    }
    int best = 0, iph = 1;
    for (int k = 1; k <= P.nphase; ++k) {
        A.phase_ratio[gf_pr(d, e, k - 1)] = cnt[k] / (nm * 1.0);
        if (cnt[k] > best) {
            best = cnt[k];
            iph = k;
        }
    }
    A.iphase[e] = iph;
    if (!all) {
        R *aps = (R *)A.aps;
        R a0 = aps[e];
        R v = a0 - a0 / R((float)nm);
        aps[e] = v > R(0.0) ? v : R(0.0);
        A.e_flag[e] = 0;
    }
}
template <class R> __global__ void __launch_bounds__(GF_THREADS) k_phase_recount(const DevParams *__restrict__ Pp, DevClock *__restrict__ C, DevArrays A, GfDims d, int all) {
    gf_pdl_entry();
    b_k_phase_recount<R>(Pp, C, A, d, all, (GF_IDX)blockIdx.x * blockDim.x + threadIdx.x);
}

// ======================================================================
// itest_mesh angle criterion (rem_test.f90:77-118): min over all triangles
__device__ __forceinline__ void b_k_min_angle(DevArrays A, GfDims d, unsigned long long *out, GF_IDX e) {
    double amin = 180.0;
    if (e < d.E) {
        int j, i;
        elem_ji(d, e, j, i);
        Quad q;
        load_quad(A.cord, d, j, i, q);
        const double raddeg = 180.0 / 3.14159265358979323846;
        // local vertex ids of the 4 triangles (rem_test.f90:84-92)
        const int tv[4][3] = {{0, 1, 2}, {1, 3, 2}, {0, 1, 3}, {0, 3, 2}};
#pragma unroll
        for (int t = 0; t < 4; ++t) {
            int v[4] = {tv[t][0], tv[t][1], tv[t][2], tv[t][0]};
            double ang[3];
#pragma unroll
            for (int k = 1; k <= 2; ++k) {
                double xa = q.x[v[k + 1]] - q.x[v[k]], ya = q.y[v[k + 1]] - q.y[v[k]];
                double xxal = sqrt(xa * xa + ya * ya);
                double xb = q.x[v[k - 1]] - q.x[v[k]], yb = q.y[v[k - 1]] - q.y[v[k]];
                double xxbl = sqrt(xb * xb + yb * yb);
                ang[k] = raddeg * acos((xa * xb + ya * yb) / (xxal * xxbl));
            }
            ang[0] = 180.0 - ang[1] - ang[2];
            amin = fmin(amin, fmin(ang[0], fmin(ang[1], ang[2])));
        }
    }
    amin = warp_min(amin);
    if ((threadIdx.x & 31) == 0) atomic_min_pos(out, fmax(amin, 0.0));
}
__global__ void __launch_bounds__(GF_THREADS) k_min_angle(DevArrays A, GfDims d, unsigned long long *out) {
    gf_pdl_entry();
    b_k_min_angle(A, d, out, (GF_IDX)blockIdx.x * blockDim.x + threadIdx.x);
}

// FP64 host array -> R device array
template <class R> __device__ __forceinline__ void b_k_convert(const double *__restrict__ src, R *__restrict__ dst, GF_IDX n, GF_IDX t) {
    if (t < n) dst[t] = R(src[t]);
}
template <class R> __global__ void k_convert(const double *__restrict__ src, R *__restrict__ dst, GF_IDX n) {
    gf_pdl_entry();
    b_k_convert<R>(src, dst, n, (GF_IDX)blockIdx.x * blockDim.x + threadIdx.x);
}
template <class R> __device__ __forceinline__ void b_k_convert_back(const R *__restrict__ src, double *__restrict__ dst, GF_IDX n, GF_IDX t) {
    if (t < n) dst[t] = (double)src[t];
}
template <class R> __global__ void k_convert_back(const R *__restrict__ src, double *__restrict__ dst, GF_IDX n) {
    gf_pdl_entry();
    b_k_convert_back<R>(src, dst, n, (GF_IDX)blockIdx.x * blockDim.x + threadIdx.x);
}

} // namespace gfk
} // namespace

// ---------------------------------------------------------------- launchers
// Launch with programmatic stream serialization (the kernel starts with
// gf_pdl_entry); `n` items, GF_THREADS per CTA.
template <class... KArgs, class... Args>
inline void gf_launch_pdl(void (*kern)(KArgs...), unsigned grid, cudaStream_t s, Args... args) {
    cudaLaunchConfig_t lc = {};
    lc.gridDim = dim3(grid);
    lc.blockDim = dim3(GF_THREADS);
    lc.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    lc.attrs = at;
    lc.numAttrs = 1;
    cudaLaunchKernelEx(&lc, kern, (KArgs)args...);
}
#define GF_LAUNCH(kern, n, ...)                                                                                        \
    do {                                                                                                               \
        if ((n) > 0) {                                                                                                 \
            gf_launch_pdl(kern, gfk::grid_for(n), g.s, __VA_ARGS__);                                                   \
            ++*g.launches;                                                                                             \
        }                                                                                                              \
    } while (0)

// The table read by plastic_table_state's elements: one thread per (phase,
// state), each evaluating pre_plast_phase and plastic_consts as the element
// path does, with a plastic strain in the state's branch (-inf: before
// softening, plstrain1: at its start, +inf: after it).
namespace { // internal linkage, one copy per precision's translation unit
namespace gfk {
template <class R> __global__ void k_plastic_table(const DevParams *__restrict__ Pp, R *__restrict__ tab) {
    const DevParams &P = *Pp;
    const int t = threadIdx.x;
    if (t >= GF_MAXPH * GF_PT_STATES) return;
    const int k = t / GF_PT_STATES, s = t % GF_PT_STATES;
    R pl1, bulkm, rmu, ten_off;
    if constexpr (sizeof(R) == sizeof(float)) {
        pl1 = P.f_pl1[k]; bulkm = P.f_bulkm[k]; rmu = P.f_rm[k]; ten_off = P.f_ten_off;
    } else {
        pl1 = P.plstrain1[k]; bulkm = P.bulkm[k]; rmu = P.rm[k]; ten_off = P.ten_off;
    }
    const R pls = s == 0 ? R(-INFINITY) : (s == 1 ? pl1 : R(INFINITY));
    R phi = 0, coh = 0, psi = 0, hardn = 0;
    pre_plast_phase(P, k, R(1), pls, phi, coh, psi, hardn);
    phi = R(1) / phi;
    coh = R(1) / coh;
    const PlasticConsts<R> c = plastic_consts<R>(bulkm, rmu, coh, phi, psi, ten_off);
    R *o = tab + (s * GF_MAXPH + k) * GF_PT_W;
    o[0] = c.anphi; o[1] = c.anpsi; o[2] = c.amc; o[3] = c.e1;
    o[4] = c.e2; o[5] = c.x1; o[6] = c.ten_max; o[7] = hardn;
}
} // namespace gfk
} // namespace
template <class R> void GfKernels<R>::plastic_table(const GfLaunch &g) {
    if (g.A.plast_tab) {
        gfk::k_plastic_table<R><<<1, GF_MAXPH * GF_PT_STATES, 0, g.s>>>(g.P, (R *)g.A.plast_tab);
        ++*g.launches;
    }
}

template <class R> void GfKernels<R>::therm_prep(const GfLaunch &g) {
    using namespace gfk;
    if (sizeof(R) == sizeof(float)) GF_LAUNCH(k_therm_prep32, g.d.E, g.P, g.A, g.d, (float *)g.A.t_coef);
}

template <class R> void GfKernels<R>::therm_sweeps(const GfLaunch &g) {
    using namespace gfk;
    if (sizeof(R) != sizeof(float)) return;
    const float *tc = (const float *)g.A.t_coef;
    float *d0 = (float *)g.A.t_delta0;
    GF_LAUNCH(k_therm_sweep32, g.d.N, g.P, g.C, g.A, g.d, tc, d0, g.A.t_delta1, 0);
    GF_LAUNCH(k_therm_sweep32, g.d.N, g.P, g.C, g.A, g.d, tc, d0, g.A.t_delta1, 1);
    GF_LAUNCH(k_therm_apply32, g.d.N, g.P, g.A, g.d, g.A.t_delta1);
}

template <class R> void GfKernels<R>::therm(const GfLaunch &g, int sweeps, int keep_temp0) {
    using namespace gfk;
    if (sizeof(R) == sizeof(float)) {
        therm_prep(g);
        therm_sweeps(g);
        return;
    }
    int kmax = sweeps > 0 ? (sweeps < GF_THERM_KMAX ? sweeps : GF_THERM_KMAX) : GF_THERM_KMAX;
    GF_LAUNCH(k_therm_prep<R>, g.d.E, g.P, g.C, g.A, g.d, g.A.t_coef);
    // the sweeps and the boundary pass: one co-resident launch
    static int occ[64] = {0}, sms[64] = {0};
    int dev = 0;
    cudaGetDevice(&dev);
    dev = dev & 63;
    if (occ[dev] == 0) {
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ[dev], k_therm_sweeps, GF_THREADS, 0);
        cudaDeviceGetAttribute(&sms[dev], cudaDevAttrMultiProcessorCount, dev);
        if (occ[dev] <= 0) occ[dev] = 1;
    }
    const GF_IDX need = (g.d.N + GF_THREADS - 1) / GF_THREADS;
    const GF_IDX cap = (GF_IDX)occ[dev] * sms[dev];
    // arrivals and the error flag start at zero in every launch (the
    // generation counter only has to change)
    cudaMemsetAsync(g.therm_bar, 0, sizeof(unsigned), g.s);
    cudaMemsetAsync(g.therm_bar + 2, 0, sizeof(unsigned), g.s);
    cudaLaunchConfig_t lc = {};
    lc.gridDim = dim3((unsigned)(need < cap ? need : cap));
    lc.blockDim = dim3(GF_THREADS);
    lc.stream = g.s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    lc.attrs = attr;
    lc.numAttrs = 1;
    cudaLaunchKernelEx(&lc, k_therm_sweeps, g.P, g.C, g.A, g.d, (const double *)g.A.t_coef, g.A.t_delta0,
                       g.A.t_delta1, kmax, keep_temp0, g.therm_bar);
    ++*g.launches;
}

template <class R> void GfKernels<R>::rheol(const GfLaunch &g, int update_visc, int avg_mode) {
    using namespace gfk;
    GF_LAUNCH(k_rheol<R>, g.d.E, g.P, g.C, g.A, g.d, update_visc, 0);
    if (avg_mode > 0) {
        GF_LAUNCH(k_rheol_avg<R>, g.d.E, g.C, g.A, g.d, avg_mode == 2 ? 1 : 0);
        if (avg_mode == 2) {
            k_rheol_clock<<<1, 1, 0, g.s>>>(g.C, 1);
            ++*g.launches;
        }
    }
}

namespace {
namespace gfk {
__global__ void __launch_bounds__(GF_THREADS) k_elem_forces(DevArrays A, GfDims d) {
    gf_pdl_entry();
    const GF_IDX e = (GF_IDX)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= d.E) return;
    int j, i;
    elem_ji(d, e, j, i);
    const float *st = (const float *)A.stress0;
    const float *area = (const float *)A.area;
    float ar[4], sn[4][4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        ar[k] = area[gf_ek(d, e, k)];
#pragma unroll
        for (int c = 0; c < 4; ++c) sn[c][k] = st[gf_s(d, e, c, k)];
    }
    QuadF q;
    load_quad_rel(A, d, j, i, q);
    float dx[3][4], dz[3][4];
    shape_derivs_f(q, ar, dx, dz);
    elem_corner_forces(dx, dz, ar, sn, A.e_frc, d.E, e);
}
} // namespace gfk
} // namespace

template <class R> void GfKernels<R>::elem_forces(const GfLaunch &g) {
    using namespace gfk;
    if (sizeof(R) == sizeof(float)) GF_LAUNCH(k_elem_forces, g.d.E, g.A, g.d);
}

template <class R> void GfKernels<R>::node(const GfLaunch &g) {
    using namespace gfk;
    GF_LAUNCH(k_node<R>, g.d.N, g.P, g.C, g.A, g.d, g.node_terms);
}

template <class R> void GfKernels<R>::move_cord(const GfLaunch &g) {
    using namespace gfk;
    GF_LAUNCH(k_move_cord, 2 * g.d.N, g.C, g.A, g.d);
}
template <class R> void GfKernels<R>::move_elem(const GfLaunch &g) {
    using namespace gfk;
    GF_LAUNCH(k_move_elem<R>, g.d.E, g.C, g.A, g.d, g.advance_time);
}
template <class R> void GfKernels<R>::move(const GfLaunch &g) {
    move_cord(g);
    move_elem(g);
}

template <class R> void GfKernels<R>::rmasses(const GfLaunch &g) {
    using namespace gfk;
    GF_LAUNCH(k_elem_dens<R>, g.d.E, g.P, g.C, g.A, g.d);
    k_frac_fix<R><<<1, 1, 0, g.s>>>(g.P, g.C, g.A, g.d);
    ++*g.launches;
    GF_LAUNCH(k_node_gather_tri<R>, g.d.N, (const R *)g.A.e_tri, g.A.rmass, g.d);
}

template <class R> void GfKernels<R>::dt_mass(const GfLaunch &g) {
    using namespace gfk;
    k_dt_reset<<<1, 1, 0, g.s>>>(g.C);
    ++*g.launches;
    GF_IDX n = g.d.E > g.d.N ? g.d.E : g.d.N;
    GF_LAUNCH(k_dt_reduce<R>, n, g.P, g.C, g.A, g.d);
    k_dt_scalars<<<1, 1, 0, g.s>>>(g.P, g.C);
    ++*g.launches;
    if (g.idt_scale == 0) {
        cudaMemcpyAsync(g.A.amass, g.A.rmass, sizeof(double) * g.d.N, cudaMemcpyDeviceToDevice, g.s);
    } else {
        GF_LAUNCH(k_elem_am3<R>, g.d.E, g.P, g.C, g.A, g.d);
        GF_LAUNCH(k_node_gather_tri<R>, g.d.N, (const R *)g.A.e_tri, g.A.amass, g.d);
    }
}

template <class R> void GfKernels<R>::init_visc(const GfLaunch &g) {
    using namespace gfk;
    GF_LAUNCH(k_init_visc<R>, g.d.E, g.P, g.A, g.d);
}

template <class R> void GfKernels<R>::change_phase(const GfLaunch &g, int nmarkers) {
    using namespace gfk;
    if (sizeof(R) == sizeof(float))
        GF_LAUNCH(k_phase_markers32, (GF_IDX)nmarkers, g.P, g.A, g.d, nmarkers);
    else
        GF_LAUNCH(k_phase_markers, (GF_IDX)nmarkers, g.P, g.A, g.d, nmarkers);
    GF_LAUNCH(k_phase_recount<R>, g.d.E, g.P, g.C, g.A, g.d, 0);
}

namespace {
namespace gfk {
__global__ void k_split(const double *__restrict__ src, float *__restrict__ hi, float *__restrict__ lo, GF_IDX n) {
    gf_pdl_entry();
    GF_IDX t = (GF_IDX)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    const double v = src[t];
    const float h = (float)v;
    hi[t] = h;
    lo[t] = (float)(v - (double)h);
}
} // namespace gfk
} // namespace

template <class R> void GfKernels<R>::split_nodes(const GfLaunch &g) {
    using namespace gfk;
    if (!g.A.cord_hi) return;
    GF_LAUNCH(k_split, 2 * g.d.N, g.A.cord, g.A.cord_hi, g.A.cord_lo, 2 * g.d.N);
    GF_LAUNCH(k_split, 2 * g.d.N, g.A.vel, g.A.vel_hi, g.A.vel_lo, 2 * g.d.N);
    if (g.A.pr_hi) GF_LAUNCH(k_split, g.d.E, g.A.p_ref, g.A.pr_hi, g.A.pr_lo, g.d.E);
    if (g.A.temp_hi) GF_LAUNCH(k_split, g.d.N, g.A.temp, g.A.temp_hi, g.A.temp_lo, g.d.N);
}

template <class R> void GfKernels<R>::phase_recount_all(const GfLaunch &g) {
    using namespace gfk;
    GF_LAUNCH(k_phase_recount<R>, g.d.E, g.P, g.C, g.A, g.d, 1);
}

template <class R> void GfKernels<R>::min_angle(const GfLaunch &g, double *d_out) {
    using namespace gfk;
    GF_LAUNCH(k_min_angle, g.d.E, g.A, g.d, (unsigned long long *)d_out);
}

template <class R>
void GfKernels<R>::convert_in(const GfLaunch &g, unsigned mask, const double *src, void *dst, long long n) {
    using namespace gfk;
    if (mask)
        GF_LAUNCH(k_convert<R>, n, src, (R *)dst, n);
    else
        GF_LAUNCH(k_convert_back<R>, n, (const R *)dst, (double *)src, n);
}

namespace {
namespace gfk {
// total stress -> (p_ref, total + p_ref on the normal components)
template <class R> __device__ __forceinline__ void b_k_stress_in(const double *__restrict__ tot, R *__restrict__ st, double *__restrict__ p_ref, GfDims d, GF_IDX e) {
    if (e >= d.E) return;
    double s = 0.0;
#pragma unroll
    for (int k = 0; k < 4; ++k) s += tot[gf_s(d, e, 0, k)] + tot[gf_s(d, e, 1, k)] + tot[gf_s(d, e, 3, k)];
    double p = -s / 12.0;
    p_ref[e] = p;
#pragma unroll
    for (int k = 0; k < 4; ++k)
#pragma unroll
        for (int c = 0; c < 4; ++c) st[gf_s(d, e, c, k)] = R(c == 2 ? tot[gf_s(d, e, c, k)] : tot[gf_s(d, e, c, k)] + p);
}
template <class R> __global__ void __launch_bounds__(GF_THREADS) k_stress_in(const double *__restrict__ tot, R *__restrict__ st, double *__restrict__ p_ref, GfDims d) {
    gf_pdl_entry();
    b_k_stress_in<R>(tot, st, p_ref, d, (GF_IDX)blockIdx.x * blockDim.x + threadIdx.x);
}

template <class R> __device__ __forceinline__ void b_k_stress_out(const R *__restrict__ st, const double *__restrict__ p_ref, double *__restrict__ tot, GfDims d, GF_IDX e) {
    if (e >= d.E) return;
    double p = p_ref[e];
#pragma unroll
    for (int k = 0; k < 4; ++k)
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            double v = (double)st[gf_s(d, e, c, k)];
            tot[gf_s(d, e, c, k)] = c == 2 ? v : v - p;
        }
}
template <class R> __global__ void __launch_bounds__(GF_THREADS) k_stress_out(const R *__restrict__ st, const double *__restrict__ p_ref, double *__restrict__ tot, GfDims d) {
    gf_pdl_entry();
    b_k_stress_out<R>(st, p_ref, tot, d, (GF_IDX)blockIdx.x * blockDim.x + threadIdx.x);
}
} // namespace gfk
} // namespace

template <class R> void GfKernels<R>::stress_in(const GfLaunch &g, const double *src) {
    using namespace gfk;
    GF_LAUNCH(k_stress_in<R>, g.d.E, src, (R *)g.A.stress0, g.A.p_ref, g.d);
    if (g.A.pr_hi) GF_LAUNCH(k_split, g.d.E, g.A.p_ref, g.A.pr_hi, g.A.pr_lo, g.d.E);
}

template <class R> void GfKernels<R>::stress_out(const GfLaunch &g, double *dst) {
    using namespace gfk;
    GF_LAUNCH(k_stress_out<R>, g.d.E, (const R *)g.A.stress0, g.A.p_ref, dst, g.d);
}
