// C-ABI of the GB300 FLAC step (include/geoflac_gb300.h): context
// management, host<->device sync points, the per-subroutine entry points
// and the graph-captured multi-step driver.

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <new>
#include <vector>

#include "../../include/geoflac_gb300.h"
#include "gf_ctx.h"
#include "gf_internal.h"
#include "gf_member.h"

namespace {

struct GraphEntry {
    unsigned sig;
    cudaGraphExec_t exec;
    long long nlaunch;
};

} // namespace

struct gf_ctx {
    gf_params p;
    gf_layout L;
    int mode;
    GfDims d;
    cudaStream_t s = nullptr;
    // mixed: second stream and fork/join events for the thermal sweeps that
    // run beside fl_rheol / fl_node
    cudaStream_t s2 = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    DevParams *dP = nullptr;
    DevClock *dC = nullptr;
    DevArrays A{};
    double *staging = nullptr; // FP64 staging for mixed-mode conversions
    double *d_angle = nullptr;
    unsigned *therm_bar = nullptr; // grid barrier of the FP64 thermal sweeps
    GfRemeshBufs rb{};         // remesh scratch
    double ar_x = 0, ar_z = 0; // mesh1 zone-pattern totals
    // host mirrors of the host-controlled scalars
    int nloop = 0, nsrate = -1, nmarkers = 0, need_remeshing = 0;
    long long launches = 0;
    std::vector<GraphEntry> graphs;
    std::vector<void *> allocs;
    int sweeps = 0; // cap on the thermal sweeps (0: library cap)
    int sync = 1;
    int frc_valid = 0; // e_frc (mixed) / n_frc (FP64) hold the node-force terms of the current stresses and mesh
};

namespace {

int cuda_err(cudaError_t e, const char *what) {
    if (e == cudaSuccess) return GF_OK;
    std::fprintf(stderr, "geoflac_gb300: CUDA error in %s: %s\n", what, cudaGetErrorString(e));
    return GF_ERR_CUDA;
}

#define GF_CK(call)                                                                                                    \
    do {                                                                                                               \
        int _rc = cuda_err((call), #call);                                                                             \
        if (_rc) return _rc;                                                                                           \
    } while (0)

template <class T> int dalloc(gf_ctx *c, T **ptr, size_t count) {
    *ptr = nullptr;
    if (count == 0) count = 1;
    void *p = nullptr;
    cudaError_t e = cudaMalloc(&p, count * sizeof(T));
    if (e != cudaSuccess) return cuda_err(e, "cudaMalloc");
    cudaMemset(p, 0, count * sizeof(T));
    c->allocs.push_back(p);
    *ptr = (T *)p;
    return GF_OK;
}

int ralloc(gf_ctx *c, void **ptr, size_t count) {
    if (c->mode == GF_MODE_MIXED) return dalloc(c, (float **)ptr, count);
    return dalloc(c, (double **)ptr, count);
}

void fill_params(DevParams &P, const gf_params &p) {
    std::memset(&P, 0, sizeof P);
    P.nx = p.nx; P.nz = p.nz; P.nphase = p.nphase;
    P.ndim = p.ndim; P.mix_strain = p.mix_strain; P.mix_stress = p.mix_stress;
    P.istress_therm = p.istress_therm; P.ishearh = p.ishearh; P.itherm = p.itherm; P.itemp_bc = p.itemp_bc;
    P.nyhydro = p.nyhydro; P.iphsub = p.iphsub > 0 ? p.iphsub : 1; P.i_prestress = p.i_prestress;
    P.idt_scale = p.idt_scale; P.i_rey = p.i_rey; P.ivis_present = p.ivis_present;
    P.itype_melting = p.itype_melting; P.nystressbc = p.nystressbc; P.movegrid = p.movegrid;
    P.nelem_serp = p.nelem_serp; P.eclogite_rule = p.eclogite_rule;
    for (int k = 0; k < GF_MAXPH; ++k) {
        P.irheol[k] = p.irheol[k];
        P.rl[k] = p.rl[k]; P.rm[k] = p.rm[k]; P.den[k] = p.den[k]; P.alfa[k] = p.alfa[k]; P.beta[k] = p.beta[k];
        P.pln[k] = p.pln[k]; P.acoef[k] = p.acoef[k]; P.eactiv[k] = p.eactiv[k]; P.vactiv[k] = p.vactiv[k];
        P.plstrain1[k] = p.plstrain1[k]; P.plstrain2[k] = p.plstrain2[k]; P.fric1[k] = p.fric1[k];
        P.fric2[k] = p.fric2[k]; P.cohesion1[k] = p.cohesion1[k]; P.cohesion2[k] = p.cohesion2[k];
        P.dilat1[k] = p.dilat1[k]; P.dilat2[k] = p.dilat2[k]; P.conduct[k] = p.conduct[k]; P.cp[k] = p.cp[k];
    }
    int w = 0;
    for (int k = 0; k < p.inhom && k < GF_MAXINH; ++k)
        if (p.igeom[k] == 100) {
            P.w_ix1[w] = p.ix1[k]; P.w_ix2[w] = p.ix2[k]; P.w_iy1[w] = p.iy1[k]; P.w_iy2[w] = p.iy2[k];
            ++w;
        }
    P.ninh100 = w;
    P.g = p.g; P.demf = p.demf; P.ten_off = p.ten_off; P.tau_heal = p.tau_heal; P.v_min = p.v_min;
    P.v_max = p.v_max; P.t_top = p.t_top; P.t_bot = p.t_bot; P.bot_bc = p.bot_bc; P.pisos = p.pisos;
    P.drosub = p.drosub; P.rzbo = p.rzbo; P.rxbo = p.rxbo; P.vbc = p.vbc; P.fmagma_max = p.fmagma_max;
    P.rho_magma = p.rho_magma; P.weaken_ratio_plastic = p.weaken_ratio_plastic;
    P.weaken_ratio_viscous = p.weaken_ratio_viscous; P.xReyn = p.xReyn; P.strain_inert = p.strain_inert;
    P.dt_scale = p.dt_scale; P.fracm = p.fracm;
    for (int k = 0; k < GF_MAXPH; ++k) {
        P.f_bulkm[k] = (float)(p.rl[k] + 2.0 * p.rm[k] / 3.0);
        P.f_rm[k] = (float)p.rm[k];
        P.f_fric1[k] = (float)p.fric1[k];
        P.f_fric2[k] = (float)p.fric2[k];
        P.f_coh1[k] = (float)p.cohesion1[k];
        P.f_coh2[k] = (float)p.cohesion2[k];
        P.f_dil1[k] = (float)p.dilat1[k];
        P.f_dil2[k] = (float)p.dilat2[k];
        P.f_pl1[k] = (float)p.plstrain1[k];
        P.f_pl2[k] = (float)p.plstrain2[k];
        P.f_cp[k] = (float)p.cp[k];
        P.f_cond[k] = (float)p.conduct[k];
        P.f_den[k] = (float)p.den[k];
        P.f_pln[k] = (float)p.pln[k];
        P.f_lacoef[k] = p.acoef[k] > 0 ? (float)std::log(0.75 * p.acoef[k]) : 0.0f;
        P.f_eactiv[k] = (float)p.eactiv[k];
        P.f_vactiv[k] = (float)p.vactiv[k];
    }
    P.f_ten_off = (float)p.ten_off;
    P.f_tau_heal = (float)p.tau_heal;
    P.f_demf = (float)p.demf;
    for (int k = 0; k < GF_MAXPH; ++k) {
        P.f_alfa[k] = (float)p.alfa[k];
        P.f_beta[k] = (float)p.beta[k];
        P.diffu[k] = (p.den[k] != 0.0 && p.cp[k] != 0.0) ? p.conduct[k] / p.den[k] / p.cp[k] : 0.0;
        // the device's per-element expressions, evaluated once per phase
        // (same IEEE operations; host code is built without contraction)
        P.bulkm[k] = p.rl[k] + 2.0 * p.rm[k] / 3.0;
        P.hsoft[k] = (p.plstrain2[k] != p.plstrain1[k])
                         ? (p.cohesion2[k] - p.cohesion1[k]) / (p.plstrain2[k] - p.plstrain1[k])
                         : 0.0;
        const double lambda = P.bulkm[k] - (2.0 / 3.0) * p.rm[k];
        double den_el = 3.0 * lambda + 2.0 * p.rm[k];
        if (std::fabs(den_el) < 1e-30) den_el = den_el < 0.0 ? -1e-30 : 1e-30;
        P.sh_lam_den[k] = lambda / den_el;
        P.sh_r2mu_y[k] = 1.0 / (2.0 * p.rm[k]);
        P.sh_r2mu_yl[k] = std::fma(-P.sh_r2mu_y[k], 2.0 * p.rm[k], 1.0) * P.sh_r2mu_y[k];
    }
    P.f_fmagma_max = (float)p.fmagma_max;
    P.topo_kappa = p.topo_kappa;
    for (int k = 0; k < GF_MAXPH; ++k) P.erodibility[k] = p.erodibility[k];
    P.f_rho_magma = (float)p.rho_magma;
    P.f_g = (float)p.g;
    P.prod_magma = p.prod_magma; P.prod_magma2 = p.prod_magma2; P.angle_mzone = p.angle_mzone;
    P.ratio_mantle_mzone = p.ratio_mantle_mzone; P.ratio_crust_mzone = p.ratio_crust_mzone;
    P.latent_heat_magma = p.latent_heat_magma; P.lambda_freeze = p.lambda_freeze;
    P.lambda_freeze_tdep = p.lambda_freeze_tdep; P.dxmin = p.dxmin; P.Amin = p.Amin; P.nelem_dike = p.nelem_dike;
}

GfLaunch launch_of(gf_ctx *c) {
    GfLaunch g;
    g.P = c->dP;
    g.C = c->dC;
    g.A = c->A;
    g.d = c->d;
    g.s = c->s;
    g.launches = &c->launches;
    g.arc_rate = 1.0 - c->p.ratio_mantle_mzone - c->p.ratio_crust_mzone;
    g.idt_scale = c->p.idt_scale;
    g.advance_time = 0;
    g.therm_bar = c->therm_bar;
    g.node_terms = 0;
    return g;
}

// Copy one FP64 host array to a device array of the context's precision
// (dir = 1 upload, 0 download).
int xfer_r(gf_ctx *c, double *host, void *dev, long long n, int dir) {
    if (!host || n <= 0) return GF_OK;
    if (c->mode == GF_MODE_FP64) {
        if (dir)
            GF_CK(cudaMemcpyAsync(dev, host, n * sizeof(double), cudaMemcpyHostToDevice, c->s));
        else
            GF_CK(cudaMemcpyAsync(host, dev, n * sizeof(double), cudaMemcpyDeviceToHost, c->s));
        return GF_OK;
    }
    GfLaunch g = launch_of(c);
    if (dir) {
        GF_CK(cudaMemcpyAsync(c->staging, host, n * sizeof(double), cudaMemcpyHostToDevice, c->s));
        GfKernels<float>::convert_in(g, 1, c->staging, dev, n);
    } else {
        GfKernels<float>::convert_in(g, 0, c->staging, dev, n);
        GF_CK(cudaMemcpyAsync(host, c->staging, n * sizeof(double), cudaMemcpyDeviceToHost, c->s));
    }
    GF_CK(cudaStreamSynchronize(c->s));
    return GF_OK;
}

template <class T> int xfer(gf_ctx *c, T *host, T *dev, long long n, int dir) {
    if (!host || n <= 0) return GF_OK;
    if (dir)
        GF_CK(cudaMemcpyAsync(dev, host, n * sizeof(T), cudaMemcpyHostToDevice, c->s));
    else
        GF_CK(cudaMemcpyAsync(host, dev, n * sizeof(T), cudaMemcpyDeviceToHost, c->s));
    return GF_OK;
}

int move_fields(gf_ctx *c, unsigned m, int dir) {
    if (dir) c->frc_valid = 0;
    const gf_layout &L = c->L;
    DevArrays &A = c->A;
    long long N = c->d.N, E = c->d.E;
    int rc = 0;
#define T_(x)                                                                                                          \
    do {                                                                                                               \
        if ((rc = (x))) return rc;                                                                                     \
    } while (0)
    if (m & GF_F_CORD) T_(xfer(c, L.cord, A.cord, 2 * N, dir));
    if (m & GF_F_VEL) T_(xfer(c, L.vel, A.vel, 2 * N, dir));
    if (m & GF_F_TEMP) {
        T_(xfer(c, L.temp, A.temp, N, dir));
        T_(xfer(c, L.temp0, A.temp0, N, dir));
    }
    if (m & GF_F_MASS) {
        T_(xfer(c, L.amass, A.amass, N, dir));
        T_(xfer(c, L.rmass, A.rmass, N, dir));
    }
    if (m & GF_F_BC) {
        T_(xfer(c, L.bc, A.bc, 2 * N, dir));
        T_(xfer(c, L.ncod, A.ncod, 2 * N, dir));
    }
    if ((m & GF_F_STRESS) && L.stress0) {
        if (c->mode == GF_MODE_FP64) {
            T_(xfer_r(c, L.stress0, A.stress0, 16 * E, dir));
        } else {
            // mixed: FP32 deviations from the element's reference pressure
            GfLaunch g = launch_of(c);
            if (dir) {
                GF_CK(cudaMemcpyAsync(c->staging, L.stress0, 16 * E * sizeof(double), cudaMemcpyHostToDevice, c->s));
                GfKernels<float>::stress_in(g, c->staging);
            } else {
                GfKernels<float>::stress_out(g, c->staging);
                GF_CK(cudaMemcpyAsync(L.stress0, c->staging, 16 * E * sizeof(double), cudaMemcpyDeviceToHost, c->s));
            }
            GF_CK(cudaStreamSynchronize(c->s));
        }
    }
    if (m & GF_F_AREA) {
        T_(xfer_r(c, L.area, A.area, 4 * E, dir));
        T_(xfer_r(c, L.dvol, A.dvol, 4 * E, dir));
    }
    if (m & GF_F_STRAIN) T_(xfer_r(c, L.strain, A.strain, 3 * E, dir));
    if (m & GF_F_APS) T_(xfer_r(c, L.aps, A.aps, E, dir));
    if (m & GF_F_VISN) T_(xfer_r(c, L.visn, A.visn, E, dir));
    if (m & GF_F_PHASE) {
        T_(xfer(c, L.iphase, A.iphase, E, dir));
        T_(xfer(c, L.phase_ratio, A.phase_ratio, (long long)c->p.nphase * E, dir));
        T_(xfer(c, L.jmoho, A.jmoho, c->p.nx - 1, dir));
    }
    if (m & GF_F_RATE) {
        T_(xfer_r(c, L.e2sr, A.e2sr, E, dir));
        T_(xfer_r(c, L.se2sr, A.se2sr, 3 * E, dir));
        T_(xfer_r(c, L.shrheat, A.shrheat, E, dir));
        T_(xfer_r(c, L.sshrheat, A.sshrheat, E, dir));
        T_(xfer(c, L.source, A.source, E, dir));
        T_(xfer(c, L.fmagma, A.fmagma, E, dir));
        T_(xfer(c, L.fmagma2, A.fmagma2, E, dir));
        T_(xfer(c, L.dike_released, A.dike_released, E, dir));
        if (A.dike_backlog) { // magma sub-model
            T_(xfer(c, L.fmelt, A.fmelt, E, dir));
            T_(xfer(c, L.fmelt2, A.fmelt2, E, dir));
            T_(xfer(c, L.dike_backlog, A.dike_backlog, E, dir));
            T_(xfer(c, L.dike_marker_vol, A.dike_marker_vol, E, dir));
            T_(xfer(c, L.mor_marker_vol, A.mor_marker_vol, E, dir));
        }
    }
    if (m & GF_F_MARKERS) {
        long long M = L.max_markers;
        T_(xfer(c, L.mark_a1, A.mark_a1, M, dir));
        T_(xfer(c, L.mark_a2, A.mark_a2, M, dir));
        T_(xfer(c, L.mark_age, A.mark_age, M, dir));
        T_(xfer(c, L.mark_dead, A.mark_dead, M, dir));
        T_(xfer(c, L.mark_phase, A.mark_phase, M, dir));
        T_(xfer(c, L.mark_ntriag, A.mark_ntriag, M, dir));
        T_(xfer(c, L.mark_id_elem, A.mark_id_elem, (long long)GF_MAX_MARKERS_PER_ELEM * E, dir));
        T_(xfer(c, L.nmark_elem, A.nmark_elem, E, dir));
        T_(xfer(c, L.dhacc_correction, A.dhacc_correction, c->p.nx, dir));
        T_(xfer(c, L.dhacc, A.dhacc, c->p.nx, dir));
        T_(xfer(c, L.extr_acc, A.extr_acc, c->p.nx, dir));
        T_(xfer(c, L.dtopo, A.dtopo, c->p.nx, dir));
        T_(xfer(c, L.xoriginal, A.orig, N, dir));
        T_(xfer(c, L.zoriginal, A.orig + N, N, dir));
        T_(xfer(c, L.q_init, A.q_init, c->p.nx, dir));
        T_(xfer(c, L.vel_flex_old, A.vel_flex_old, c->p.nx, dir));
        if (A.extrusion) T_(xfer(c, L.extrusion, A.extrusion, c->p.nx, dir));
    }
#undef T_
    if (dir && (m & (GF_F_CORD | GF_F_VEL | GF_F_TEMP)) && c->mode == GF_MODE_MIXED) {
        GfLaunch g = launch_of(c);
        GfKernels<float>::split_nodes(g);
    }
    GF_CK(cudaStreamSynchronize(c->s));
    return GF_OK;
}

// Read and clear the device status word.
int take_status(gf_ctx *c);

// Status after a per-subroutine call: waits only in sync mode.
int call_status(gf_ctx *c) {
    if (!c->sync) {
        cudaError_t e = cudaGetLastError();
        return e == cudaSuccess ? GF_OK : cuda_err(e, "launch");
    }
    return take_status(c);
}

int take_status(gf_ctx *c) {
    int st = 0;
    cudaError_t e = cudaStreamSynchronize(c->s);
    if (e != cudaSuccess) return cuda_err(e, "step");
    e = cudaMemcpy(&st, &c->dC->status, sizeof(int), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_err(e, "status");
    if (st) {
        int zero = 0;
        cudaMemcpy(&c->dC->status, &zero, sizeof(int), cudaMemcpyHostToDevice);
    }
    return st;
}

__global__ void k_clock_advance(DevClock *C) { C->time = C->time + C->dt; }

// ---- dispatch on precision
void k_therm(gf_ctx *c) {
    GfLaunch g = launch_of(c);
    if (c->mode == GF_MODE_MIXED) {
        GfKernels<float>::therm(g, c->sweeps);
    } else if (c->p.itype_melting == 1) {
        // temp0 = temp, then the magma sub-model changes temp before the
        // diffusion (fl_therm.f90:53-391)
        cudaMemcpyAsync(c->A.temp0, c->A.temp, sizeof(double) * c->d.N, cudaMemcpyDeviceToDevice, c->s);
        GfMagma::therm(g, (int)c->L.max_markers);
        GfKernels<double>::therm(g, c->sweeps, 1);
    } else {
        GfKernels<double>::therm(g, c->sweeps);
    }
}
void k_rheol(gf_ctx *c, int upd, int avg) {
    GfLaunch g = launch_of(c);
    if (c->mode == GF_MODE_MIXED) GfKernels<float>::rheol(g, upd, avg);
    else GfKernels<double>::rheol(g, upd, avg);
    c->frc_valid = 1;
}
void k_node(gf_ctx *c) {
    GfLaunch g = launch_of(c);
    if (c->mode == GF_MODE_MIXED) {
        if (!c->frc_valid) GfKernels<float>::elem_forces(g);
        c->frc_valid = 1;
        GfKernels<float>::node(g);
    } else {
        g.node_terms = c->frc_valid && c->A.n_frc;
        GfKernels<double>::node(g);
    }
}
// fl_move (fl_move.f90:4-132): the coordinate update, diff_topo (with
// resurface every ifreq_avgsr steps) when topo_kappa > 0, then areas, dvol
// and the rotation of stress and strain
template <class R> void move_step(gf_ctx *c, const GfLaunch &g) {
    GfKernels<R>::move_cord(g);
    for (int b = 0; b < c->p.nofbc; ++b) // fl_flexure: the first nbc 200 on the bottom
        if (c->p.nbc[b] == 200 && c->p.nofside[b] == 2) {
            GfRemesh<R>::flexure(g, c->p.bca[b], c->p.bcb[b]);
            break;
        }
    if (c->p.topo_kappa > 0.0)
        GfRemesh<R>::diff_topo(g, c->nloop % c->p.ifreq_avgsr == 0 ? 1 : 0, c->nloop, (int)c->L.max_markers);
    GfKernels<R>::move_elem(g);
}
void k_move(gf_ctx *c, int advance_time = 0) {
    c->frc_valid = 0;
    GfLaunch g = launch_of(c);
    g.advance_time = advance_time;
    if (c->mode == GF_MODE_MIXED) move_step<float>(c, g);
    else move_step<double>(c, g);
}
void k_rmasses(gf_ctx *c) {
    GfLaunch g = launch_of(c);
    if (c->mode == GF_MODE_MIXED) GfKernels<float>::rmasses(g);
    else GfKernels<double>::rmasses(g);
}
void k_dt_mass(gf_ctx *c) {
    GfLaunch g = launch_of(c);
    if (c->mode == GF_MODE_MIXED) GfKernels<float>::dt_mass(g);
    else GfKernels<double>::dt_mass(g);
}
void k_init_visc(gf_ctx *c) {
    GfLaunch g = launch_of(c);
    if (c->mode == GF_MODE_MIXED) GfKernels<float>::init_visc(g);
    else GfKernels<double>::init_visc(g);
}
void k_change_phase(gf_ctx *c) {
    GfLaunch g = launch_of(c);
    if (c->mode == GF_MODE_MIXED) GfKernels<float>::change_phase(g, c->nmarkers);
    else GfKernels<double>::change_phase(g, c->nmarkers);
    if (c->p.itype_melting == 1) GfMagma::melting(g);
}

// The launch sequence of one `flac` call depends only on these flags.
// mesh1 zone patterns of the x and z directions (init_cord.f90:141-179),
// computed on the host exactly as the start-up mesh and kept on the device
int mesh_templates(gf_ctx *c) {
    const gf_params &p = c->p;
    int nex = 0, nez = 0;
    for (int k = 0; k < p.nzonx; ++k) nex += p.nelz_x[k];
    for (int k = 0; k < p.nzony; ++k) nez += p.nelz_y[k];
    std::vector<double> tx((size_t)std::max(nex + 1, p.nx)), tz((size_t)std::max(nez + 1, p.nz));
    gf_host_mesh_template(p.nx, p.nzonx, p.nelz_x, p.sizez_x, tx.data(), &c->ar_x);
    gf_host_mesh_template(p.nz, p.nzony, p.nelz_y, p.sizez_y, tz.data(), &c->ar_z);
    GF_CK(cudaMemcpy(c->rb.tx, tx.data(), sizeof(double) * p.nx, cudaMemcpyHostToDevice));
    GF_CK(cudaMemcpy(c->rb.tz, tz.data(), sizeof(double) * p.nz, cudaMemcpyHostToDevice));
    return GF_OK;
}

GfRemeshArgs remesh_args(const gf_ctx *c) {
    const gf_params &p = c->p;
    GfRemeshArgs a;
    std::memset(&a, 0, sizeof a);
    a.mode_rem = p.mode_rem;
    for (int b = 0; b < p.nofbc; ++b)
        if (p.nbc[b] == 200 && p.nofside[b] == 2) a.is_flex = 1;
    a.has_dhacc = 1;
    a.x0 = p.x0; a.z0 = p.z0; a.rxbo = p.rxbo; a.rzbo = p.rzbo;
    a.ar_x = c->ar_x; a.ar_z = c->ar_z;
    a.incoming_left = p.incoming_left;
    a.incoming_right = p.incoming_right;
    int zl = 0, zr = p.nzone_age > 0 ? p.nzone_age - 1 : 0;
    a.nl_left = std::min(std::max(p.nph_layer[zl], 1), GF_MAXZONE_LAYER);
    a.nl_right = std::min(std::max(p.nph_layer[zr], 1), GF_MAXZONE_LAYER);
    for (int m = 0; m < GF_MAXZONE_LAYER; ++m) {
        a.hc_left[m] = p.hc[zl][m]; a.iph_left[m] = p.iph_col[zl][m];
        a.hc_right[m] = p.hc[zr][m]; a.iph_right[m] = p.iph_col[zr][m];
    }
    a.nloop = c->nloop;
    a.nmarkers = c->nmarkers;
    a.max_markers = (int)c->L.max_markers;
    return a;
}

// sidewalltemp (init_temp.f90:313-353) for material entering through a
// wall: the age zone's geotherm on the three node columns next to it and
// the heat source of the column behind them, on the host
int sidewall_temps(gf_ctx *c) {
    const gf_params &p = c->p;
    const GfDims &d = c->d;
    std::vector<double> cord(2 * d.N), temp(d.N), source(d.E);
    GF_CK(cudaStreamSynchronize(c->s));
    GF_CK(cudaMemcpy(cord.data(), c->A.cord, sizeof(double) * 2 * d.N, cudaMemcpyDeviceToHost));
    GF_CK(cudaMemcpy(temp.data(), c->A.temp, sizeof(double) * d.N, cudaMemcpyDeviceToHost));
    GF_CK(cudaMemcpy(source.data(), c->A.source, sizeof(double) * d.E, cudaMemcpyDeviceToHost));
    gf_layout L = c->L;
    L.cord = cord.data();
    L.temp = temp.data();
    L.source = source.data();
    gf_params pp = p;
    const int idist = 2, nx = p.nx, nz = p.nz;
    if (p.incoming_left == 1) {
        int rc = gf_host_geotherm_columns(&pp, &L, 0, 0, idist);
        if (rc) return rc;
        for (int i = 0; i < idist; ++i)
            for (int j = 0; j < nz - 1; ++j) source[gf_elem(d, j, i)] = source[gf_elem(d, j, idist)];
    }
    if (p.incoming_right == 1) {
        int rc = gf_host_geotherm_columns(&pp, &L, p.nzone_age - 1, nx - 1 - idist, nx - 1);
        if (rc) return rc;
        for (int i = nx - 1 - idist; i < nx - 1; ++i)
            for (int j = 0; j < nz - 1; ++j) source[gf_elem(d, j, i)] = source[gf_elem(d, j, nx - 2 - idist)];
    }
    GF_CK(cudaMemcpy(c->A.temp, temp.data(), sizeof(double) * d.N, cudaMemcpyHostToDevice));
    GF_CK(cudaMemcpy(c->A.source, source.data(), sizeof(double) * d.E, cudaMemcpyHostToDevice));
    return GF_OK;
}

void drop_graphs(gf_ctx *c) {
    for (auto &g : c->graphs) cudaGraphExecDestroy(g.exec);
    c->graphs.clear();
}

// marker2elem's top-up, count_phase_ratio of every element and jmoho; the
// device marker count follows, the host copy is read back by the caller
template <class R> void enqueue_marker2elem(gf_ctx *c, const GfLaunch &g, const GfRemeshArgs &a) {
    GfRemesh<R>::top_up_markers(g, a, c->rb);
    GfKernels<R>::phase_recount_all(g);
    GfRemesh<R>::jmoho(g);
}

template <class R> int enqueue_remesh(gf_ctx *c) {
    c->frc_valid = 0;
    GfLaunch g = launch_of(c);
    GfRemeshArgs a = remesh_args(c);
    GfRemesh<R>::regrid(g, a, c->rb);
    if (c->p.incoming_left == 1 || c->p.incoming_right == 1) {
        int rc = sidewall_temps(c);
        if (rc) return rc;
    }
    GfKernels<R>::split_nodes(g); // new coordinates, interpolated velocities and temperatures
    if (c->p.ivis_present == 1) GfKernels<R>::init_visc(g);
    GfRemesh<R>::init_areas(g);
    GfKernels<R>::rmasses(g);
    GfKernels<R>::dt_mass(g);
    GfRemesh<R>::rebin_markers(g, a, c->rb);
    enqueue_marker2elem<R>(c, g, a);
    return GF_OK;
}

unsigned step_signature(const gf_ctx *c) {
    const gf_params &p = c->p;
    unsigned sig = 0;
    if (p.itherm != 2) {
        sig |= 1u;
        if (c->nloop % p.ifreq_rmasses == 0) sig |= 2u | 16u;
        if (c->nloop % p.ifreq_visc == 0) sig |= 4u;
        if (c->nsrate == p.ifreq_avgsr) sig |= 8u << 8;
        else if (c->nsrate == -1) sig |= 4u << 8;
        if (c->nloop % p.ifreq_imasses == 0) sig |= 32u;
        // resurface: its random seeds use nloop, so such steps run uncaptured
        if (p.movegrid != 0 && p.topo_kappa > 0.0 && c->nloop % p.ifreq_avgsr == 0) sig |= 64u;
    }
    return sig;
}

// Enqueue one step (flac.f90:5-91 + par.f90:84-87) for a signature.
void enqueue_step(gf_ctx *c, unsigned sig) {
    // Mixed path: on steps where fl_rheol and fl_node read nothing that the
    // thermal update writes (no viscosity update, no change_phase, no
    // thermal stress, no Winkler foundation, whose pressure reads the new
    // temperatures), the two thermal sweeps and the boundary pass run on a
    // second stream beside them.  The coefficient pass comes first (it reads
    // the shear heating that fl_rheol's averaging rewrites) and the streams
    // join before fl_move, which changes the mesh the sweeps' boundary pass
    // may read.
    const bool fork = c->mode == GF_MODE_MIXED && c->s2 && (sig & 1u) && !(sig & 2u) && !(sig & 4u) &&
                      c->p.istress_therm == 0 && c->p.nyhydro == 0;
    if (fork) {
        GfLaunch g = launch_of(c);
        GfKernels<float>::therm_prep(g);
        cudaEventRecord(c->ev_fork, c->s);
        cudaStreamWaitEvent(c->s2, c->ev_fork, 0);
        GfLaunch g2 = g;
        g2.s = c->s2;
        GfKernels<float>::therm_sweeps(g2);
        cudaEventRecord(c->ev_join, c->s2);
    } else {
        k_therm(c);
    }
    // par.f90:86 adds the dt that dt_mass may have just changed, so time
    // advances inside fl_move's kernel only on steps without dt_mass
    bool folded = false;
    if (sig & 1u) {
        if (sig & 2u) k_change_phase(c);
        int avg = (sig & (8u << 8)) ? 2 : ((sig & (4u << 8)) ? 1 : 0);
        k_rheol(c, (sig & 4u) ? 1 : 0, avg);
        k_node(c);
        if (fork) cudaStreamWaitEvent(c->s, c->ev_join, 0);
        if (c->p.movegrid != 0) {
            folded = !(sig & 32u);
            k_move(c, folded ? 1 : 0);
        }
        if (sig & 16u) k_rmasses(c);
        if (sig & 32u) k_dt_mass(c);
    }
    if (!folded) {
        k_clock_advance<<<1, 1, 0, c->s>>>(c->dC);
        ++c->launches;
    }
}

// host bookkeeping that mirrors the device's after one step
void advance_host(gf_ctx *c, unsigned sig) {
    if (sig & 1u) {
        if (sig & (8u << 8)) c->nsrate = 0;
        c->nsrate = c->nsrate + 1;
    }
    c->nloop = c->nloop + 1;
}

int run_graph(gf_ctx *c, unsigned sig) {
    for (auto &g : c->graphs)
        if (g.sig == sig) {
            GF_CK(cudaGraphLaunch(g.exec, c->s));
            c->launches += g.nlaunch;
            return GF_OK;
        }
    cudaGraph_t graph;
    long long before = c->launches;
    GF_CK(cudaStreamBeginCapture(c->s, cudaStreamCaptureModeThreadLocal));
    enqueue_step(c, sig);
    GF_CK(cudaStreamEndCapture(c->s, &graph));
    cudaGraphExec_t exec;
    cudaError_t e = cudaGraphInstantiate(&exec, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) return cuda_err(e, "cudaGraphInstantiate");
    long long n = c->launches - before;
    c->launches = before;
    c->graphs.push_back(GraphEntry{sig, exec, n});
    GF_CK(cudaGraphLaunch(exec, c->s));
    c->launches += n;
    return GF_OK;
}

} // namespace

extern "C" {

int gf_create(gf_ctx **out, const gf_params *p, const gf_layout *L, int mode) {
    if (!out || !p || !L) return GF_ERR_ARG;
    *out = nullptr;
    if (mode != GF_MODE_FP64 && mode != GF_MODE_MIXED) return GF_ERR_ARG;
    if (L->nx != p->nx || L->nz != p->nz || L->nphase != p->nphase || p->nx < 2 || p->nz < 2) return GF_ERR_ARG;
    if (p->nystressbc != 0) return GF_ERR_UNSUPPORTED;
    // the magma sub-model runs in FP64 contexts only
    if (p->itype_melting != 0 && (p->itype_melting != 1 || mode == GF_MODE_MIXED)) return GF_ERR_UNSUPPORTED;
    // the flexural bottom (nbc 200) runs in FP64 contexts only
    for (int b = 0; b < p->nofbc; ++b)
        if (mode == GF_MODE_MIXED && p->nbc[b] == 200 && p->nofside[b] == 2) return GF_ERR_UNSUPPORTED;
    if (p->nphase > 32) return GF_ERR_UNSUPPORTED;
    // the mixed kernels index with 32-bit integers: the largest arrays hold
    // 32 entries per element or node (mark_id_elem, the marker arrays)
    if (mode == GF_MODE_MIXED && 32LL * (long long)p->nx * p->nz >= 0x7fffffffLL) return GF_ERR_LIMIT;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        std::fprintf(stderr, "geoflac_gb300: no CUDA device\n");
        return GF_ERR_CUDA;
    }
    gf_ctx *c = new (std::nothrow) gf_ctx();
    if (!c) return GF_ERR_NOMEM;
    c->p = *p;
    c->L = *L;
    c->mode = mode;
    c->d = GfDims{p->nx, p->nz, p->nphase, (long long)p->nx * p->nz, (long long)(p->nx - 1) * (p->nz - 1)};
    c->sweeps = p->therm_sweeps;
    long long N = c->d.N, E = c->d.E, M = L->max_markers;
    int rc = 0;
#define A_(x)                                                                                                          \
    do {                                                                                                               \
        if ((rc = (x))) {                                                                                              \
            gf_destroy(c);                                                                                             \
            return rc;                                                                                                 \
        }                                                                                                              \
    } while (0)
    A_(cuda_err(cudaStreamCreateWithFlags(&c->s, cudaStreamNonBlocking), "cudaStreamCreate"));
    if (mode == GF_MODE_MIXED) {
        A_(cuda_err(cudaStreamCreateWithFlags(&c->s2, cudaStreamNonBlocking), "cudaStreamCreate"));
        A_(cuda_err(cudaEventCreateWithFlags(&c->ev_fork, cudaEventDisableTiming), "cudaEventCreate"));
        A_(cuda_err(cudaEventCreateWithFlags(&c->ev_join, cudaEventDisableTiming), "cudaEventCreate"));
    }
    A_(dalloc(c, &c->dP, 1));
    A_(dalloc(c, &c->dC, 1));
    DevArrays &A = c->A;
    A_(dalloc(c, &A.cord, 2 * N));
    A_(dalloc(c, &A.vel, 2 * N));
    A_(dalloc(c, &A.temp, N));
    A_(dalloc(c, &A.temp0, N));
    A_(dalloc(c, &A.amass, N));
    A_(dalloc(c, &A.rmass, N));
    A_(dalloc(c, &A.bc, 2 * N));
    A_(dalloc(c, &A.ncod, 2 * N));
    A_(dalloc(c, &A.dhacc_correction, p->nx));
    A_(dalloc(c, &A.dhacc, p->nx));
    A_(dalloc(c, &A.extr_acc, p->nx));
    A_(dalloc(c, &A.dtopo, p->nx));
    A_(dalloc(c, &A.q_init, p->nx));
    A_(dalloc(c, &A.vel_flex_old, p->nx));
    A_(dalloc(c, &A.flex, (size_t)12 * p->nx));
    A_(ralloc(c, &A.stress0, 16 * E));
    A_(ralloc(c, &A.area, 4 * E));
    A_(ralloc(c, &A.dvol, 4 * E));
    A_(ralloc(c, &A.strain, 3 * E));
    A_(ralloc(c, &A.se2sr, 3 * E));
    A_(ralloc(c, &A.aps, E));
    A_(ralloc(c, &A.visn, E));
    A_(ralloc(c, &A.e2sr, E));
    A_(ralloc(c, &A.shrheat, E));
    A_(ralloc(c, &A.sshrheat, E));
    A_(dalloc(c, &A.source, E));
    A_(dalloc(c, &A.fmagma, E));
    A_(dalloc(c, &A.fmagma2, E));
    A_(dalloc(c, &A.dike_released, E));
    A_(dalloc(c, &A.phase_ratio, (size_t)p->nphase * E));
    A_(dalloc(c, &A.iphase, E));
    A_(dalloc(c, &A.jmoho, p->nx));
    A_(dalloc(c, &A.mark_a1, M));
    A_(dalloc(c, &A.mark_a2, M));
    A_(dalloc(c, &A.mark_age, M));
    A_(dalloc(c, &A.mark_dead, M));
    A_(dalloc(c, &A.mark_phase, M));
    A_(dalloc(c, &A.mark_ntriag, M));
    A_(dalloc(c, &A.mark_id_elem, (size_t)GF_MAX_MARKERS_PER_ELEM * E));
    A_(dalloc(c, &A.nmark_elem, E));
    A_(dalloc(c, &A.t_delta0, N));
    A_(dalloc(c, &A.t_delta1, N));
    A_(dalloc(c, &A.t_coef, (size_t)18 * E));
    A_(dalloc(c, &A.t_chg, 2 * N));
    if (mode == GF_MODE_FP64) A_(dalloc(c, &A.t_pred, N));
    A_(dalloc(c, &c->therm_bar, 4));
    A_(dalloc(c, &A.e_dens, E));
    A_(dalloc(c, &A.e_tri, 4 * E));
    A_(dalloc(c, &A.p_ref, E));
    A_(dalloc(c, &A.e_rho, E));
    A_(dalloc(c, &A.e_flag, E));
    A_(dalloc(c, &A.nmarkers, 1));
    A_(dalloc(c, &c->d_angle, 1));
    A_(dalloc(c, &A.cord_old, 2 * N));
    A_(dalloc(c, &A.orig, 2 * N));
    if (p->itype_melting == 1) {
        A_(dalloc(c, &A.fmelt, E));
        A_(dalloc(c, &A.fmelt2, E));
        A_(dalloc(c, &A.dike_added, E));
        A_(dalloc(c, &A.dike_backlog, E));
        A_(dalloc(c, &A.dike_marker_vol, E));
        A_(dalloc(c, &A.mor_marker_vol, E));
        A_(dalloc(c, &A.extrusion, p->nx));
        A_(dalloc(c, &A.mg_e, E));
        A_(dalloc(c, &A.mg_src, (size_t)GF_MG_SRC_W * E));
        A_(dalloc(c, &A.mg_src2, (size_t)GF_MG_SRC_W * E));
        A_(dalloc(c, &A.mg_list2, E));
        A_(dalloc(c, &A.mg_order, 6 * E));
        A_(dalloc(c, &A.mg_s, 16));
        A_(dalloc(c, &A.mg_c, p->nx));
        A_(dalloc(c, &A.mg_list, E));
        A_(dalloc(c, &A.mg_blk, E / 1024 + 2));
        A_(dalloc(c, &A.mg_i, 32));
        A_(dalloc(c, &A.mg_col, 2 * p->nx));
        A_(dalloc(c, &A.mg_mask, E));
    }
    {
        GfRemeshBufs &b = c->rb;
        A_(dalloc(c, &b.tx, p->nx));
        A_(dalloc(c, &b.tz, p->nz));
        A_(dalloc(c, &b.cold, 2 * E));
        A_(dalloc(c, &b.cnew, 2 * E));
        A_(dalloc(c, &b.pt, 12 * E));
        A_(dalloc(c, &b.numtr, N));
        A_(dalloc(c, &b.bc, 3 * N));
        A_(dalloc(c, &b.plane, N));
        A_(dalloc(c, &b.m_elem, M));
        A_(dalloc(c, &b.m_slot, M));
        A_(dalloc(c, &b.e_count, E));
        A_(dalloc(c, &b.e_offset, E + 1));
        A_(dalloc(c, &b.e_fill, E));
        A_(dalloc(c, &b.d_scalars, 4));
        A_(mesh_templates(c));
    }
    if (mode == GF_MODE_FP64) {
        A_(dalloc(c, &A.n_frc, 24 * E));
        double *tab = nullptr;
        A_(dalloc(c, &tab, GF_PT_STATES * GF_MAXPH * GF_PT_W));
        A.plast_tab = tab;
    } else {
        float *tab = nullptr;
        A_(dalloc(c, &tab, GF_PT_STATES * GF_MAXPH * GF_PT_W));
        A.plast_tab = tab;
    }
    if (mode == GF_MODE_MIXED) {
        A_(dalloc(c, &c->staging, 16 * E));
        A_(dalloc(c, &A.cord_hi, 2 * N));
        A_(dalloc(c, &A.cord_lo, 2 * N));
        A_(dalloc(c, &A.vel_hi, 2 * N));
        A_(dalloc(c, &A.vel_lo, 2 * N));
        A_(dalloc(c, &A.pr_hi, E));
        A_(dalloc(c, &A.pr_lo, E));
        A_(dalloc(c, &A.e_frc, 16 * E));
        A_(dalloc(c, &A.temp_hi, N));
        A_(dalloc(c, &A.temp_lo, N));
    }
    DevParams P;
    fill_params(P, *p);
    A_(cuda_err(cudaMemcpy(c->dP, &P, sizeof P, cudaMemcpyHostToDevice), "params"));
    if (mode == GF_MODE_FP64)
        GfKernels<double>::plastic_table(launch_of(c));
    else
        GfKernels<float>::plastic_table(launch_of(c));
    A_(cuda_err(cudaGetLastError(), "plastic table"));
    DevClock C0;
    std::memset(&C0, 0, sizeof C0);
    C0.frac = p->frac;
    A_(cuda_err(cudaMemcpy(c->dC, &C0, sizeof C0, cudaMemcpyHostToDevice), "clock"));
#undef A_
    *out = c;
    return GF_OK;
}

void gf_destroy(gf_ctx *c) {
    if (!c) return;
    if (c->s) cudaStreamSynchronize(c->s);
    for (auto &g : c->graphs) cudaGraphExecDestroy(g.exec);
    for (void *p : c->allocs) cudaFree(p);
    if (c->s2) {
        cudaStreamSynchronize(c->s2);
        cudaStreamDestroy(c->s2);
    }
    if (c->ev_fork) cudaEventDestroy(c->ev_fork);
    if (c->ev_join) cudaEventDestroy(c->ev_join);
    if (c->s) cudaStreamDestroy(c->s);
    delete c;
}

int gf_upload(gf_ctx *c, unsigned mask) {
    if (!c) return GF_ERR_ARG;
    return move_fields(c, mask, 1);
}

int gf_download(gf_ctx *c, unsigned mask) {
    if (!c) return GF_ERR_ARG;
    return move_fields(c, mask, 0);
}

int gf_set_params(gf_ctx *c, const gf_params *p) {
    if (!c || !p) return GF_ERR_ARG;
    if (p->nx != c->p.nx || p->nz != c->p.nz || p->nphase != c->p.nphase) return GF_ERR_ARG;
    c->p = *p;
    c->sweeps = p->therm_sweeps;
    DevParams P;
    fill_params(P, *p);
    GF_CK(cudaStreamSynchronize(c->s));
    GF_CK(cudaMemcpy(c->dP, &P, sizeof P, cudaMemcpyHostToDevice));
    if (c->mode == GF_MODE_FP64)
        GfKernels<double>::plastic_table(launch_of(c));
    else
        GfKernels<float>::plastic_table(launch_of(c));
    GF_CK(cudaGetLastError());
    for (auto &g : c->graphs) cudaGraphExecDestroy(g.exec);
    c->graphs.clear();
    return GF_OK;
}

int gf_get_params(gf_ctx *c, gf_params *p) {
    if (!c || !p) return GF_ERR_ARG;
    *p = c->p;
    return GF_OK;
}

int gf_set_clock(gf_ctx *c, const gf_clock *k) {
    if (!c || !k) return GF_ERR_ARG;
    GF_CK(cudaStreamSynchronize(c->s));
    DevClock C;
    GF_CK(cudaMemcpy(&C, c->dC, sizeof C, cudaMemcpyDeviceToHost));
    C.dt = k->dt; C.time = k->time; C.dtavg = k->dtavg; C.dt_elastic = k->dt_elastic;
    C.dt_maxwell = k->dt_maxwell; C.dtmax_therm = k->dtmax_therm; C.frac = k->frac;
    C.vel_max = k->vel_max; C.dlmin = k->dlmin;
    GF_CK(cudaMemcpy(c->dC, &C, sizeof C, cudaMemcpyHostToDevice));
    c->nloop = k->nloop;
    c->nsrate = k->nsrate;
    c->nmarkers = k->nmarkers;
    c->need_remeshing = k->need_remeshing;
    return GF_OK;
}

int gf_get_clock(gf_ctx *c, gf_clock *k) {
    if (!c || !k) return GF_ERR_ARG;
    GF_CK(cudaStreamSynchronize(c->s));
    DevClock C;
    GF_CK(cudaMemcpy(&C, c->dC, sizeof C, cudaMemcpyDeviceToHost));
    k->dt = C.dt; k->time = C.time; k->dtavg = C.dtavg; k->dt_elastic = C.dt_elastic;
    k->dt_maxwell = C.dt_maxwell; k->dtmax_therm = C.dtmax_therm; k->frac = C.frac;
    k->vel_max = C.vel_max; k->dlmin = C.dlmin;
    k->therm_sweeps = C.therm_sweeps_used;
    k->therm_unconverged = C.therm_unconverged;
    k->nloop = c->nloop;
    k->nsrate = c->nsrate;
    k->nmarkers = c->nmarkers;
    k->need_remeshing = c->need_remeshing;
    return GF_OK;
}

// One reference subroutine per entry point; each waits for its kernels and
// returns the device status (the reference's stop code where it would stop).
static int sync_markers_after_resurface(gf_ctx *c);

int gf_fl_therm(gf_ctx *c) {
    if (!c) return GF_ERR_ARG;
    const bool magma = c->mode == GF_MODE_FP64 && c->p.itype_melting == 1; // may add markers
    if (magma) GF_CK(cudaMemcpyAsync(c->A.nmarkers, &c->nmarkers, sizeof(int), cudaMemcpyHostToDevice, c->s));
    k_therm(c);
    if (magma) {
        int rc = sync_markers_after_resurface(c);
        if (rc) return rc;
    }
    return call_status(c);
}

int gf_change_phase(gf_ctx *c) {
    if (!c) return GF_ERR_ARG;
    k_change_phase(c);
    return call_status(c);
}

int gf_fl_rheol(gf_ctx *c) {
    if (!c) return GF_ERR_ARG;
    const gf_params &p = c->p;
    int avg = (c->nsrate == p.ifreq_avgsr) ? 2 : (c->nsrate == -1 ? 1 : 0);
    k_rheol(c, c->nloop % p.ifreq_visc == 0, avg);
    if (avg == 2) c->nsrate = 0;
    c->nsrate = c->nsrate + 1;
    return call_status(c);
}

int gf_fl_node(gf_ctx *c) {
    if (!c) return GF_ERR_ARG;
    k_node(c);
    return call_status(c);
}

int gf_fl_move(gf_ctx *c) {
    if (!c) return GF_ERR_ARG;
    if (c->p.movegrid == 0) return GF_OK;
    const bool resurf = c->p.topo_kappa > 0.0 && c->nloop % c->p.ifreq_avgsr == 0;
    if (resurf) GF_CK(cudaMemcpyAsync(c->A.nmarkers, &c->nmarkers, sizeof(int), cudaMemcpyHostToDevice, c->s));
    k_move(c);
    if (resurf) {
        int rc = sync_markers_after_resurface(c);
        if (rc) return rc;
    }
    return call_status(c);
}

int gf_rmasses(gf_ctx *c) {
    if (!c) return GF_ERR_ARG;
    k_rmasses(c);
    return call_status(c);
}

int gf_dt_mass(gf_ctx *c) {
    if (!c) return GF_ERR_ARG;
    k_dt_mass(c);
    return call_status(c);
}

int gf_init_visc(gf_ctx *c) {
    if (!c) return GF_ERR_ARG;
    k_init_visc(c);
    return call_status(c);
}

int gf_marker2elem(gf_ctx *c) {
    if (!c) return GF_ERR_ARG;
    GF_CK(cudaMemcpyAsync(c->A.nmarkers, &c->nmarkers, sizeof(int), cudaMemcpyHostToDevice, c->s));
    GfLaunch g = launch_of(c);
    GfRemeshArgs a = remesh_args(c);
    if (c->mode == GF_MODE_MIXED)
        enqueue_marker2elem<float>(c, g, a);
    else
        enqueue_marker2elem<double>(c, g, a);
    GF_CK(cudaMemcpyAsync(&c->nmarkers, c->A.nmarkers, sizeof(int), cudaMemcpyDeviceToHost, c->s));
    GF_CK(cudaStreamSynchronize(c->s));
    drop_graphs(c); // change_phase's launch covers nmarkers markers
    return take_status(c);
}

int gf_finish_setflac(gf_ctx *c) {
    if (!c) return GF_ERR_ARG;
    // xoriginal = cord(:,:,1), zoriginal = cord(:,:,2) (setflac.f90:54-55)
    // (when the host layout does not provide the start-up positions)
    if (!c->L.xoriginal || !c->L.zoriginal)
        GF_CK(cudaMemcpyAsync(c->A.orig, c->A.cord, sizeof(double) * 2 * c->d.N, cudaMemcpyDeviceToDevice, c->s));
    k_rmasses(c);
    if (c->p.ivis_present == 1) k_init_visc(c);
    k_dt_mass(c);
    int st = take_status(c);
    if (st) return st;
    gf_clock k;
    int rc = gf_get_clock(c, &k);
    if (rc) return rc;
    k.dtavg = 0.0;
    k.nsrate = -1;
    return gf_set_clock(c, &k);
}

int gf_flac(gf_ctx *c) {
    if (!c) return GF_ERR_ARG;
    unsigned sig = step_signature(c);
    // the magma sub-model's fl_therm may add markers: the host count is
    // re-read after every call, so that it is current for the next one
    const bool resync = (sig & 64u) || (c->mode == GF_MODE_FP64 && c->p.itype_melting == 1);
    if (resync) GF_CK(cudaMemcpyAsync(c->A.nmarkers, &c->nmarkers, sizeof(int), cudaMemcpyHostToDevice, c->s));
    enqueue_step(c, sig);
    if (resync) {
        int rc = sync_markers_after_resurface(c);
        if (rc) return rc;
    }
    advance_host(c, sig);
    return call_status(c);
}

int gf_ctx_view(gf_ctx *c, GfMemberView *v) {
    if (!c || !v) return GF_ERR_ARG;
    v->P = c->dP;
    v->C = c->dC;
    v->A = c->A;
    v->d = c->d;
    v->mode = c->mode;
    v->idt_scale = c->p.idt_scale;
    v->movegrid = c->p.movegrid;
    v->itherm = c->p.itherm;
    v->nmarkers = c->nmarkers;
    v->nloop = c->nloop;
    v->nsrate = c->nsrate;
    v->ifreq_rmasses = c->p.ifreq_rmasses;
    v->ifreq_visc = c->p.ifreq_visc;
    v->ifreq_imasses = c->p.ifreq_imasses;
    v->ifreq_avgsr = c->p.ifreq_avgsr;
    v->z0 = c->p.z0;
    v->rzbo = c->p.rzbo;
    v->g = c->p.g;
    v->s = c->s;
    v->hp = &c->p;
    v->L = &c->L;
    return GF_OK;
}

} // extern "C"
namespace {
template <class R> __global__ void k_fill(R *p, long long n, R v) {
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n) p[t] = v;
}
template <class R> void restart_fields(gf_ctx *c) {
    const long long E = c->d.E, N = c->d.N;
    auto nb = [](long long n) { return (unsigned)((n + 255) / 256); };
    k_fill<R><<<nb(E), 256, 0, c->s>>>((R *)c->A.shrheat, E, R(0));
    k_fill<R><<<nb(E), 256, 0, c->s>>>((R *)c->A.sshrheat, E, R(0));
    k_fill<R><<<nb(3 * E), 256, 0, c->s>>>((R *)c->A.se2sr, 3 * E, R(1e-16));
    k_fill<R><<<nb(E), 256, 0, c->s>>>((R *)c->A.e2sr, E, R(1e-16));
    k_fill<R><<<nb(4 * E), 256, 0, c->s>>>((R *)c->A.dvol, 4 * E, R(0));
    cudaMemcpyAsync(c->A.temp0, c->A.temp, sizeof(double) * N, cudaMemcpyDeviceToDevice, c->s);
    c->launches += 5;
}
} // namespace
extern "C" {

int gf_ctx_restart_finish(gf_ctx *c) {
    if (!c) return GF_ERR_ARG;
    int rc;
    GfLaunch g = launch_of(c);
    if (c->mode == GF_MODE_MIXED) {
        GfRemesh<float>::init_areas(g);
        restart_fields<float>(c);
    } else {
        GfRemesh<double>::init_areas(g);
        restart_fields<double>(c);
    }
    rc = take_status(c);
    if (rc) return rc;
    k_rmasses(c);
    if (c->p.ivis_present == 1) k_init_visc(c);
    k_dt_mass(c);
    rc = take_status(c);
    if (rc) return rc;
    DevClock C;
    GF_CK(cudaMemcpy(&C, c->dC, sizeof C, cudaMemcpyDeviceToHost));
    C.dtavg = 0.0;
    GF_CK(cudaMemcpy(c->dC, &C, sizeof C, cudaMemcpyHostToDevice));
    c->nsrate = -1;
    drop_graphs(c);
    return GF_OK;
}

unsigned gf_ctx_signature(const gf_ctx *c) { return step_signature(c); }

void gf_ctx_advance(gf_ctx *c, unsigned sig) {
    c->frc_valid = 0; // the batch step moved the mesh after its own gather
    advance_host(c, sig);
}

int gf_ctx_take_status(gf_ctx *c) { return take_status(c); }

void gf_ctx_invalidate_forces(gf_ctx *c) { c->frc_valid = 0; }

// After a step with resurface or the magma sub-model: the device marker
// count is the current one (both add markers); graphs whose change_phase
// launch covers an older count are dropped.
static int sync_markers_after_resurface(gf_ctx *c) {
    int nm = c->nmarkers;
    GF_CK(cudaMemcpyAsync(&nm, c->A.nmarkers, sizeof(int), cudaMemcpyDeviceToHost, c->s));
    GF_CK(cudaStreamSynchronize(c->s));
    if (nm != c->nmarkers) {
        c->nmarkers = nm;
        drop_graphs(c);
    }
    return GF_OK;
}

int gf_step(gf_ctx *c, int nsteps) {
    if (!c || nsteps < 0) return GF_ERR_ARG;
    // The magma sub-model's fl_therm may add markers on any step (device
    // count).  Its steps are graph-replayed too; the host copy of the count
    // is brought up to date before a step that uses it (change_phase's
    // launch, a resurface step) and at the end.
    const bool magma = c->mode == GF_MODE_FP64 && c->p.itype_melting == 1;
    if (magma) // the host count is current between calls
        GF_CK(cudaMemcpyAsync(c->A.nmarkers, &c->nmarkers, sizeof(int), cudaMemcpyHostToDevice, c->s));
    for (int k = 0; k < nsteps; ++k) {
        unsigned sig = step_signature(c);
        if (magma && (sig & (2u | 64u))) {
            int rc = sync_markers_after_resurface(c);
            if (rc) return rc;
        }
        if (sig & 64u) { // resurface: uncaptured (its seeds use nloop)
            GF_CK(cudaMemcpyAsync(c->A.nmarkers, &c->nmarkers, sizeof(int), cudaMemcpyHostToDevice, c->s));
            enqueue_step(c, sig);
            int rc = sync_markers_after_resurface(c);
            if (rc) return rc;
        } else {
            int rc = run_graph(c, sig);
            if (rc) return rc;
        }
        advance_host(c, sig);
    }
    if (magma) {
        int rc = sync_markers_after_resurface(c);
        if (rc) return rc;
    }
    return take_status(c);
}

int gf_itest_mesh(gf_ctx *c, double *min_angle) {
    if (!c) return GF_ERR_ARG;
    double init = 180.0;
    GF_CK(cudaMemcpyAsync(c->d_angle, &init, sizeof init, cudaMemcpyHostToDevice, c->s));
    GfLaunch g = launch_of(c);
    GfKernels<double>::min_angle(g, c->d_angle);
    double a = 0.0;
    GF_CK(cudaMemcpyAsync(&a, c->d_angle, sizeof a, cudaMemcpyDeviceToHost, c->s));
    GF_CK(cudaStreamSynchronize(c->s));
    if (min_angle) *min_angle = a;
    // rem_test.f90:23-66: shortening (code 2), surface topography change
    // (code 3), before the angle (code 1)
    const gf_params &p = c->p;
    const int nx = p.nx;
    const long long N = c->d.N;
    int need = 0;
    if (p.mode_rem == 11 || p.mode_rem == 3) {
        double x0 = 0.0, xn = 0.0;
        GF_CK(cudaMemcpy(&x0, c->A.cord + gf_node(c->d, 0, 0), sizeof(double), cudaMemcpyDeviceToHost));
        GF_CK(cudaMemcpy(&xn, c->A.cord + gf_node(c->d, 0, nx - 1), sizeof(double), cudaMemcpyDeviceToHost));
        double testcr = p.dx_rem * p.rxbo / (nx - 1);
        double shortening = std::fabs(xn - x0 - p.rxbo);
        if (shortening > testcr) need = 2;
    }
    const double arc_extrusion_rate = 1.0 - p.ratio_mantle_mzone;
    if (need == 0 && (p.topo_kappa > 0 || arc_extrusion_rate > 0)) {
        std::vector<double> dh(nx), ex(nx);
        double z00 = 0.0, z10 = 0.0;
        GF_CK(cudaMemcpy(dh.data(), c->A.dhacc, sizeof(double) * nx, cudaMemcpyDeviceToHost));
        GF_CK(cudaMemcpy(ex.data(), c->A.extr_acc, sizeof(double) * nx, cudaMemcpyDeviceToHost));
        GF_CK(cudaMemcpy(&z00, c->A.cord + N + gf_node(c->d, 0, 0), sizeof(double), cudaMemcpyDeviceToHost));
        GF_CK(cudaMemcpy(&z10, c->A.cord + N + gf_node(c->d, 1, 0), sizeof(double), cudaMemcpyDeviceToHost));
        for (int i = 0; i < nx - 1; ++i) {
            double testcr = (z00 - z10) * 0.3333;
            double topochanges = std::fabs(dh[i]) + ex[i];
            if (topochanges > testcr) need = 3;
        }
    }
    if (need == 0 && a <= p.angle_rem) need = 1;
    c->need_remeshing = need;
    return GF_OK;
}

int gf_remesh(gf_ctx *c) {
    if (!c) return GF_ERR_ARG;
    const int mr = c->p.mode_rem;
    if (!(mr == 1 || mr == 3 || mr == 4 || mr == 11)) return GF_ERR_UNSUPPORTED;
    if (c->p.nx < 4 || c->p.nz < 3) return GF_ERR_UNSUPPORTED; // element-centre grid needs 2 x 3 cells
    GF_CK(cudaMemcpyAsync(c->A.nmarkers, &c->nmarkers, sizeof(int), cudaMemcpyHostToDevice, c->s));
    int rc = c->mode == GF_MODE_MIXED ? enqueue_remesh<float>(c) : enqueue_remesh<double>(c);
    if (rc) return rc;
    GF_CK(cudaMemsetAsync(c->A.dhacc_correction, 0, sizeof(double) * c->p.nx, c->s));
    GF_CK(cudaMemcpyAsync(&c->nmarkers, c->A.nmarkers, sizeof(int), cudaMemcpyDeviceToHost, c->s));
    GF_CK(cudaStreamSynchronize(c->s));
    drop_graphs(c);
    c->need_remeshing = 0;
    return take_status(c);
}

int gf_set_sync(gf_ctx *c, int sync) {
    if (!c) return GF_ERR_ARG;
    c->sync = sync ? 1 : 0;
    return GF_OK;
}

void *gf_stream(gf_ctx *c) { return c ? (void *)c->s : nullptr; }

int gf_status(gf_ctx *c) {
    if (!c) return GF_ERR_ARG;
    return take_status(c);
}

long long gf_launch_count(gf_ctx *c) { return c ? c->launches : 0; }

const char *gf_strerror(int code) {
    switch (code) {
    case GF_OK: return "ok";
    case GF_ERR_CUDA: return "CUDA error";
    case GF_ERR_ARG: return "bad argument";
    case GF_ERR_IO: return "cannot open file";
    case GF_ERR_PARSE: return "malformed .inp file";
    case GF_ERR_UNSUPPORTED: return "feature not supported by the GPU path";
    case GF_ERR_TIMEOUT: return "device wait timed out";
    case GF_ERR_NOMEM: return "out of memory";
    case GF_ERR_NONFINITE: return "non-finite value";
    case GF_ERR_LIMIT: return "input larger than the fixed device scratch (gf_min_angle_noalloc: 2,097,152 elements at most)";
    case 22: return "Maxwell: time step too large (reference stop 22)";
    case 40: return "negative area (reference stop 40)";
    case 41: return "negative area at start-up (reference stop 41)";
    case 133: return "marker top-up failed (reference stop 133)";
    case 134: return "no markers in an element";
    default: return code > 0 ? "reference stop code" : "unknown error";
    }
}

} // extern "C"
