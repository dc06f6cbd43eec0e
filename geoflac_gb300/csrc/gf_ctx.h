// Device-side state of one model (one gf_ctx) and the kernel launchers.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/geoflac_gb300.h"
#include "gf_index.h"

#define GF_THREADS 256
#define GF_THREADS_MAX 512 // the largest CTA of any kernel (the ensemble step's)
#define GF_THERM_KMAX 24 // cap on the thermal fixed-point sweeps per fl_therm

// Read-only model constants the kernels use (copied once per context into
// device global memory; every thread of a warp reads the same entries).
struct DevParams {
    int nx, nz, nphase;
    int ndim, mix_strain, mix_stress, istress_therm, ishearh, itherm, itemp_bc;
    int nyhydro, iphsub, i_prestress, idt_scale, i_rey, ivis_present, itype_melting;
    int nystressbc, movegrid, nelem_serp, eclogite_rule, ninh100;
    int irheol[GF_MAXPH];
    double rl[GF_MAXPH], rm[GF_MAXPH], den[GF_MAXPH], alfa[GF_MAXPH], beta[GF_MAXPH], pln[GF_MAXPH],
        acoef[GF_MAXPH], eactiv[GF_MAXPH], vactiv[GF_MAXPH], plstrain1[GF_MAXPH], plstrain2[GF_MAXPH],
        fric1[GF_MAXPH], fric2[GF_MAXPH], cohesion1[GF_MAXPH], cohesion2[GF_MAXPH], dilat1[GF_MAXPH],
        dilat2[GF_MAXPH], conduct[GF_MAXPH], cp[GF_MAXPH];
    // Eff_visc fixed weak zones (igeom == 100), 1-based element ranges
    int w_ix1[GF_MAXINH], w_ix2[GF_MAXINH], w_iy1[GF_MAXINH], w_iy2[GF_MAXINH];
    double g, demf, ten_off, tau_heal, v_min, v_max, t_top, t_bot, bot_bc, pisos, drosub, rzbo, rxbo, vbc,
        fmagma_max, rho_magma, weaken_ratio_plastic, weaken_ratio_viscous, xReyn, strain_inert, dt_scale, fracm;
    // FP32 copies of the per-phase constants for the mixed kernels
    // (f_lacoef = log(0.75 * acoef), f_bulkm = rl + 2/3 rm)
    float f_bulkm[GF_MAXPH], f_rm[GF_MAXPH], f_fric1[GF_MAXPH], f_fric2[GF_MAXPH], f_coh1[GF_MAXPH],
        f_coh2[GF_MAXPH], f_dil1[GF_MAXPH], f_dil2[GF_MAXPH], f_pl1[GF_MAXPH], f_pl2[GF_MAXPH], f_cp[GF_MAXPH],
        f_cond[GF_MAXPH], f_den[GF_MAXPH], f_pln[GF_MAXPH], f_lacoef[GF_MAXPH], f_eactiv[GF_MAXPH],
        f_vactiv[GF_MAXPH];
    float f_ten_off, f_demf, f_g, f_tau_heal;
    float f_alfa[GF_MAXPH], f_beta[GF_MAXPH], f_fmagma_max, f_rho_magma;
    double diffu[GF_MAXPH]; // conduct / den / cp (dt_mass.f90:130)
    double bulkm[GF_MAXPH]; // rl + 2 rm / 3 (fl_rheol.f90:192)
    double hsoft[GF_MAXPH]; // (cohesion2 - cohesion1) / (plstrain2 - plstrain1) (rh_plastic.f90:264)
    // shear heating's per-phase factors (fl_rheol.f90:344-361): lambda / den_el
    // and the reciprocal pair of 2 mu
    double sh_lam_den[GF_MAXPH], sh_r2mu_y[GF_MAXPH], sh_r2mu_yl[GF_MAXPH];
    double topo_kappa, erodibility[GF_MAXPH]; // surface processes (diff_topo)
    // magma sub-model (itype_melting = 1)
    double prod_magma, prod_magma2, angle_mzone, ratio_mantle_mzone, ratio_crust_mzone, latent_heat_magma,
        lambda_freeze, lambda_freeze_tdep, dxmin, Amin;
    int nelem_dike;
};

// Scalars the step reads and writes, resident on the device so that a
// captured step needs no host round trip.
struct DevClock {
    double dt, time, dtavg;
    double dt_elastic, dt_maxwell, dtmax_therm, frac, vel_max, dlmin;
    // reduction slots (bit patterns of non-negative doubles order like ints)
    unsigned long long r_dlmin, r_velmax, r_diffmax;
    long long frac_writer; // serial position + 1 of the last Eff_dens that wrote frac
    unsigned int phase_mask;
    int status;     // first error code (reference stop code or GF_ERR_*)
    int status_aux; // element/node index of the first error
    int therm_sweeps_used;  // sweeps of the last fl_therm (converged at the last)
    int therm_unconverged;  // fl_therm calls that hit the sweep cap
    int therm_flags[GF_THERM_KMAX]; // sweep k changed some value
};

// Device arrays of a context.  In GF_MODE_MIXED the element fields listed
// under "R" are FP32 (R = float); in GF_MODE_FP64 everything is double.
#define GF_PT_STATES 3 // plastic strain before, at the start of, after softening
#define GF_PT_W 8

struct DevArrays {
    // node fields (always FP64: coordinates, temperature, masses)
    double *cord, *vel, *temp, *temp0, *amass, *rmass, *bc;
    int *ncod;
    double *dhacc_correction;
    double *dhacc, *extr_acc, *dtopo; // surface processes (nx each)
    double *q_init, *vel_flex_old;    // flexural bottom (nx each)
    double *flex;                     // flexure scratch (12 nx)
    // element fields stored as R
    void *stress0, *area, *dvol, *strain, *se2sr, *aps, *visn, *e2sr, *shrheat, *sshrheat;
    // element fields always FP64
    double *source, *fmagma, *fmagma2, *dike_released, *phase_ratio;
    int *iphase, *jmoho;
    // markers
    double *mark_a1, *mark_a2, *mark_age;
    int8_t *mark_dead, *mark_phase;
    int *mark_ntriag, *mark_id_elem, *nmark_elem;
    // scratch
    double *t_delta0, *t_delta1; // thermal sweep iterates (node)
    double *t_coef;              // thermal per-element coefficients (18 per element)
    uint8_t *t_chg;              // FP64 thermal sweeps: node changed in sweep k (2 x N, by parity)
    double *t_pred;              // FP64 thermal sweeps: each node's last increment (the next start)
    double *p_ref; // mixed: per-element reference pressure; stored normal stresses are total + p_ref
    double *e_dens;                                   // per-element density (rmasses)
    double *e_tri;                                    // per-triangle mass shares (4 per element)
    double *e_rho;                                    // per-element inertial density (dt_mass)
    uint8_t *e_flag;                                  // change_phase element flags
    int *m_count, *m_offset;                          // marker2elem scan
    double *cord_old;                                 // remesh
    double *orig; // xoriginal, zoriginal (nz, nx, 2): start-up node positions carried through remeshing
    // mixed: FP32 hi/lo splits of the FP64 coordinates and velocities
    // (x = hi + lo), so differences of neighbouring values need no FP64
    float *cord_hi, *cord_lo, *vel_hi, *vel_lo;
    float *pr_hi, *pr_lo;     // the same split of p_ref
    float *temp_hi, *temp_lo; // and of the temperatures
    // mixed: per-element corner forces for the node gather, [16][E]: for
    // corner c (0..3) the force of the element's stresses less its own
    // triangle-1 stress (x, z) and the geometric sums G (x, z)
    float *e_frc;
    // FP64: each element's terms of fl_node's force sum (fl_node.f90:50-254),
    // written by fl_rheol from the new stresses: for corner c and the k-th
    // of its three triangles, fx at [(6c + 2k) E + e], fy at [(6c + 2k + 1) E + e]
    double *n_frc;
    // plastic constants of single-phase elements, [GF_PT_STATES][GF_MAXPH][GF_PT_W]
    // (anphi, anpsi, amc, e1, e2, x1, ten_max, hardn per phase and strain
    // branch), in the element fields' precision
    void *plast_tab;
    int *nmarkers;                                    // device marker count
    // magma sub-model (allocated when itype_melting = 1): melt fractions,
    // dike / MOR accumulators (E each), the last arc extrusion (nx), and
    // scratch: per-element values (E), per-source / per-candidate records
    // (GF_MG_SRC_W x E, two lists), zone scalars, per-column values (nx),
    // ordered element lists (E, two) with their block counts, element masks (E)
    double *fmelt, *fmelt2, *dike_added, *dike_backlog, *dike_marker_vol, *mor_marker_vol, *extrusion;
    double *mg_e, *mg_src, *mg_src2, *mg_s, *mg_c;
    int *mg_list, *mg_list2, *mg_blk, *mg_i, *mg_col;
    int *mg_order; // melting walk order per loop, flux order, level-sorted candidates (6 E)
    uint8_t *mg_mask;
};

#define GF_MG_SRC_W 16 // doubles per migration source / melting candidate

struct GfLaunch {
    const DevParams *P;
    DevClock *C;
    DevArrays A;
    GfDims d;
    cudaStream_t s;
    long long *launches;
    int idt_scale;   // host copy of the mass-scaling mode (selects launches)
    int advance_time; // fold par.f90's time += dt into the step's last kernel
    double arc_rate;  // arc extrusion rate 1 - ratio_mantle_mzone - ratio_crust_mzone (diff_topo)
    unsigned *therm_bar; // grid barrier of the FP64 thermal sweeps (arrivals, generation, error flag)
    int node_terms;      // FP64 fl_node: A.n_frc holds the terms of the current stresses and mesh
};

// Launchers, one set per precision (template instantiated in its own TU).
template <class R> struct GfKernels {
    // keep_temp0: temp0 was taken before the magma sub-model changed temp
    static void therm(const GfLaunch &g, int sweeps, int keep_temp0 = 0);
    // mixed: the coefficient pass and the two sweeps + boundary pass of
    // therm, for steps that run the sweeps beside fl_rheol / fl_node
    static void therm_prep(const GfLaunch &g);
    static void therm_sweeps(const GfLaunch &g);
    static void rheol(const GfLaunch &g, int update_visc, int avg_mode);
    static void node(const GfLaunch &g);
    // mixed: the corner forces of the current stresses (fl_rheol writes them
    // as it updates the stresses; this recomputes them after other changes)
    static void elem_forces(const GfLaunch &g);
    static void move(const GfLaunch &g);
    // fl_move in two parts, for diff_topo between them
    static void move_cord(const GfLaunch &g);
    static void move_elem(const GfLaunch &g);
    static void rmasses(const GfLaunch &g);
    static void dt_mass(const GfLaunch &g);
    static void init_visc(const GfLaunch &g);
    static void change_phase(const GfLaunch &g, int nmarkers);
    static void min_angle(const GfLaunch &g, double *d_out);
    static void convert_in(const GfLaunch &g, unsigned mask, const double *src, void *dst, long long n);
    // mixed: total stress (FP64 staging) <-> stored deviations from -p_ref
    static void stress_in(const GfLaunch &g, const double *src);
    static void stress_out(const GfLaunch &g, double *dst);
    // count_phase_ratio of every element (marker2elem.f90:58)
    static void phase_recount_all(const GfLaunch &g);
    // refresh the hi/lo splits after the FP64 coordinates / velocities changed
    static void split_nodes(const GfLaunch &g);
    // the per-phase plastic constants of single-phase elements, after every
    // upload of the model constants
    static void plastic_table(const GfLaunch &g);
};

// Remesh event (par.f90:94-110): host-prepared constants, passed by value.
struct GfRemeshArgs {
    int mode_rem, is_flex, has_dhacc;
    double x0, z0, rxbo, rzbo;
    double ar_x, ar_z; // mesh1 zone-pattern totals (init_cord.f90:141-179)
    int incoming_left, incoming_right;
    int nl_left, nl_right; // nph_layer of the first / last age zone
    double hc_left[GF_MAXZONE_LAYER], hc_right[GF_MAXZONE_LAYER];
    int iph_left[GF_MAXZONE_LAYER], iph_right[GF_MAXZONE_LAYER];
    int nloop, nmarkers, max_markers;
};

// Device scratch of the remesh event (allocated with the context).
struct GfRemeshBufs {
    double *tx, *tz;     // mesh1 zone patterns along x (nx) and z (nz)
    double *cold, *cnew; // element centres, old and new mesh (2 planes of E)
    double *pt;          // 6 barycentric coefficients per old-mesh triangle
    int *numtr;          // containing old triangle (1-based) per new point
    double *bc;          // 3 planes of barycentric weights per new point
    double *plane;       // copy of the field being interpolated
    int *m_elem;         // new element of each marker (-1: none)
    int *m_slot;         // markers grouped by element
    int *e_count, *e_offset, *e_fill; // per element (e_offset has E + 1)
    int *d_scalars;      // [0] scan total
};

// Magma sub-model (itype_melting = 1, FP64 contexts): melting after
// change_phase's recount (change_phase.f90:264-483) and fl_therm's magma
// part between temp0 = temp and the diffusion (fl_therm.f90:56-391).
struct GfMagma {
    static void melting(const GfLaunch &g);
    static void therm(const GfLaunch &g, int max_markers);
};

template <class R> struct GfRemesh {
    // bar2euler, rem_cord, element and node interpolation, incoming phases
    static void regrid(const GfLaunch &g, const GfRemeshArgs &a, const GfRemeshBufs &b);
    static void init_areas(const GfLaunch &g);
    // lpeuler2bar, then marker2elem's top-up and jmoho (phase recount by the caller)
    static void rebin_markers(const GfLaunch &g, const GfRemeshArgs &a, const GfRemeshBufs &b);
    static void top_up_markers(const GfLaunch &g, const GfRemeshArgs &a, const GfRemeshBufs &b);
    static void jmoho(const GfLaunch &g);
    // diff_topo (and resurface when `resurface`) after the coordinate update
    static void diff_topo(const GfLaunch &g, int resurface, int nloop, int max_markers);
    // fl_flexure (nbc 200 on the bottom): plate thickness Te, fluid density rho_m
    static void flexure(const GfLaunch &g, double Te, double rho_m);
};

