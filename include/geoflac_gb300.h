/*
 * geoflac_gb300.h -- C-ABI of the GB300-native explicit FLAC time step.
 *
 * The reference (GeoFLAC) advances its model with argument-less Fortran
 * subroutines that read and write module globals (src/arrays.f90:55-130,
 * src/params.f90, src/marker_data.f90:12-18).  This header replaces that
 * implicit interface with plain pointers and sizes:
 *
 *   - gf_params  : every value src/read_params.f90:3-348 reads from a .inp
 *                  file, plus the values src/setflac.f90 derives at start-up.
 *   - gf_clock   : the scalars the step routines both read and write
 *                  (nloop, time, dt, dtavg, nsrate, dt_elastic, ...).
 *   - gf_layout  : host arrays in the reference's column-major layout
 *                  (j = depth index fastest), e.g. stress0(nz-1,nx-1,4,4).
 *
 * The host arrays stay owned by the caller (a Fortran program passes c_loc()
 * of its allocatables).  gf_create() makes device mirrors; gf_upload() /
 * gf_download() are the explicit sync points, placed where the reference has
 * `!$ACC update` / `!$ACC wait` (src/par.f90:113, src/fl_move.f90:34).
 * Between sync points the device copy is authoritative.
 *
 * Every entry point returns 0 on success, a positive value equal to the
 * reference's `stop` code when the reference would stop (22: Maxwell time
 * step, src/rh_maxwell.f90:24-30; 40: negative area, src/fl_move.f90:110-126;
 * 133: marker top-up failed, src/marker2elem.f90:52; 134: no marker in an
 * element, src/marker_data.f90:148), or a negative GF_ERR_* code.
 * No kernel traps: kernels record the first error in a device status word
 * that the host reads after each call.
 *
 * Threading: one host thread per context; calls on one context are not
 * re-entrant.  Each context owns one CUDA stream.
 */
#ifndef GEOFLAC_GB300_H
#define GEOFLAC_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Array bounds of the reference (src/params.f90:5-13, src/marker_data.f90:5). */
#define GF_MAXZONE 10
#define GF_MAXBC 20
#define GF_MAXZONE_AGE 32
#define GF_MAXZONE_LAYER 10
#define GF_MAXPH 20
#define GF_MAXINH 100
#define GF_MAX_MARKERS_PER_ELEM 32
#define GF_SEC_YEAR 3.1558e+7

/* Negative status codes (positive codes are the reference's stop codes). */
#define GF_OK 0
#define GF_ERR_CUDA (-1)
#define GF_ERR_ARG (-2)
#define GF_ERR_IO (-3)
#define GF_ERR_PARSE (-4)
#define GF_ERR_UNSUPPORTED (-5)
#define GF_ERR_TIMEOUT (-6)
#define GF_ERR_NOMEM (-7)
#define GF_ERR_NONFINITE (-8)
#define GF_ERR_LIMIT (-9) /* input larger than a fixed device scratch array */

/* Precision modes of a context. */
#define GF_MODE_FP64 0  /* every field and every operation in FP64          */
#define GF_MODE_MIXED 1 /* element fields, stresses, rheology and forces in FP32;
                           coordinates, temperature, masses and the dt
                           reductions in FP64                                */

/* Field masks for gf_upload / gf_download. */
#define GF_F_CORD (1u << 0)
#define GF_F_VEL (1u << 1)
#define GF_F_TEMP (1u << 2)
#define GF_F_STRESS (1u << 3)
#define GF_F_AREA (1u << 4)  /* area and dvol */
#define GF_F_STRAIN (1u << 5)
#define GF_F_APS (1u << 6)
#define GF_F_VISN (1u << 7)
#define GF_F_MASS (1u << 8)  /* amass and rmass */
#define GF_F_PHASE (1u << 9) /* iphase and phase_ratio */
#define GF_F_RATE (1u << 10) /* e2sr, se2sr, shrheat, sshrheat, temp0, source */
#define GF_F_BC (1u << 11)   /* bc and ncod */
#define GF_F_MARKERS (1u << 12) /* markers, and the surface and bottom accumulators:
                                   dhacc_correction, dhacc, extr_acc, dtopo,
                                   xoriginal, zoriginal, q_init, vel_flex_old */
#define GF_F_ALL 0xffffffffu

/* Every value of the .inp file, in the order src/read_params.f90:3-348
 * reads them, plus start-up values derived by src/setflac.f90:4-89. */
typedef struct gf_params {
    /* mesh (read_params.f90:14-75); nx, nz are node counts (input + 1) */
    int nx, nz;
    double x0, z0, rxbo, rzbo;
    int ircoord;
    char coordfile[200];
    int nzonx, nzony;
    int nelz_x[GF_MAXZONE], nelz_y[GF_MAXZONE];
    double sizez_x[GF_MAXZONE], sizez_y[GF_MAXZONE];
    /* mechanical conditions (read_params.f90:77-99) */
    int nystressbc, nydrsides, nofbc;
    int nofside[GF_MAXBC], nbc1[GF_MAXBC], nbc2[GF_MAXBC], nbc[GF_MAXBC];
    double bca[GF_MAXBC], bcb[GF_MAXBC], bcc[GF_MAXBC], bcd[GF_MAXBC], bce[GF_MAXBC],
        bcf[GF_MAXBC], bcg[GF_MAXBC], bch[GF_MAXBC], bci[GF_MAXBC];
    int nyhydro, iphsub;
    double pisos, drosub, damp_vis, g;
    /* thermal conditions (read_params.f90:103-187) */
    int i_prestress, itherm, istress_therm, ishearh, itemp_bc, irtemp;
    double extra_pres, t_top, t_bot, hs, hr, bot_bc;
    char tempfile[200];
    int nzone_age;
    int ictherm[GF_MAXZONE_AGE], ixtb1[GF_MAXZONE_AGE], ixtb2[GF_MAXZONE_AGE];
    int nph_layer[GF_MAXZONE_AGE], iph_col_trans[GF_MAXZONE_AGE];
    int iph_col[GF_MAXZONE_AGE][GF_MAXZONE_LAYER];
    double age_1[GF_MAXZONE_AGE], tp1[GF_MAXZONE_AGE], tp2[GF_MAXZONE_AGE];
    double hc[GF_MAXZONE_AGE][GF_MAXZONE_LAYER];
    /* rheology, one entry per phase, 0-based here (read_params.f90:189-200) */
    int nphase;
    int irheol[GF_MAXPH];
    double visc[GF_MAXPH], den[GF_MAXPH], alfa[GF_MAXPH], beta[GF_MAXPH], pln[GF_MAXPH],
        acoef[GF_MAXPH], eactiv[GF_MAXPH], vactiv[GF_MAXPH], rl[GF_MAXPH], rm[GF_MAXPH],
        plstrain1[GF_MAXPH], plstrain2[GF_MAXPH], fric1[GF_MAXPH], fric2[GF_MAXPH],
        cohesion1[GF_MAXPH], cohesion2[GF_MAXPH], dilat1[GF_MAXPH], dilat2[GF_MAXPH],
        conduct[GF_MAXPH], cp[GF_MAXPH], ts[GF_MAXPH], tl[GF_MAXPH], tk[GF_MAXPH],
        erodibility[GF_MAXPH];
    int irphase;
    char phasefile[200];
    /* inhomogeneities (read_params.f90:218-230) */
    int inhom;
    int ix1[GF_MAXINH], ix2[GF_MAXINH], iy1[GF_MAXINH], iy2[GF_MAXINH],
        inphase[GF_MAXINH], igeom[GF_MAXINH];
    double xinitaps[GF_MAXINH];
    double ten_off, tau_heal, v_min, v_max, efoldc;
    int ivis_shape;
    /* magma (read_params.f90:243-255); weaken_ratio_viscous is stored as its log */
    int itype_melting, nelem_serp, nelem_dike;
    double prod_magma, prod_magma2, rho_magma, angle_mzone, fmagma_max, ratio_mantle_mzone,
        ratio_crust_mzone, latent_heat_magma, lambda_freeze, lambda_freeze_tdep,
        weaken_ratio_plastic, weaken_ratio_viscous;
    /* remeshing (read_params.f90:257-272) */
    int ny_rem, mode_rem, ntest_rem;
    double angle_rem, dx_rem, topo_kappa, fac_kappa;
    /* process control (read_params.f90:275-313) */
    int idt_scale, i_rey, ifreq_rmasses, ifreq_imasses, ifreq_visc, ifreq_avgsr;
    double dt_scale, strain_inert, xReyn, frac, fracm, demf;
    int movegrid, ndim, mix_strain, mix_stress;
    /* output (read_params.f90:315-341); times converted to seconds */
    double time_max, dtout_screen, dtout_file, dtsave_file;
    int io_flags[19];
    int lastout, lastsave;
    /* derived at start-up (setflac.f90, init_cord.f90:80-81, init_bc.f90:385-409) */
    double dxmin, dzmin, vbc, Amin;
    int ivis_present, incoming_left, incoming_right, nopbmax;
    /* options with no .inp counterpart (defaults reproduce the reference) */
    int markers_per_side; /* 3 => 9 markers per element (init_marker.f90:52-91) */
    int eclogite_rule;    /* 0 => Hacker-2003 lines (change_phase.f90:159-170);
                             1 => simple rule: T >= 600 C and P >= 1.5 GPa   */
    int therm_sweeps;     /* cap on the sweeps of the thermal update
                             (gf_fl_therm); 0 => the library's cap (24) */
} gf_params;

/* Scalars that the step routines read and write.  The reference keeps them
 * in module params; a Fortran caller copies them in and out around calls. */
typedef struct gf_clock {
    int nloop;   /* step counter (par.f90:85) */
    int nsrate;  /* strain-rate averaging counter (fl_rheol.f90:395-421) */
    int nmarkers;
    int need_remeshing;
    double time, dt, dtavg;
    double dt_elastic, dt_maxwell, dtmax_therm;
    double frac; /* written by Eff_dens, see matprops.f90:37,48 */
    double vel_max, dlmin;
    int therm_sweeps;      /* sweeps the last fl_therm needed (read only) */
    int therm_unconverged; /* fl_therm calls that hit the sweep cap (read only) */
} gf_clock;

/* Host arrays, column-major with the depth index j fastest, 1-based in the
 * reference and 0-based here: cord[(k*nx + i)*nz + j] is cord(j+1,i+1,k+1).
 * A NULL pointer means "not provided"; gf_create() then keeps a
 * device-only copy initialised to zero. */
typedef struct gf_layout {
    int nx, nz, nphase, max_markers;
    /* node fields (nz, nx[, 2]) */
    double *cord, *vel, *temp, *temp0, *amass, *rmass, *bc;
    int *ncod;
    /* element fields (nz-1, nx-1[, k]) */
    double *stress0;     /* (nz-1, nx-1, 4, 4) */
    double *area, *dvol; /* (nz-1, nx-1, 4) */
    double *strain;      /* (nz-1, nx-1, 3) */
    double *se2sr;       /* (nz-1, nx-1, 3) */
    double *aps, *visn, *e2sr, *source, *shrheat, *sshrheat;
    double *fmagma, *fmagma2, *dike_released;
    int *iphase;
    double *phase_ratio; /* (nphase, nz-1, nx-1) */
    int *jmoho;          /* (nx-1) */
    double *dhacc_correction; /* (nx) */
    /* markers (marker_data.f90:12-18), max_markers entries */
    double *mark_a1, *mark_a2, *mark_age;
    int8_t *mark_dead, *mark_phase;
    int *mark_ntriag;
    int *mark_id_elem; /* (32, nz-1, nx-1) */
    int *nmark_elem;   /* (nz-1, nx-1) */
    /* surface processes (diff_topo, fl_move.f90:138-315), nx entries each:
     * accumulated topography change per surface element (dhacc, nx-1 used)
     * and arc extrusion (extr_acc, nx-1 used; stays zero without the magma
     * sub-model), and the last step's topography change per surface node */
    double *dhacc, *extr_acc, *dtopo;
    /* start-up node positions carried through remeshing (xoriginal,
     * zoriginal: (nz, nx) each, arrays.f90:12) and the flexural bottom's
     * state (fl_flexure.f90: q_init, vel_flex_old; nx each) */
    double *xoriginal, *zoriginal, *q_init, *vel_flex_old;
    /* magma sub-model (itype_melting = 1): the melt fractions of the last
     * change_phase (change_phase.f90:264-483), the dike-intrusion backlog and
     * marker-volume accumulators and the MOR marker-volume accumulator
     * (fl_therm.f90:330-391), (nz-1, nx-1) each; the last arc-extrusion
     * height per surface element (fl_move.f90:213-237; nx, nx-1 used) */
    double *fmelt, *fmelt2, *dike_backlog, *dike_marker_vol, *mor_marker_vol, *extrusion;
} gf_layout;

typedef struct gf_ctx gf_ctx;

/* ---- host-side set-up (the reference's read_params + setflac chain) ---- */

/* Parse a GeoFLAC .inp file.  Replaces read_params (src/read_params.f90:3-348);
 * same list-directed semantics, `;` comment lines (AdvanceToNextInputLine,
 * :351-373), nx/nz incremented to node counts (:22-23).  Returns GF_ERR_PARSE
 * (the reference stops with code 11) on a malformed file. */
int gf_read_params(const char *path, gf_params *p);

/* Sizes the caller must allocate for gf_layout (in elements, not bytes). */
int gf_layout_sizes(const gf_params *p, size_t *n_node, size_t *n_elem, size_t *max_markers);

/* Host part of setflac (src/setflac.f90:8-66): init_cord, init_phase,
 * init_marker (serial LCG chain, init_marker.f90:52-91) with marker2elem,
 * check_visc_rheol, init_areas, Amin, init_temp, init_stress, init_bc and the
 * field defaults.  rmasses, init_visc and dt_mass (setflac.f90:71-81) run on
 * the device: see gf_finish_setflac(). */
int gf_setflac_host(gf_params *p, gf_clock *c, gf_layout *L);

/* ---- device context ---- */

/* Create a device context mirroring L.  mode is GF_MODE_FP64 or
 * GF_MODE_MIXED.  Allocates all device storage; nothing is copied yet.
 * GF_ERR_UNSUPPORTED: applied stress boundary conditions (nystressbc = 1),
 * and, in GF_MODE_MIXED, the magma sub-model (itype_melting = 1) and the
 * flexural bottom (nbc 200 on side 2).  GF_ERR_LIMIT: in GF_MODE_MIXED,
 * meshes of 32 * nx * nz >= 2^31 (67 M nodes; its kernels index with 32-bit
 * integers). */
int gf_create(gf_ctx **ctx, const gf_params *p, const gf_layout *L, int mode);
void gf_destroy(gf_ctx *ctx);
int gf_upload(gf_ctx *ctx, unsigned field_mask);
int gf_download(gf_ctx *ctx, unsigned field_mask);
int gf_set_clock(gf_ctx *ctx, const gf_clock *c);
int gf_get_clock(gf_ctx *ctx, gf_clock *c);
int gf_set_params(gf_ctx *ctx, const gf_params *p);

/* rmasses + init_visc + dt_mass and the averaging reset of setflac
 * (src/setflac.f90:71-81) on the device. */
int gf_finish_setflac(gf_ctx *ctx);

/* ---- the per-step subroutines (drop-in for the reference's names) ---- */

/* fl_therm (src/fl_therm.f90:393-598): explicit diffusion + radiogenic and
 * shear heating, then the temperature boundary conditions.  The reference
 * updates temp in place (a Gauss-Seidel sweep, i outer, j inner); its result
 * is reproduced bit for bit by sweeping the same expression to its exact
 * floating-point fixed point. */
int gf_fl_therm(gf_ctx *ctx);
/* change_phase (src/change_phase.f90:35-262): marker phase rules, recount of
 * phase_ratio/iphase for changed elements, aps reduction. */
int gf_change_phase(gf_ctx *ctx);
/* fl_rheol (src/fl_rheol.f90:4-424): strain rates on the four overlaid
 * triangles, elastic/Maxwell/Mohr-Coulomb update, aps, strain, averaging. */
int gf_fl_rheol(gf_ctx *ctx);
/* fl_node (src/fl_node.f90:3-393): node-centric force gather (no atomics),
 * gravity, water load and Winkler foundation, damping, velocity update. */
int gf_fl_node(gf_ctx *ctx);
/* fl_move (src/fl_move.f90:4-132): coordinate update, areas, dvol and the
 * Jaumann rotation of stress and strain; stop code 40 on a negative area. */
int gf_fl_move(gf_ctx *ctx);
/* rmasses (src/rmasses.f90:4-63) as a node gather in colour order. */
int gf_rmasses(gf_ctx *ctx);
/* dt_mass (src/dt_mass.f90:16-232): dlmin, vel_max, amass, dt. */
int gf_dt_mass(gf_ctx *ctx);
/* init_visc (src/init_visc.f90) */
int gf_init_visc(gf_ctx *ctx);
/* marker2elem (src/marker2elem.f90:1-81): top-up of elements with <= 4
 * markers, count_phase_ratio, jmoho. */
int gf_marker2elem(gf_ctx *ctx);

/* One call of `flac` (src/flac.f90:5-91) with its frequency tests, followed
 * by the bookkeeping of src/par.f90:84-87 (nloop += 1, time += dt). */
int gf_flac(gf_ctx *ctx);
/* nsteps calls of gf_flac; the step sequence is captured once into a CUDA
 * graph per frequency phase and replayed. */
int gf_step(gf_ctx *ctx, int nsteps);

/* itest_mesh (src/rem_test.f90:9-139): minimum triangle angle; sets
 * clock.need_remeshing.  Returns the angle in *min_angle (degrees). */
int gf_itest_mesh(gf_ctx *ctx, double *min_angle);
/* The remesh event of src/par.f90:94-110: bar2euler, remesh, lpeuler2bar,
 * marker2elem. */
int gf_remesh(gf_ctx *ctx);

/* ---- output frames and restart files (drop-in for the reference's I/O) ----
 * Files go to directory `dir` (NULL or "" = the working directory, as in
 * the reference) in the reference's binary layouts: gfortran direct-access
 * records (fixed record length, no record markers, native byte order).
 * Every field of the reference's frames and restart files is written from
 * the model's state (the magma fields stay zero unless itype_melting = 1). */

/* outflac (src/outflac.f90:5-431): one float32 frame of the node, element
 * and surface fields selected by io_flags, appended as record nrec of each
 * `<field>.0` file and listed in `_contents.0`.  fresh = 1 starts a new
 * series (the reference's lastout == 1: nrec = 1, `_contents.0` rewritten);
 * fresh = 0 appends after the last record listed. */
int gf_outflac(gf_ctx *ctx, const char *dir, int fresh);
/* outmarker (src/outmarker.f90:1-100): marker1.NNNNNN.0 (x, z in km, age
 * in Myr, a1, a2 as float32 records) and marker2.NNNNNN.0 (dead, phase,
 * ntriag as int32 records), listed in `_markers.0`. */
int gf_outmarker(gf_ctx *ctx, const char *dir, int fresh);
/* saveflac (src/saveflac.f90:5-172): the FP64 restart files `*.rs`, Amin.rs,
 * pisos.rs (nyhydro == 2) and `_contents.save`.  Downloads every field into
 * the host arrays first (the layout must provide them). */
int gf_saveflac(gf_ctx *ctx, const char *dir);
/* rsflac (src/rsflac.f90:3-266): reads the restart files of record nrec
 * named in `_contents.rs` (or, if absent, `_contents.save`) into the host
 * arrays and the context, rebuilds the element marker lists (stop 999 on a
 * bad triangle number), then marker2elem, check_visc_rheol, init_areas,
 * init_bc, the field resets, rmasses, init_visc and dt_mass.  The context
 * must come from gf_create on the same .inp (sizes, phases, boundary
 * conditions); its parameters gain the restored Amin, pisos, dxmin, dzmin,
 * ivis_present and vbc (read them back with gf_get_params). */
int gf_rsflac(gf_ctx *ctx, const char *dir);
/* The context's current parameters (the counterpart of gf_set_params). */
int gf_get_params(gf_ctx *ctx, gf_params *p);

/* Per-subroutine calls wait for their kernels and return the device status
 * (sync = 1, the default: the reference's stop-on-error behaviour).  With
 * sync = 0 they only enqueue work on the context's stream; errors surface at
 * the next gf_status / gf_get_clock / gf_download.  No reference
 * counterpart (the reference's OpenACC regions are asynchronous on queue 1
 * and synchronised at !$ACC wait). */
int gf_set_sync(gf_ctx *ctx, int sync);
/* The context's CUDA stream (a cudaStream_t), for callers that interleave
 * their own work or record events on it. */
void *gf_stream(gf_ctx *ctx);
/* Last device status (0 when clean); also cleared by this call. */
int gf_status(gf_ctx *ctx);
/* Number of kernel launches issued by this context so far. */
long long gf_launch_count(gf_ctx *ctx);
/* Human-readable description of a status code. */
const char *gf_strerror(int code);
/* Smallest triangle angle (degrees) of the mesh held in the caller's device
 * array d_cord (the reference's cord(nz,nx,2) layout: depth fastest, then x
 * column, then component), the test of src/rem_test.f90:77-118, for callers
 * that must not allocate device memory: code whose device arrays belong to
 * an OpenACC data region or a caching allocator, where a cudaMalloc bypasses
 * that runtime and cudaFree stalls the whole device.  Allocates nothing: its
 * scratch is a fixed 65,792-byte array inside this library, so at most
 * 2,097,152 elements ((nx-1)*(nz-1)); larger meshes return GF_ERR_LIMIT.
 * The first call in each CUDA context looks up that array's address (a
 * caller-made driver context holds its own copy of the array).  All calls
 * share the array, so calls must not overlap in time on one device
 * (serialise them on one stream); each call clears the array's completion
 * ticket and result before its launch and returns GF_ERR_CUDA, not a stale
 * angle, if the launch did not finish the result.  Runs on `stream` (a
 * cudaStream_t; NULL = default stream) and synchronises it, copying the
 * result into host memory: it cannot be called while that stream is being
 * captured into a CUDA graph.
 * No reference counterpart (itest_mesh works on the host's module arrays). */
int gf_min_angle_noalloc(const double *d_cord, int nx, int nz, void *stream, double *min_angle);

/* ---- Ensembles (no reference counterpart) -----------------------------
 * A batch advances many independent models together: one persistent,
 * co-resident kernel per step walks every member's elements and nodes in
 * tiles of one member each, phase by phase (the reference runs one model
 * per process).  Members are GF_MODE_MIXED contexts that share the step
 * schedule (nloop, nsrate, ifreq_*, itherm); they stay owned by the caller,
 * must outlive the batch, and must not be stepped by other calls while a
 * batch step runs.  Their states stay readable with gf_download. */
typedef struct gf_batch gf_batch;
typedef struct gf_batch_config {
    int threads;          /* threads per CTA: 128, 256 or 512 */
    int items_per_thread; /* a tile is threads * items_per_thread items of one member */
    int ctas_per_sm;      /* resident CTAs per SM (capped by occupancy) */
    int graph_steps;      /* steps per captured CUDA graph; 0 = direct launches */
} gf_batch_config;
int gf_batch_create(gf_batch **out, gf_ctx **members, int n);
void gf_batch_destroy(gf_batch *b);
int gf_batch_set_config(gf_batch *b, const gf_batch_config *cfg);
int gf_batch_get_config(gf_batch *b, gf_batch_config *cfg);
/* Times every configuration over trial_steps steps (after one untimed step)
 * and keeps the fastest; the trial steps advance the members. */
int gf_batch_tune(gf_batch *b, int trial_steps, gf_batch_config *best, double *best_ms_per_step);
/* nsteps steps of every member (flac.f90:5-91 and par.f90:84-87 each). */
int gf_batch_step(gf_batch *b, int nsteps);
void *gf_batch_stream(gf_batch *b);
/* Every member's fields resampled to an H x W grid, FP32 [n][H][W][9]:
 * vx, vz, sxx, szz, sxz (total stress), plastic strain, temperature, the
 * fraction of phase `phase_id`, and the vertical displacement from the
 * regular start-up mesh (device pointer; bilinear in each member's index
 * space; asynchronous on the batch's stream). */
int gf_batch_sample(gf_batch *b, float *grid, int H, int W, int phase_id);
/* The inverse for a predicted grid of the same layout: velocities,
 * temperatures and vertical node positions, stresses (the out-of-plane
 * stress keeps its deviation) and plastic strain of every member, and the
 * element areas of the moved mesh; stop 41 if an element inverts. */
int gf_batch_inject(gf_batch *b, const float *grid, int H, int W);
/* Force imbalance of every member's current state (fl_node.f90's forces
 * without damping): sum over free nodes of |F| divided by the sum of
 * |gravity| and the magnitudes of the stress-divergence terms. */
int gf_batch_force_residual(gf_batch *b, double *residual);
/* Device copy of the fields gf_batch_inject writes, for every member (the
 * copy is allocated at the first call and kept), and the restore of the
 * listed members from it. */
int gf_batch_backup(gf_batch *b);
int gf_batch_restore(gf_batch *b, const int *members, int count);
long long gf_batch_elements(gf_batch *b);
int gf_batch_grid(gf_batch *b);
/* Check of the bounded grid barrier that separates the phases of the
 * persistent kernels (the ensemble step, the FP64 thermal sweeps): a
 * two-CTA co-resident launch in which CTA `absent_cta` (0 or 1) never
 * arrives, so the other gives up after `limit` polls (about 64 ns each) and
 * the call returns GF_ERR_TIMEOUT with the device still usable; absent_cta
 * = -1 lets both arrive (GF_OK).  passed[k] = 1 if CTA k left the barrier
 * normally, 0 if it gave up, -1 if it never reached it.  No reference
 * counterpart. */
int gf_grid_barrier_selftest(int absent_cta, long long limit, int *passed);

/* sizeof(gf_params), sizeof(gf_clock), sizeof(gf_layout) for which = 0, 1, 2:
 * lets a binding (ctypes, cgo, ISO_C_BINDING) check its struct mirrors.
 * No reference counterpart (the reference shares modules, not structs). */
size_t gf_struct_size(int which);

#ifdef __cplusplus
}
#endif

#endif /* GEOFLAC_GB300_H */
