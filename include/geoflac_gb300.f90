! Fortran (ISO_C_BINDING) mirror of include/geoflac_gb300.h: the bind(C)
! derived types gf_params_t, gf_clock_t and gf_layout_t (field by field, in
! the C order; C's row-major 2-D arrays appear with their dimensions
! reversed) and interfaces of the entry points a GeoFLAC build calls.
! Fortran 2003; compile it before include/geoflac_gb300_shim.f90.

module geoflac_gb300
  use iso_c_binding
  implicit none

  integer, parameter :: gf_maxzone = 10, gf_maxbc = 20, gf_maxzone_age = 32, gf_maxzone_layer = 10, &
       gf_maxph = 20, gf_maxinh = 100, gf_max_markers_per_elem = 32

  integer(c_int), parameter :: GF_OK = 0, GF_ERR_CUDA = -1, GF_ERR_ARG = -2, GF_ERR_IO = -3, &
       GF_ERR_PARSE = -4, GF_ERR_UNSUPPORTED = -5, GF_ERR_TIMEOUT = -6, GF_ERR_NOMEM = -7, &
       GF_ERR_NONFINITE = -8, GF_ERR_LIMIT = -9
  integer(c_int), parameter :: GF_MODE_FP64 = 0, GF_MODE_MIXED = 1
  ! field masks of gf_upload / gf_download (unsigned in C)
  integer(c_int), parameter :: GF_F_CORD = 1, GF_F_VEL = 2, GF_F_TEMP = 4, GF_F_STRESS = 8, &
       GF_F_AREA = 16, GF_F_STRAIN = 32, GF_F_APS = 64, GF_F_VISN = 128, GF_F_MASS = 256, &
       GF_F_PHASE = 512, GF_F_RATE = 1024, GF_F_BC = 2048, GF_F_MARKERS = 4096, GF_F_ALL = -1

  type, bind(C) :: gf_params_t
     integer(c_int) :: nx, nz
     real(c_double) :: x0, z0, rxbo, rzbo
     integer(c_int) :: ircoord
     character(kind=c_char) :: coordfile(200)
     integer(c_int) :: nzonx, nzony
     integer(c_int) :: nelz_x(gf_maxzone), nelz_y(gf_maxzone)
     real(c_double) :: sizez_x(gf_maxzone), sizez_y(gf_maxzone)
     integer(c_int) :: nystressbc, nydrsides, nofbc
     integer(c_int) :: nofside(gf_maxbc), nbc1(gf_maxbc), nbc2(gf_maxbc), nbc(gf_maxbc)
     real(c_double) :: bca(gf_maxbc), bcb(gf_maxbc), bcc(gf_maxbc), bcd(gf_maxbc), bce(gf_maxbc), &
          bcf(gf_maxbc), bcg(gf_maxbc), bch(gf_maxbc), bci(gf_maxbc)
     integer(c_int) :: nyhydro, iphsub
     real(c_double) :: pisos, drosub, damp_vis, g
     integer(c_int) :: i_prestress, itherm, istress_therm, ishearh, itemp_bc, irtemp
     real(c_double) :: extra_pres, t_top, t_bot, hs, hr, bot_bc
     character(kind=c_char) :: tempfile(200)
     integer(c_int) :: nzone_age
     integer(c_int) :: ictherm(gf_maxzone_age), ixtb1(gf_maxzone_age), ixtb2(gf_maxzone_age)
     integer(c_int) :: nph_layer(gf_maxzone_age), iph_col_trans(gf_maxzone_age)
     integer(c_int) :: iph_col(gf_maxzone_layer, gf_maxzone_age)  ! iph_col(n, m) of params is iph_col(m, n) here
     real(c_double) :: age_1(gf_maxzone_age), tp1(gf_maxzone_age), tp2(gf_maxzone_age)
     real(c_double) :: hc(gf_maxzone_layer, gf_maxzone_age)       ! likewise hc
     integer(c_int) :: nphase
     integer(c_int) :: irheol(gf_maxph)
     real(c_double) :: visc(gf_maxph), den(gf_maxph), alfa(gf_maxph), beta(gf_maxph), pln(gf_maxph), &
          acoef(gf_maxph), eactiv(gf_maxph), vactiv(gf_maxph), rl(gf_maxph), rm(gf_maxph), &
          plstrain1(gf_maxph), plstrain2(gf_maxph), fric1(gf_maxph), fric2(gf_maxph), &
          cohesion1(gf_maxph), cohesion2(gf_maxph), dilat1(gf_maxph), dilat2(gf_maxph), &
          conduct(gf_maxph), cp(gf_maxph), ts(gf_maxph), tl(gf_maxph), tk(gf_maxph), &
          erodibility(gf_maxph)
     integer(c_int) :: irphase
     character(kind=c_char) :: phasefile(200)
     integer(c_int) :: inhom
     integer(c_int) :: ix1(gf_maxinh), ix2(gf_maxinh), iy1(gf_maxinh), iy2(gf_maxinh), &
          inphase(gf_maxinh), igeom(gf_maxinh)
     real(c_double) :: xinitaps(gf_maxinh)
     real(c_double) :: ten_off, tau_heal, v_min, v_max, efoldc
     integer(c_int) :: ivis_shape
     integer(c_int) :: itype_melting, nelem_serp, nelem_dike
     real(c_double) :: prod_magma, prod_magma2, rho_magma, angle_mzone, fmagma_max, ratio_mantle_mzone, &
          ratio_crust_mzone, latent_heat_magma, lambda_freeze, lambda_freeze_tdep, &
          weaken_ratio_plastic, weaken_ratio_viscous
     integer(c_int) :: ny_rem, mode_rem, ntest_rem
     real(c_double) :: angle_rem, dx_rem, topo_kappa, fac_kappa
     integer(c_int) :: idt_scale, i_rey, ifreq_rmasses, ifreq_imasses, ifreq_visc, ifreq_avgsr
     real(c_double) :: dt_scale, strain_inert, xReyn, frac, fracm, demf
     integer(c_int) :: movegrid, ndim, mix_strain, mix_stress
     real(c_double) :: time_max, dtout_screen, dtout_file, dtsave_file
     integer(c_int) :: io_flags(19)
     integer(c_int) :: lastout, lastsave
     real(c_double) :: dxmin, dzmin, vbc, Amin
     integer(c_int) :: ivis_present, incoming_left, incoming_right, nopbmax
     integer(c_int) :: markers_per_side, eclogite_rule, therm_sweeps
  end type gf_params_t

  type, bind(C) :: gf_clock_t
     integer(c_int) :: nloop, nsrate, nmarkers, need_remeshing
     real(c_double) :: time, dt, dtavg
     real(c_double) :: dt_elastic, dt_maxwell, dtmax_therm
     real(c_double) :: frac
     real(c_double) :: vel_max, dlmin
     integer(c_int) :: therm_sweeps, therm_unconverged
  end type gf_clock_t

  ! c_loc() of the reference's module arrays (arrays.f90, marker_data.f90)
  type, bind(C) :: gf_layout_t
     integer(c_int) :: nx, nz, nphase, max_markers
     type(c_ptr) :: cord, vel, temp, temp0, amass, rmass, bc
     type(c_ptr) :: ncod
     type(c_ptr) :: stress0
     type(c_ptr) :: area, dvol
     type(c_ptr) :: strain
     type(c_ptr) :: se2sr
     type(c_ptr) :: aps, visn, e2sr, source, shrheat, sshrheat
     type(c_ptr) :: fmagma, fmagma2, dike_released
     type(c_ptr) :: iphase
     type(c_ptr) :: phase_ratio
     type(c_ptr) :: jmoho
     type(c_ptr) :: dhacc_correction
     type(c_ptr) :: mark_a1, mark_a2, mark_age
     type(c_ptr) :: mark_dead, mark_phase
     type(c_ptr) :: mark_ntriag
     type(c_ptr) :: mark_id_elem
     type(c_ptr) :: nmark_elem
     type(c_ptr) :: dhacc, extr_acc, dtopo
     type(c_ptr) :: xoriginal, zoriginal, q_init, vel_flex_old
     type(c_ptr) :: fmelt, fmelt2, dike_backlog, dike_marker_vol, mor_marker_vol, extrusion
  end type gf_layout_t

  interface
     ! host-side set-up (read_params + setflac)
     integer(c_int) function gf_read_params(path, p) bind(C, name='gf_read_params')
       import :: c_int, c_char, gf_params_t
       character(kind=c_char), intent(in) :: path(*)
       type(gf_params_t), intent(inout) :: p
     end function gf_read_params
     integer(c_int) function gf_setflac_host(p, c, l) bind(C, name='gf_setflac_host')
       import :: c_int, gf_params_t, gf_clock_t, gf_layout_t
       type(gf_params_t), intent(inout) :: p
       type(gf_clock_t), intent(inout) :: c
       type(gf_layout_t), intent(in) :: l
     end function gf_setflac_host
     ! context
     integer(c_int) function gf_create(ctx, p, l, mode) bind(C, name='gf_create')
       import :: c_int, c_ptr, gf_params_t, gf_layout_t
       type(c_ptr), intent(out) :: ctx
       type(gf_params_t), intent(in) :: p
       type(gf_layout_t), intent(in) :: l
       integer(c_int), value :: mode
     end function gf_create
     subroutine gf_destroy(ctx) bind(C, name='gf_destroy')
       import :: c_ptr
       type(c_ptr), value :: ctx
     end subroutine gf_destroy
     integer(c_int) function gf_upload(ctx, mask) bind(C, name='gf_upload')
       import :: c_int, c_ptr
       type(c_ptr), value :: ctx
       integer(c_int), value :: mask
     end function gf_upload
     integer(c_int) function gf_download(ctx, mask) bind(C, name='gf_download')
       import :: c_int, c_ptr
       type(c_ptr), value :: ctx
       integer(c_int), value :: mask
     end function gf_download
     integer(c_int) function gf_set_clock(ctx, c) bind(C, name='gf_set_clock')
       import :: c_int, c_ptr, gf_clock_t
       type(c_ptr), value :: ctx
       type(gf_clock_t), intent(in) :: c
     end function gf_set_clock
     integer(c_int) function gf_get_clock(ctx, c) bind(C, name='gf_get_clock')
       import :: c_int, c_ptr, gf_clock_t
       type(c_ptr), value :: ctx
       type(gf_clock_t), intent(out) :: c
     end function gf_get_clock
     integer(c_int) function gf_set_params(ctx, p) bind(C, name='gf_set_params')
       import :: c_int, c_ptr, gf_params_t
       type(c_ptr), value :: ctx
       type(gf_params_t), intent(in) :: p
     end function gf_set_params
     integer(c_int) function gf_get_params(ctx, p) bind(C, name='gf_get_params')
       import :: c_int, c_ptr, gf_params_t
       type(c_ptr), value :: ctx
       type(gf_params_t), intent(out) :: p
     end function gf_get_params
     integer(c_int) function gf_finish_setflac(ctx) bind(C, name='gf_finish_setflac')
       import :: c_int, c_ptr
       type(c_ptr), value :: ctx
     end function gf_finish_setflac
     ! the per-step subroutines of flac.f90 and the remesh event of par.f90
     integer(c_int) function gf_fl_therm(ctx) bind(C, name='gf_fl_therm')
       import :: c_int, c_ptr
       type(c_ptr), value :: ctx
     end function gf_fl_therm
     integer(c_int) function gf_change_phase(ctx) bind(C, name='gf_change_phase')
       import :: c_int, c_ptr
       type(c_ptr), value :: ctx
     end function gf_change_phase
     integer(c_int) function gf_fl_rheol(ctx) bind(C, name='gf_fl_rheol')
       import :: c_int, c_ptr
       type(c_ptr), value :: ctx
     end function gf_fl_rheol
     integer(c_int) function gf_fl_node(ctx) bind(C, name='gf_fl_node')
       import :: c_int, c_ptr
       type(c_ptr), value :: ctx
     end function gf_fl_node
     integer(c_int) function gf_fl_move(ctx) bind(C, name='gf_fl_move')
       import :: c_int, c_ptr
       type(c_ptr), value :: ctx
     end function gf_fl_move
     integer(c_int) function gf_rmasses(ctx) bind(C, name='gf_rmasses')
       import :: c_int, c_ptr
       type(c_ptr), value :: ctx
     end function gf_rmasses
     integer(c_int) function gf_dt_mass(ctx) bind(C, name='gf_dt_mass')
       import :: c_int, c_ptr
       type(c_ptr), value :: ctx
     end function gf_dt_mass
     integer(c_int) function gf_init_visc(ctx) bind(C, name='gf_init_visc')
       import :: c_int, c_ptr
       type(c_ptr), value :: ctx
     end function gf_init_visc
     integer(c_int) function gf_marker2elem(ctx) bind(C, name='gf_marker2elem')
       import :: c_int, c_ptr
       type(c_ptr), value :: ctx
     end function gf_marker2elem
     integer(c_int) function gf_flac(ctx) bind(C, name='gf_flac')
       import :: c_int, c_ptr
       type(c_ptr), value :: ctx
     end function gf_flac
     integer(c_int) function gf_step(ctx, nsteps) bind(C, name='gf_step')
       import :: c_int, c_ptr
       type(c_ptr), value :: ctx
       integer(c_int), value :: nsteps
     end function gf_step
     integer(c_int) function gf_itest_mesh(ctx, min_angle) bind(C, name='gf_itest_mesh')
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: ctx
       real(c_double), intent(out) :: min_angle
     end function gf_itest_mesh
     integer(c_int) function gf_remesh(ctx) bind(C, name='gf_remesh')
       import :: c_int, c_ptr
       type(c_ptr), value :: ctx
     end function gf_remesh
     ! output frames and restart files
     integer(c_int) function gf_outflac(ctx, dir, fresh) bind(C, name='gf_outflac')
       import :: c_int, c_ptr, c_char
       type(c_ptr), value :: ctx
       character(kind=c_char), intent(in) :: dir(*)
       integer(c_int), value :: fresh
     end function gf_outflac
     integer(c_int) function gf_outmarker(ctx, dir, fresh) bind(C, name='gf_outmarker')
       import :: c_int, c_ptr, c_char
       type(c_ptr), value :: ctx
       character(kind=c_char), intent(in) :: dir(*)
       integer(c_int), value :: fresh
     end function gf_outmarker
     integer(c_int) function gf_saveflac(ctx, dir) bind(C, name='gf_saveflac')
       import :: c_int, c_ptr, c_char
       type(c_ptr), value :: ctx
       character(kind=c_char), intent(in) :: dir(*)
     end function gf_saveflac
     integer(c_int) function gf_rsflac(ctx, dir) bind(C, name='gf_rsflac')
       import :: c_int, c_ptr, c_char
       type(c_ptr), value :: ctx
       character(kind=c_char), intent(in) :: dir(*)
     end function gf_rsflac
     ! status
     integer(c_int) function gf_status(ctx) bind(C, name='gf_status')
       import :: c_int, c_ptr
       type(c_ptr), value :: ctx
     end function gf_status
     type(c_ptr) function gf_strerror(code) bind(C, name='gf_strerror')
       import :: c_int, c_ptr
       integer(c_int), value :: code
     end function gf_strerror
     integer(c_size_t) function gf_struct_size(which) bind(C, name='gf_struct_size')
       import :: c_int, c_size_t
       integer(c_int), value :: which
     end function gf_struct_size
     ! mesh-quality test on a device copy of cord, for hosts that cannot
     ! allocate device memory (acc_deviceptr(cord) of an OpenACC data region)
     integer(c_int) function gf_min_angle_noalloc(d_cord, nx, nz, stream, min_angle) &
          bind(C, name='gf_min_angle_noalloc')
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: d_cord, stream
       integer(c_int), value :: nx, nz
       real(c_double), intent(out) :: min_angle
     end function gf_min_angle_noalloc
  end interface

end module geoflac_gb300
