! Drop-in bodies for GeoFLAC's per-step subroutines on the GB300 library.
!
! A GeoFLAC build compiles this file (after include/geoflac_gb300.f90) in
! place of the bodies of the routines it replaces: fl_therm, change_phase,
! fl_rheol, fl_node, fl_move, rmasses, dt_mass, init_visc (src/*.f90 of the
! same names, called from src/flac.f90:18-83 and src/setflac.f90:71-77),
! and the remesh path of src/par.f90:94-108 (itest_mesh, bar2euler, remesh,
! lpeuler2bar, marker2elem).  Callers do not change.  Each body copies the
! clock scalars of module params to the library, calls the library's
! routine of the same name, copies the scalars back and stops with the
! library's status where the reference stops (22 Maxwell time step, 40/41
! negative area, 133/134 markers, 999 restart).
!
! Two edits to the reference go with it:
! * the allocatable arrays of modules arrays and marker_data get the
!   TARGET attribute (c_loc of them is passed to the library once);
! * the original bodies of marker2elem, bar2euler and lpeuler2bar are kept
!   renamed marker2elem_host, bar2euler_host and lpeuler2bar_host: the
!   start-up (init_marker) runs on the host before the library holds the
!   model, and the library's gf_remesh runs all three on the device
!   afterwards.
! The state lives on the device between sync points: call
! gf_shim_sync_host at the !$ACC wait of par.f90:113 (before outflac,
! outmarker, saveflac), and gf_shim_sync_device after the host changes
! arrays (rsflac).

module gf_shim
  use iso_c_binding
  use geoflac_gb300
  implicit none
  type(c_ptr), save :: gf_ctx = c_null_ptr
  type(gf_params_t), save :: gfp
  type(gf_layout_t), save :: gfl
  type(gf_clock_t), save :: gfk
  integer(c_int), save :: gf_mode = GF_MODE_FP64

contains

  ! The reference's stop codes for a library status.
  subroutine gf_stop_on(rc)
    integer(c_int), intent(in) :: rc
    select case (rc)
    case (0)
      return
    case (22)
      stop 22
    case (40)
      stop 40
    case (41)
      stop 41
    case (133)
      stop 133
    case (134)
      stop 134
    case (999)
      stop 999
    case default
      write(*, *) 'geoflac_gb300: library status ', rc
      stop 1
    end select
  end subroutine gf_stop_on

  subroutine gf_fill_string(dst, src)
    character(kind=c_char), intent(out) :: dst(:)
    character(len=*), intent(in) :: src
    integer :: k, n
    dst = c_null_char
    n = min(len_trim(src), size(dst) - 1)
    do k = 1, n
      dst(k) = src(k:k)
    end do
  end subroutine gf_fill_string

  ! Every value of module params that gf_params carries, in its order.
  subroutine gf_fill_params()
    use params
    integer :: n, m
    gfp%nx = nx
    gfp%nz = nz
    gfp%x0 = x0
    gfp%z0 = z0
    gfp%rxbo = rxbo
    gfp%rzbo = rzbo
    gfp%ircoord = ircoord
    call gf_fill_string(gfp%coordfile, coordfile)
    gfp%nzonx = nzonx
    gfp%nzony = nzony
    gfp%nelz_x = nelz_x
    gfp%nelz_y = nelz_y
    gfp%sizez_x = sizez_x
    gfp%sizez_y = sizez_y
    gfp%nystressbc = nystressbc
    gfp%nydrsides = nydrsides
    gfp%nofbc = nofbc
    gfp%nofside = nofside
    gfp%nbc1 = nbc1
    gfp%nbc2 = nbc2
    gfp%nbc = nbc
    gfp%bca = bca
    gfp%bcb = bcb
    gfp%bcc = bcc
    gfp%bcd = bcd
    gfp%bce = bce
    gfp%bcf = bcf
    gfp%bcg = bcg
    gfp%bch = bch
    gfp%bci = bci
    gfp%nyhydro = nyhydro
    gfp%iphsub = iphsub
    gfp%pisos = pisos
    gfp%drosub = drosub
    gfp%damp_vis = damp_vis
    gfp%g = g
    gfp%i_prestress = i_prestress
    gfp%itherm = itherm
    gfp%istress_therm = istress_therm
    gfp%ishearh = ishearh
    gfp%itemp_bc = itemp_bc
    gfp%irtemp = irtemp
    gfp%extra_pres = extra_pres
    gfp%t_top = t_top
    gfp%t_bot = t_bot
    gfp%hs = hs
    gfp%hr = hr
    gfp%bot_bc = bot_bc
    call gf_fill_string(gfp%tempfile, tempfile)
    gfp%nzone_age = nzone_age
    gfp%ictherm = ictherm
    gfp%ixtb1 = ixtb1
    gfp%ixtb2 = ixtb2
    gfp%nph_layer = nph_layer
    gfp%iph_col_trans = iph_col_trans
    do n = 1, maxzone_age
      do m = 1, maxzone_layer
        gfp%iph_col(m, n) = iph_col(n, m)
        gfp%hc(m, n) = hc(n, m)
      end do
    end do
    gfp%age_1 = age_1
    gfp%tp1 = tp1
    gfp%tp2 = tp2
    gfp%nphase = nphase
    gfp%irheol = irheol
    gfp%visc = visc
    gfp%den = den
    gfp%alfa = alfa
    gfp%beta = beta
    gfp%pln = pln
    gfp%acoef = acoef
    gfp%eactiv = eactiv
    gfp%vactiv = vactiv
    gfp%rl = rl
    gfp%rm = rm
    gfp%plstrain1 = plstrain1
    gfp%plstrain2 = plstrain2
    gfp%fric1 = fric1
    gfp%fric2 = fric2
    gfp%cohesion1 = cohesion1
    gfp%cohesion2 = cohesion2
    gfp%dilat1 = dilat1
    gfp%dilat2 = dilat2
    gfp%conduct = conduct
    gfp%cp = cp
    gfp%ts = ts
    gfp%tl = tl
    gfp%tk = tk
    gfp%erodibility = erodibility
    gfp%irphase = irphase
    call gf_fill_string(gfp%phasefile, phasefile)
    gfp%inhom = inhom
    gfp%ix1 = ix1
    gfp%ix2 = ix2
    gfp%iy1 = iy1
    gfp%iy2 = iy2
    gfp%inphase = inphase
    gfp%igeom = igeom
    gfp%xinitaps = xinitaps
    gfp%ten_off = ten_off
    gfp%tau_heal = tau_heal
    gfp%v_min = v_min
    gfp%v_max = v_max
    gfp%efoldc = efoldc
    gfp%ivis_shape = ivis_shape
    gfp%itype_melting = itype_melting
    gfp%nelem_serp = nelem_serp
    gfp%nelem_dike = nelem_dike
    gfp%prod_magma = prod_magma
    gfp%prod_magma2 = prod_magma2
    gfp%rho_magma = rho_magma
    gfp%angle_mzone = angle_mzone
    gfp%fmagma_max = fmagma_max
    gfp%ratio_mantle_mzone = ratio_mantle_mzone
    gfp%ratio_crust_mzone = ratio_crust_mzone
    gfp%latent_heat_magma = latent_heat_magma
    gfp%lambda_freeze = lambda_freeze
    gfp%lambda_freeze_tdep = lambda_freeze_tdep
    gfp%weaken_ratio_plastic = weaken_ratio_plastic
    gfp%weaken_ratio_viscous = weaken_ratio_viscous   ! read_params stores its log
    gfp%ny_rem = ny_rem
    gfp%mode_rem = mode_rem
    gfp%ntest_rem = ntest_rem
    gfp%angle_rem = angle_rem
    gfp%dx_rem = dx_rem
    gfp%topo_kappa = topo_kappa
    gfp%fac_kappa = fac_kappa
    gfp%idt_scale = idt_scale
    gfp%i_rey = i_rey
    gfp%ifreq_rmasses = ifreq_rmasses
    gfp%ifreq_imasses = ifreq_imasses
    gfp%ifreq_visc = ifreq_visc
    gfp%ifreq_avgsr = ifreq_avgsr
    gfp%dt_scale = dt_scale
    gfp%strain_inert = strain_inert
    gfp%xReyn = xReyn
    gfp%frac = frac
    gfp%fracm = fracm
    gfp%demf = demf
    gfp%movegrid = movegrid
    gfp%ndim = ndim
    gfp%mix_strain = mix_strain
    gfp%mix_stress = mix_stress
    gfp%time_max = time_max
    gfp%dtout_screen = dtout_screen
    gfp%dtout_file = dtout_file
    gfp%dtsave_file = dtsave_file
    gfp%io_flags = (/ io_vel, io_srII, io_eII, io_aps, io_sII, io_sxx, io_szz, io_sxz, io_pres, &
         io_temp, io_phase, io_visc, io_unused, io_density, io_src, io_diss, io_forc, io_hfl, io_topo /)
    gfp%lastout = lastout
    gfp%lastsave = lastsave
    gfp%dxmin = dxmin
    gfp%dzmin = dzmin
    gfp%vbc = vbc
    gfp%Amin = Amin
    gfp%ivis_present = ivis_present
    gfp%incoming_left = incoming_left
    gfp%incoming_right = incoming_right
    gfp%nopbmax = nopbmax
    gfp%markers_per_side = 3
    gfp%eclogite_rule = 0
    gfp%therm_sweeps = 0
  end subroutine gf_fill_params

  ! Addresses of the module arrays (they carry the TARGET attribute).
  subroutine gf_fill_layout()
    use params
    use arrays
    use marker_data
    gfl%nx = nx
    gfl%nz = nz
    gfl%nphase = nphase
    gfl%max_markers = max_markers
    gfl%cord = c_loc(cord)
    gfl%vel = c_loc(vel)
    gfl%temp = c_loc(temp)
    gfl%temp0 = c_loc(temp0)
    gfl%amass = c_loc(amass)
    gfl%rmass = c_loc(rmass)
    gfl%bc = c_loc(bc)
    gfl%ncod = c_loc(ncod)
    gfl%stress0 = c_loc(stress0)
    gfl%area = c_loc(area)
    gfl%dvol = c_loc(dvol)
    gfl%strain = c_loc(strain)
    gfl%se2sr = c_loc(se2sr)
    gfl%aps = c_loc(aps)
    gfl%visn = c_loc(visn)
    gfl%e2sr = c_loc(e2sr)
    gfl%source = c_loc(source)
    gfl%shrheat = c_loc(shrheat)
    gfl%sshrheat = c_loc(sshrheat)
    gfl%fmagma = c_loc(fmagma)
    gfl%fmagma2 = c_loc(fmagma2)
    gfl%dike_released = c_loc(dike_released)
    gfl%iphase = c_loc(iphase)
    gfl%phase_ratio = c_loc(phase_ratio)
    gfl%jmoho = c_loc(jmoho)
    gfl%dhacc_correction = c_loc(dhacc_correction)
    gfl%mark_a1 = c_loc(mark_a1)
    gfl%mark_a2 = c_loc(mark_a2)
    gfl%mark_age = c_loc(mark_age)
    gfl%mark_dead = c_loc(mark_dead)
    gfl%mark_phase = c_loc(mark_phase)
    gfl%mark_ntriag = c_loc(mark_ntriag)
    gfl%mark_id_elem = c_loc(mark_id_elem)
    gfl%nmark_elem = c_loc(nmark_elem)
    gfl%dhacc = c_loc(dhacc)
    gfl%extr_acc = c_loc(extr_acc)
    gfl%dtopo = c_loc(dtopo)
    gfl%xoriginal = c_loc(xoriginal)
    gfl%zoriginal = c_loc(zoriginal)
    gfl%q_init = c_loc(q_init)
    gfl%vel_flex_old = c_loc(vel_flex_old)
    gfl%fmelt = c_loc(fmelt)
    gfl%fmelt2 = c_loc(fmelt2)
    gfl%dike_backlog = c_loc(dike_backlog)
    gfl%dike_marker_vol = c_loc(dike_marker_vol)
    gfl%mor_marker_vol = c_loc(mor_marker_vol)
    gfl%extrusion = c_loc(extrusion)
  end subroutine gf_fill_layout

  ! The scalars the step reads and writes: module params -> library.
  subroutine gf_push_clock()
    use params
    gfk%nloop = nloop
    gfk%nsrate = nsrate
    gfk%nmarkers = nmarkers
    gfk%need_remeshing = 0
    gfk%time = time
    gfk%dt = dt
    gfk%dtavg = dtavg
    gfk%dt_elastic = dt_elastic
    gfk%dt_maxwell = dt_maxwell
    gfk%frac = frac
    call gf_stop_on(gf_set_clock(gf_ctx, gfk))
  end subroutine gf_push_clock

  ! ... and back (dt, dtavg, nsrate and frac change inside the step; the
  ! marker count after change_phase, fl_therm's magma part or a remesh).
  subroutine gf_pull_clock()
    use params
    call gf_stop_on(gf_get_clock(gf_ctx, gfk))
    nloop = gfk%nloop
    nsrate = gfk%nsrate
    nmarkers = gfk%nmarkers
    time = gfk%time
    dt = gfk%dt
    dtavg = gfk%dtavg
    dt_elastic = gfk%dt_elastic
    dt_maxwell = gfk%dt_maxwell
    frac = gfk%frac
  end subroutine gf_pull_clock

  ! First call: the library takes the model (set-up state of setflac).
  subroutine gf_shim_init()
    if (c_associated(gf_ctx)) return
    call gf_fill_params()
    call gf_fill_layout()
    call gf_stop_on(gf_create(gf_ctx, gfp, gfl, gf_mode))
    call gf_stop_on(gf_upload(gf_ctx, GF_F_ALL))
    call gf_push_clock()
  end subroutine gf_shim_init

  ! Device -> module arrays (before outflac, outmarker, saveflac).
  subroutine gf_shim_sync_host()
    if (.not. c_associated(gf_ctx)) return
    call gf_stop_on(gf_download(gf_ctx, GF_F_ALL))
    call gf_pull_clock()
  end subroutine gf_shim_sync_host

  ! Module arrays -> device (after the host changed them, e.g. rsflac).
  subroutine gf_shim_sync_device()
    if (.not. c_associated(gf_ctx)) return
    call gf_fill_params()
    call gf_stop_on(gf_set_params(gf_ctx, gfp))
    call gf_stop_on(gf_upload(gf_ctx, GF_F_ALL))
    call gf_push_clock()
  end subroutine gf_shim_sync_device

end module gf_shim

! ---- the reference's routines, same names and call sites ----------------

subroutine fl_therm
  use gf_shim
  integer(c_int) :: rc
  call gf_shim_init()
  call gf_push_clock()
  rc = gf_fl_therm(gf_ctx)
  call gf_pull_clock()
  call gf_stop_on(rc)
end subroutine fl_therm

subroutine change_phase
  use gf_shim
  integer(c_int) :: rc
  call gf_shim_init()
  call gf_push_clock()
  rc = gf_change_phase(gf_ctx)
  call gf_pull_clock()
  call gf_stop_on(rc)
end subroutine change_phase

subroutine fl_rheol
  use gf_shim
  integer(c_int) :: rc
  call gf_shim_init()
  call gf_push_clock()
  rc = gf_fl_rheol(gf_ctx)
  call gf_pull_clock()
  call gf_stop_on(rc)
end subroutine fl_rheol

subroutine fl_node
  use gf_shim
  integer(c_int) :: rc
  call gf_shim_init()
  call gf_push_clock()
  rc = gf_fl_node(gf_ctx)
  call gf_pull_clock()
  call gf_stop_on(rc)
end subroutine fl_node

subroutine fl_move
  use gf_shim
  integer(c_int) :: rc
  call gf_shim_init()
  call gf_push_clock()
  rc = gf_fl_move(gf_ctx)
  call gf_pull_clock()
  call gf_stop_on(rc)
end subroutine fl_move

subroutine rmasses
  use gf_shim
  integer(c_int) :: rc
  call gf_shim_init()
  call gf_push_clock()
  rc = gf_rmasses(gf_ctx)
  call gf_pull_clock()
  call gf_stop_on(rc)
end subroutine rmasses

subroutine dt_mass
  use gf_shim
  integer(c_int) :: rc
  call gf_shim_init()
  call gf_push_clock()
  rc = gf_dt_mass(gf_ctx)
  call gf_pull_clock()
  call gf_stop_on(rc)
end subroutine dt_mass

subroutine init_visc
  use gf_shim
  integer(c_int) :: rc
  call gf_shim_init()
  call gf_push_clock()
  rc = gf_init_visc(gf_ctx)
  call gf_pull_clock()
  call gf_stop_on(rc)
end subroutine init_visc

! par.f90:94-95: need_remeshing from the library's mesh-quality test
subroutine itest_mesh(need_remeshing)
  use gf_shim
  integer, intent(out) :: need_remeshing
  integer(c_int) :: rc
  real(c_double) :: angle
  call gf_shim_init()
  call gf_push_clock()
  rc = gf_itest_mesh(gf_ctx, angle)
  call gf_pull_clock()
  call gf_stop_on(rc)
  need_remeshing = gfk%need_remeshing
end subroutine itest_mesh

! par.f90:96-107: the library's remesh event covers bar2euler, remesh,
! lpeuler2bar, marker2elem and the dhacc_correction reset
subroutine remesh
  use gf_shim
  integer(c_int) :: rc
  call gf_shim_init()
  call gf_push_clock()
  rc = gf_remesh(gf_ctx)
  call gf_pull_clock()
  call gf_stop_on(rc)
end subroutine remesh

subroutine bar2euler
  use gf_shim
  if (.not. c_associated(gf_ctx)) call bar2euler_host()
end subroutine bar2euler

subroutine lpeuler2bar
  use gf_shim
  if (.not. c_associated(gf_ctx)) call lpeuler2bar_host()
end subroutine lpeuler2bar

! init_marker (set-up, host arrays) keeps the reference's marker2elem; once
! the library holds the model its remesh event has already run it
subroutine marker2elem
  use gf_shim
  if (.not. c_associated(gf_ctx)) call marker2elem_host()
end subroutine marker2elem
