! shearbox_c.f90 -- Fortran 2003 ISO_C_BINDING interface of the GB300
! shearing-box time stepper (include/shearbox.h), for the reference's drivers:
! disk3d (main.f90:273-281), calc_dns_disk3d (gmres_shear.f90:2951-3120) and
! shoot_shear.f90:527 call sb_cross / sb_crosst in place of cross / crosst.
! Arrays keep the reference's own layouts (vor, phi, tb: the buffsize arrays,
! complex(0:my1,0:mx1,0:mz1); u00, w00, tb00: real(0:my1)), so the calls copy
! nothing on the Fortran side.  Every function returns 0 on success; the text
! of the last error comes from sb_last_error (a C string).
! This file is an interface only; no Fortran compiler is used by the build.
module shearbox_c
  use iso_c_binding
  implicit none

  integer(c_int), parameter :: SB_FP64 = 0, SB_MIXED = 1
  integer(c_int), parameter :: SB_TRACE_RECORD = 24, SB_TRACE_RECORD_T = 29

  type, bind(C) :: sb_params
     integer(c_int)  :: mgalx, my, mgalz
     real(c_double)  :: Re, alp, Ly, gam
     real(c_double)  :: s, chi, CFL
     real(c_double)  :: vbulk
     real(c_double)  :: fixed_dt
     integer(c_int)  :: readflag
     real(c_double)  :: uprim
     integer(c_int)  :: nhist
     real(c_double)  :: etime, dumptime, dtimag
     integer(c_int)  :: keep_laminar
     integer(c_int)  :: les, les_visc
     real(c_double)  :: cs
     integer(c_int)  :: ydeal
     integer(c_int)  :: temperature
     real(c_double)  :: fkappa, bym, gbeta
     integer(c_int)  :: damping
     real(c_double)  :: damp_up, damp_aa
     integer(c_int)  :: force
     real(c_double)  :: force_roll, xforce
     integer(c_int)  :: implicit_visc
  end type sb_params

  type, bind(C) :: sb_status
     integer(c_int)  :: istop, steps_done, ntrace, flags
     real(c_double)  :: time, deltat, xoffb, xofft, cfl, cflv
  end type sb_status

  interface
     integer(c_int) function sb_create(p, batch, precision, h) bind(C, name="sb_create")
       import :: c_int, c_ptr, sb_params
       type(sb_params), intent(in) :: p
       integer(c_int), value :: batch, precision
       type(c_ptr), intent(out) :: h
     end function sb_create

     integer(c_int) function sb_destroy(h) bind(C, name="sb_destroy")
       import :: c_int, c_ptr
       type(c_ptr), value :: h
     end function sb_destroy

     integer(c_int) function sb_set_member_re(h, member, Re) bind(C, name="sb_set_member_re")
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: h
       integer(c_int), value :: member
       real(c_double), value :: Re
     end function sb_set_member_re

     integer(c_int) function sb_set_member_etime(h, member, etime) &
          bind(C, name="sb_set_member_etime")
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: h
       integer(c_int), value :: member
       real(c_double), value :: etime
     end function sb_set_member_etime

     integer(c_int) function sb_set_state(h, member, vor, phi, u00, w00, time, xoffb, xofft) &
          bind(C, name="sb_set_state")
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: h
       integer(c_int), value :: member
       real(c_double), intent(in) :: vor(*), phi(*), u00(*), w00(*)
       real(c_double), value :: time, xoffb, xofft
     end function sb_set_state

     integer(c_int) function sb_get_state(h, member, vor, phi, u00, w00, time, xoffb, xofft) &
          bind(C, name="sb_get_state")
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: h
       integer(c_int), value :: member
       real(c_double), intent(out) :: vor(*), phi(*), u00(*), w00(*)
       real(c_double), intent(out) :: time, xoffb, xofft
     end function sb_get_state

     integer(c_int) function sb_set_temperature(h, member, tb, tb00) &
          bind(C, name="sb_set_temperature")
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: h
       integer(c_int), value :: member
       real(c_double), intent(in) :: tb(*), tb00(*)
     end function sb_set_temperature

     integer(c_int) function sb_get_temperature(h, member, tb, tb00) &
          bind(C, name="sb_get_temperature")
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: h
       integer(c_int), value :: member
       real(c_double), intent(out) :: tb(*), tb00(*)
     end function sb_get_temperature

     integer(c_int) function sb_step(h, nsteps) bind(C, name="sb_step")
       import :: c_int, c_ptr
       type(c_ptr), value :: h
       integer(c_int), value :: nsteps
     end function sb_step

     integer(c_int) function sb_get_status(h, member, st) bind(C, name="sb_get_status")
       import :: c_int, c_ptr, sb_status
       type(c_ptr), value :: h
       integer(c_int), value :: member
       type(sb_status), intent(out) :: st
     end function sb_get_status

     integer(c_int) function sb_get_trace(h, member, out, maxrec, nrec) &
          bind(C, name="sb_get_trace")
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: h
       integer(c_int), value :: member, maxrec
       real(c_double), intent(out) :: out(*)
       integer(c_int), intent(out) :: nrec
     end function sb_get_trace

     integer(c_int) function sb_cross(h, vor, phi, u00, w00, time, xoffb, xofft, nstep, st) &
          bind(C, name="sb_cross")
       import :: c_int, c_ptr, c_double, sb_status
       type(c_ptr), value :: h
       real(c_double), intent(inout) :: vor(*), phi(*), u00(*), w00(*)
       real(c_double), intent(inout) :: time, xoffb, xofft
       integer(c_int), value :: nstep
       type(sb_status), intent(out) :: st
     end function sb_cross

     integer(c_int) function sb_crosst(h, vor, phi, u00, w00, tb, tb00, time, xoffb, xofft, &
          nstep, st) bind(C, name="sb_crosst")
       import :: c_int, c_ptr, c_double, sb_status
       type(c_ptr), value :: h
       real(c_double), intent(inout) :: vor(*), phi(*), u00(*), w00(*), tb(*), tb00(*)
       real(c_double), intent(inout) :: time, xoffb, xofft
       integer(c_int), value :: nstep
       type(sb_status), intent(out) :: st
     end function sb_crosst

     ! stats/stats2 (23,0:my1), spectra (8,0:mx1,0:mz1), tstats (5,0:my1),
     ! splt (4,0:mx1,0:mz1): the arrays of module statistics (mod.f90:94-115)
     integer(c_int) function sb_get_statistics(h, member, stats, stats2, spec, spec2, tstats, &
          tspec, nacum, total_dt) bind(C, name="sb_get_statistics")
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: h
       integer(c_int), value :: member
       real(c_double), intent(out) :: stats(*), stats2(*), spec(*), spec2(*)
       type(c_ptr), value :: tstats, tspec   ! c_null_ptr without the temperature
       integer(c_int), intent(out) :: nacum
       real(c_double), intent(out) :: total_dt
     end function sb_get_statistics

     integer(c_int) function sb_stats(h, member, uner, uner2) bind(C, name="sb_stats")
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: h
       integer(c_int), value :: member
       real(c_double), intent(out) :: uner(10), uner2(4)
     end function sb_stats

     ! block of period-map products for matvec_dns_disk3d: vectors are
     ! [vor | phi | u00 | w00]
     integer(c_int) function sb_jv_batch(h, x0, time0, xoffb, xofft, T, dirs, ndir, &
          eps_jacobi, central, out) bind(C, name="sb_jv_batch")
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: h
       real(c_double), intent(in) :: x0(*), dirs(*)
       real(c_double), value :: time0, xoffb, xofft, T, eps_jacobi
       integer(c_int), value :: ndir, central
       real(c_double), intent(out) :: out(*)
     end function sb_jv_batch

     integer(c_int) function sb_physical_fields(h, member, mask, out) &
          bind(C, name="sb_physical_fields")
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: h
       integer(c_int), value :: member, mask
       real(c_double), intent(out) :: out(*)
     end function sb_physical_fields

     integer(c_int) function sb_write_restart(path, p, vor, phi, u00, w00, time, xoffb, &
          xofft, deltat) bind(C, name="sb_write_restart")
       import :: c_int, c_char, c_double, sb_params
       character(kind=c_char), intent(in) :: path(*)   ! NUL-terminated
       type(sb_params), intent(in) :: p
       real(c_double), intent(in) :: vor(*), phi(*), u00(*), w00(*)
       real(c_double), value :: time, xoffb, xofft, deltat
     end function sb_write_restart

     ! device-resident unknown vectors of the Newton / Arnoldi drivers: x is a
     ! device address (for example a column of a Krylov space, sb_kspace_col);
     ! sca = (sca_u, sca_g, sca_p) of throwing (gmres_shear.f90:411-413)
     integer(c_long) function sb_packed_length(h) bind(C, name="sb_packed_length")
       import :: c_long, c_ptr
       type(c_ptr), value :: h
     end function sb_packed_length

     integer(c_int) function sb_set_state_packed(h, member, x, sca, time, xoffb, xofft) &
          bind(C, name="sb_set_state_packed")
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: h, x
       integer(c_int), value :: member
       real(c_double), intent(in) :: sca(3)
       real(c_double), value :: time, xoffb, xofft
     end function sb_set_state_packed

     integer(c_int) function sb_get_state_packed(h, member, x, sca, shiftx, shiftz) &
          bind(C, name="sb_get_state_packed")
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: h, x
       integer(c_int), value :: member
       real(c_double), intent(in) :: sca(3)
       real(c_double), value :: shiftx, shiftz
     end function sb_get_state_packed

     integer(c_int) function sb_packed_shift_tangent(h, x, out, dir) &
          bind(C, name="sb_packed_shift_tangent")
       import :: c_int, c_ptr
       type(c_ptr), value :: h, x, out
       integer(c_int), value :: dir
     end function sb_packed_shift_tangent

     ! a Krylov space of FP64 device columns: the vv(nl, k_gmres+1) of
     ! gmres_k_shear with its dotp / vecadd / norm on the GPU
     integer(c_int) function sb_kspace_create(n, cols, stream, ks) bind(C, name="sb_kspace_create")
       import :: c_int, c_long, c_ptr
       integer(c_long), value :: n
       integer(c_int), value :: cols
       type(c_ptr), value :: stream
       type(c_ptr), intent(out) :: ks
     end function sb_kspace_create

     integer(c_int) function sb_kspace_destroy(ks) bind(C, name="sb_kspace_destroy")
       import :: c_int, c_ptr
       type(c_ptr), value :: ks
     end function sb_kspace_destroy

     type(c_ptr) function sb_kspace_col(ks, col) bind(C, name="sb_kspace_col")
       import :: c_int, c_ptr
       type(c_ptr), value :: ks
       integer(c_int), value :: col
     end function sb_kspace_col

     integer(c_int) function sb_kspace_gram(ks, r0, r1, a0, m, b0, p, C) &
          bind(C, name="sb_kspace_gram")
       import :: c_int, c_long, c_ptr, c_double
       type(c_ptr), value :: ks
       integer(c_long), value :: r0, r1
       integer(c_int), value :: a0, m, b0, p
       real(c_double), intent(out) :: C(*)   ! m x p, row-major (C(p,m) in Fortran order)
     end function sb_kspace_gram

     integer(c_int) function sb_kspace_update(ks, r0, r1, a0, m, b0, p, C, alpha) &
          bind(C, name="sb_kspace_update")
       import :: c_int, c_long, c_ptr, c_double
       type(c_ptr), value :: ks
       integer(c_long), value :: r0, r1
       integer(c_int), value :: a0, m, b0, p
       real(c_double), intent(in) :: C(*)
       real(c_double), value :: alpha
     end function sb_kspace_update

     ! cols b0..b0+p-1 <- (cols b0..) M in place, p <= 64, M p x p row-major
     integer(c_int) function sb_kspace_transform(ks, r0, r1, b0, p, M) &
          bind(C, name="sb_kspace_transform")
       import :: c_int, c_long, c_ptr, c_double
       type(c_ptr), value :: ks
       integer(c_long), value :: r0, r1
       integer(c_int), value :: b0, p
       real(c_double), intent(in) :: M(*)
     end function sb_kspace_transform

     ! the space's CUDA stream and a blocking wait on it
     type(c_ptr) function sb_kspace_stream(ks) bind(C, name="sb_kspace_stream")
       import :: c_ptr
       type(c_ptr), value :: ks
     end function sb_kspace_stream

     integer(c_int) function sb_kspace_sync(ks) bind(C, name="sb_kspace_sync")
       import :: c_int, c_ptr
       type(c_ptr), value :: ks
     end function sb_kspace_sync

     integer(c_int) function sb_kspace_combine(ks, r0, r1, dst, nsrc, src, coef) &
          bind(C, name="sb_kspace_combine")
       import :: c_int, c_long, c_ptr, c_double
       type(c_ptr), value :: ks
       integer(c_long), value :: r0, r1
       integer(c_int), value :: dst, nsrc
       integer(c_int), intent(in) :: src(*)
       real(c_double), intent(in) :: coef(*)
     end function sb_kspace_combine

     integer(c_int) function sb_kspace_perturb(ks, r0, r1, dst, x0, d, e) &
          bind(C, name="sb_kspace_perturb")
       import :: c_int, c_long, c_ptr, c_double
       type(c_ptr), value :: ks
       integer(c_long), value :: r0, r1
       integer(c_int), value :: dst, x0, d
       real(c_double), value :: e
     end function sb_kspace_perturb

     integer(c_int) function sb_kspace_fd(ks, r0, r1, dst, order, g, eps) &
          bind(C, name="sb_kspace_fd")
       import :: c_int, c_long, c_ptr, c_double
       type(c_ptr), value :: ks
       integer(c_long), value :: r0, r1
       integer(c_int), value :: dst, order
       integer(c_int), intent(in) :: g(*)
       real(c_double), value :: eps
     end function sb_kspace_fd

     integer(c_int) function sb_kspace_set(ks, col, off, len, host) bind(C, name="sb_kspace_set")
       import :: c_int, c_long, c_ptr, c_double
       type(c_ptr), value :: ks
       integer(c_int), value :: col
       integer(c_long), value :: off, len
       real(c_double), intent(in) :: host(*)
     end function sb_kspace_set

     integer(c_int) function sb_kspace_get(ks, col, off, len, host) bind(C, name="sb_kspace_get")
       import :: c_int, c_long, c_ptr, c_double
       type(c_ptr), value :: ks
       integer(c_int), value :: col
       integer(c_long), value :: off, len
       real(c_double), intent(out) :: host(*)
     end function sb_kspace_get

     ! tiles of the step (plane stages, warps per y-line solve, y-line form)
     integer(c_int) function sb_autotune(h, choice) bind(C, name="sb_autotune")
       import :: c_int, c_ptr
       type(c_ptr), value :: h
       integer(c_int), intent(out) :: choice(3)
     end function sb_autotune

     integer(c_int) function sb_get_tuning(h, out) bind(C, name="sb_get_tuning")
       import :: c_int, c_ptr
       type(c_ptr), value :: h
       integer(c_int), intent(out) :: out(4)
     end function sb_get_tuning

     integer(c_int) function sb_set_line_segments(h, nseg) bind(C, name="sb_set_line_segments")
       import :: c_int, c_ptr
       type(c_ptr), value :: h
       integer(c_int), value :: nseg
     end function sb_set_line_segments

     ! y-line kernels of a substep: 1 fused, 0 split
     integer(c_int) function sb_set_line_form(h, form) bind(C, name="sb_set_line_form")
       import :: c_int, c_ptr
       type(c_ptr), value :: h
       integer(c_int), value :: form
     end function sb_set_line_form

     integer(c_int) function sb_get_line_form(h, form) bind(C, name="sb_get_line_form")
       import :: c_int, c_ptr
       type(c_ptr), value :: h
       integer(c_int), intent(out) :: form
     end function sb_get_line_form

     ! side work run as concurrent graph branches: bit 0 spectra, bit 1 scalars
     integer(c_int) function sb_set_side_branch(h, mask) bind(C, name="sb_set_side_branch")
       import :: c_int, c_ptr
       type(c_ptr), value :: h
       integer(c_int), value :: mask
     end function sb_set_side_branch

     integer(c_int) function sb_get_side_branch(h, mask) bind(C, name="sb_get_side_branch")
       import :: c_int, c_ptr
       type(c_ptr), value :: h
       integer(c_int), intent(out) :: mask
     end function sb_get_side_branch

     ! getfil on the run's grid; info: pass a buffer of at least 584 bytes
     ! (sb_restart_info), flags = 1 keeps the vorticity of a changed Re
     integer(c_int) function sb_read_restart_ex(path, p, flags, vor, phi, u00, w00, info) &
          bind(C, name="sb_read_restart_ex")
       import :: c_int, c_char, c_double, c_ptr, sb_params
       character(kind=c_char), intent(in) :: path(*)   ! NUL-terminated
       type(sb_params), intent(in) :: p
       integer(c_int), value :: flags
       real(c_double), intent(out) :: vor(*), phi(*), u00(*), w00(*)
       type(c_ptr), value :: info
     end function sb_read_restart_ex

     ! getfil of a file on the run's grid only (sb_read_restart_ex with flags 0)
     integer(c_int) function sb_read_restart(path, p, vor, phi, u00, w00, info) &
          bind(C, name="sb_read_restart")
       import :: c_int, c_char, c_double, c_ptr, sb_params
       character(kind=c_char), intent(in) :: path(*)   ! NUL-terminated
       type(sb_params), intent(in) :: p
       real(c_double), intent(out) :: vor(*), phi(*), u00(*), w00(*)
       type(c_ptr), value :: info
     end function sb_read_restart

     ! the handle's CUDA stream (cudaStream_t) and a blocking wait on it
     type(c_ptr) function sb_get_stream(h) bind(C, name="sb_get_stream")
       import :: c_ptr
       type(c_ptr), value :: h
     end function sb_get_stream

     integer(c_int) function sb_sync(h) bind(C, name="sb_sync")
       import :: c_int, c_ptr
       type(c_ptr), value :: h
     end function sb_sync

     ! y-line operators on DEVICE lines u, out (c_ptr of device memory, e.g.
     ! from CUDA Fortran or an OpenACC host_data region), element (line, j) at
     ! the complex u(line + j*ldu); shp, shm, k2 are host arrays of nlines
     ! entries; stream is a cudaStream_t (c_null_ptr: the legacy stream)
     ! derivyc (diffy_shear_hepta.f90:333-450), iord 1 or 2
     integer(c_int) function sb_op_derivyc(my, Ly, iord, nlines, u, ldu, out, ldo, shp, shm, &
          stream) bind(C, name="sb_op_derivyc")
       import :: c_int, c_long, c_double, c_double_complex, c_ptr
       integer(c_int), value :: my, iord, nlines
       real(c_double), value :: Ly
       type(c_ptr), value :: u, out, stream
       integer(c_long), value :: ldu, ldo
       complex(c_double_complex), intent(in) :: shp(*), shm(*)
     end function sb_op_derivyc

     ! the same without device allocation (fixed library scratch, error 6 when
     ! the request does not fit)
     integer(c_int) function sb_op_derivyc_noalloc(my, Ly, iord, nlines, u, ldu, out, ldo, &
          shp, shm, stream) bind(C, name="sb_op_derivyc_noalloc")
       import :: c_int, c_long, c_double, c_double_complex, c_ptr
       integer(c_int), value :: my, iord, nlines
       real(c_double), value :: Ly
       type(c_ptr), value :: u, out, stream
       integer(c_long), value :: ldu, ldo
       complex(c_double_complex), intent(in) :: shp(*), shm(*)
     end function sb_op_derivyc_noalloc

     ! lapcdy (diffy_shear_hepta.f90:466-525): (d2/dy2 - k2) out = u
     integer(c_int) function sb_op_lapcdy(my, Ly, nlines, u, ldu, out, ldo, k2, shp, shm, &
          stream) bind(C, name="sb_op_lapcdy")
       import :: c_int, c_long, c_double, c_double_complex, c_ptr
       integer(c_int), value :: my, nlines
       real(c_double), value :: Ly
       type(c_ptr), value :: u, out, stream
       integer(c_long), value :: ldu, ldo
       real(c_double), intent(in) :: k2(*)
       complex(c_double_complex), intent(in) :: shp(*), shm(*)
     end function sb_op_lapcdy

     ! filterc (filter_shear_hepta.f90:104-148)
     integer(c_int) function sb_op_filterc(my, nlines, u, ldu, out, ldo, shp, stream) &
          bind(C, name="sb_op_filterc")
       import :: c_int, c_long, c_double_complex, c_ptr
       integer(c_int), value :: my, nlines
       type(c_ptr), value :: u, out, stream
       integer(c_long), value :: ldu, ldo
       complex(c_double_complex), intent(in) :: shp(*)
     end function sb_op_filterc

     ! cfty / rfty (cftdoublew.F:151-201, rftdoublew.F:133-158) in place on
     ! device lines c; iopt < 0 forward (scaled by 1/my), > 0 backward
     integer(c_int) function sb_op_cfty(my, nlines, c, ldc, iopt, stream) &
          bind(C, name="sb_op_cfty")
       import :: c_int, c_long, c_ptr
       integer(c_int), value :: my, nlines, iopt
       type(c_ptr), value :: c, stream
       integer(c_long), value :: ldc
     end function sb_op_cfty

     integer(c_int) function sb_op_rfty(my, nlines, c, ldc, iopt, stream) &
          bind(C, name="sb_op_rfty")
       import :: c_int, c_long, c_ptr
       integer(c_int), value :: my, nlines, iopt
       type(c_ptr), value :: c, stream
       integer(c_long), value :: ldc
     end function sb_op_rfty

     integer(c_int) function sb_sizes(p, out) bind(C, name="sb_sizes")
       import :: c_int, sb_params
       type(sb_params), intent(in) :: p
       integer(c_int), intent(out) :: out(8)
     end function sb_sizes

     type(c_ptr) function sb_last_error() bind(C, name="sb_last_error")
       import :: c_ptr
     end function sb_last_error

     integer(c_int) function sb_version() bind(C, name="sb_version")
       import :: c_int
     end function sb_version
  end interface
end module shearbox_c
