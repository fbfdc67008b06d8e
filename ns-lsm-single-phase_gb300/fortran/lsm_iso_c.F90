! lsm_iso_c.F90 -- Fortran 2003 iso_c_binding interface to liblsm_gb300.so
! (include/lsm_c.h, include/lsm_batch.h) for the reference solver.
!
! Add this file to the reference's object list (before mg_driver) and link
! with -L<dir> -llsm_gb300.  Arrays are passed as the reference holds them
! (column-major, explicit bounds il:iu, jl:ju, kl:ku; vectors (1:3, ...),
! velocity q(1:4, ...)); the library stages host arrays to the GPU.
! The structs mirror lsm_grid / lsm_params / lsm_batch_instance /
! lsm_batch_config field by field.
!
! lsm_levelsetmethod_f is the drop-in for `call levelsetmethod(...)` in
! mg_driver (src/mg_driver.F90:567-580): it fills the two structs from the
! module globals the caller passes in and calls lsm_levelsetmethod.
module lsm_iso_c
   use iso_c_binding
   implicit none

   integer(c_int), parameter :: LSM_OK = 0

   type, bind(C) :: lsm_grid
      integer(c_int) :: il, iu, jl, ju, kl, ku
      integer(c_int) :: igp, jgp, kgp
      real(c_double) :: dc, de, dz
      integer(c_int) :: physical_face(6)       ! i1, im, j1, jm, k1, km: 1 where physical
   end type lsm_grid

   type, bind(C) :: lsm_params
      real(c_double) :: epslsm
      integer(c_int) :: numiter_lsm
      real(c_double) :: delti_lsm
      integer(c_int) :: RNitermax
      real(c_double) :: RNtimestep
      integer(c_int) :: RNfreq
      integer(c_int) :: btype_lsm(6)
      integer(c_int) :: bc_extrapolation_order, isnarrow
      real(c_double) :: narrowcoef
      integer(c_int) :: orderAD, sussman_correction_method
      integer(c_int) :: call_levelsetmethod, call_reinitialisation, hybrid_reinitialisation
      integer(c_int) :: TotalVolumeComputation, GlobalMassCorrection
      real(c_double) :: BigPhi, epsReinitialisation
      integer(c_int) :: M_Sphi0, reinit_scheme, write_global_volume
      integer(c_int) :: OrderReinitialisationBoundaries, ENOBCReinitialisation
      real(c_double) :: ConvergenceToleranceGeomReini
   end type lsm_params

   type, bind(C) :: lsm_geom_info
      integer(c_int) :: nnodes, ntetrahedra, nsecond, newton_iterations, newton_converged
      real(c_double) :: C
   end type lsm_geom_info

   type, bind(C) :: lsm_batch_instance
      integer(c_int) :: ni, nj, nk
      real(c_double) :: dt, dtau, eps
   end type lsm_batch_instance

   type, bind(C) :: lsm_batch_config
      integer(c_int) :: RNitermax, btype_lsm(6)
      real(c_double) :: BigPhi
      integer(c_int) :: use_graph, autotune, shape, precision, adjoint_mode, mass_correction
   end type lsm_batch_config

   interface
      subroutine lsm_params_default(p) bind(C, name="lsm_params_default")
         import :: lsm_params
         type(lsm_params), intent(out) :: p
      end subroutine

      integer(c_int) function lsm_create(h, device, stream) bind(C, name="lsm_create")
         import :: c_int, c_ptr
         type(c_ptr), intent(out) :: h
         integer(c_int), value :: device
         type(c_ptr), value :: stream
      end function

      integer(c_int) function lsm_destroy(h) bind(C, name="lsm_destroy")
         import :: c_int, c_ptr
         type(c_ptr), value :: h
      end function

      integer(c_int) function lsm_set_exchange_callback(h, fn, user) bind(C, name="lsm_set_exchange_callback")
         import :: c_int, c_ptr, c_funptr
         type(c_ptr), value :: h
         type(c_funptr), value :: fn
         type(c_ptr), value :: user
      end function

      type(c_ptr) function lsm_last_error(h) bind(C, name="lsm_last_error")
         import :: c_ptr
         type(c_ptr), value :: h
      end function

      integer(c_int) function lsm_levelsetmethod(h, g, p, q, csi, eta, zet, aj, phi, phi_n, x, y, z, it, vols) &
            bind(C, name="lsm_levelsetmethod")
         import :: c_int, c_ptr, c_double, lsm_grid, lsm_params
         type(c_ptr), value :: h
         type(lsm_grid), intent(in) :: g
         type(lsm_params), intent(in) :: p
         real(c_double), intent(in) :: q(*), csi(*), eta(*), zet(*), aj(*), phi_n(*), x(*), y(*), z(*)
         real(c_double), intent(inout) :: phi(*)
         integer(c_int), value :: it
         real(c_double), intent(out) :: vols(4)
      end function

      integer(c_int) function lsm_rhs_contra_j(h, g, q, csi, eta, zet, aj, ucn_j) bind(C, name="lsm_rhs_contra_j")
         import :: c_int, c_ptr, c_double, lsm_grid
         type(c_ptr), value :: h
         type(lsm_grid), intent(in) :: g
         real(c_double), intent(in) :: q(*), csi(*), eta(*), zet(*), aj(*)
         real(c_double), intent(out) :: ucn_j(*)
      end function

      integer(c_int) function lsm_calc_rh_ad_weno3(h, g, phi, ucn_j, nodes, rh) bind(C, name="lsm_calc_rh_ad_weno3")
         import :: c_int, c_ptr, c_double, lsm_grid
         type(c_ptr), value :: h
         type(lsm_grid), intent(in) :: g
         real(c_double), intent(in) :: phi(*), ucn_j(*)
         integer(c_int), intent(in) :: nodes(*)
         real(c_double), intent(out) :: rh(*)
      end function

      integer(c_int) function lsm_calc_rh_ad(h, g, phi, ucn_j, nodes, rh) bind(C, name="lsm_calc_rh_ad")
         import :: c_int, c_ptr, c_double, lsm_grid
         type(c_ptr), value :: h
         type(lsm_grid), intent(in) :: g
         real(c_double), intent(in) :: phi(*), ucn_j(*)
         integer(c_int), intent(in) :: nodes(*)
         real(c_double), intent(out) :: rh(*)
      end function

      integer(c_int) function lsm_ad_rktvd3(h, g, p, phi_n1, phi_n, nodes, ucn_j, aj) bind(C, name="lsm_ad_rktvd3")
         import :: c_int, c_ptr, c_double, lsm_grid, lsm_params
         type(c_ptr), value :: h
         type(lsm_grid), intent(in) :: g
         type(lsm_params), intent(in) :: p
         real(c_double), intent(out) :: phi_n1(*)
         real(c_double), intent(in) :: phi_n(*), ucn_j(*), aj(*)
         integer(c_int), intent(in) :: nodes(*)
      end function

      integer(c_int) function lsm_bcond_lsm(h, g, p, phi) bind(C, name="lsm_bcond_lsm")
         import :: c_int, c_ptr, c_double, lsm_grid, lsm_params
         type(c_ptr), value :: h
         type(lsm_grid), intent(in) :: g
         type(lsm_params), intent(in) :: p
         real(c_double), intent(inout) :: phi(*)
      end function

      integer(c_int) function lsm_reinitialization(h, g, p, phi0, csi, eta, zet, phi_out) &
            bind(C, name="lsm_reinitialization")
         import :: c_int, c_ptr, c_double, lsm_grid, lsm_params
         type(c_ptr), value :: h
         type(lsm_grid), intent(in) :: g
         type(lsm_params), intent(in) :: p
         real(c_double), intent(in) :: phi0(*), csi(*), eta(*), zet(*)
         real(c_double), intent(out) :: phi_out(*)
      end function

      integer(c_int) function lsm_reinitialisation_test2(h, g, p, phizero, csi, eta, zet, phi_out, iters) &
            bind(C, name="lsm_reinitialisation_test2")
         import :: c_int, c_ptr, c_double, lsm_grid, lsm_params
         type(c_ptr), value :: h
         type(lsm_grid), intent(in) :: g
         type(lsm_params), intent(in) :: p
         real(c_double), intent(in) :: phizero(*), csi(*), eta(*), zet(*)
         real(c_double), intent(out) :: phi_out(*)
         integer(c_int), intent(out) :: iters
      end function

      integer(c_int) function lsm_calc_normgrad_d(h, g, p, phi_rn, phizero, csi, eta, zet, normgrad) &
            bind(C, name="lsm_calc_normgrad_d")
         import :: c_int, c_ptr, c_double, lsm_grid, lsm_params
         type(c_ptr), value :: h
         type(lsm_grid), intent(in) :: g
         type(lsm_params), intent(in) :: p
         real(c_double), intent(in) :: phi_rn(*), phizero(*), csi(*), eta(*), zet(*)
         real(c_double), intent(out) :: normgrad(*)
      end function

      integer(c_int) function lsm_narrowband(h, g, p, phi_n, nband) bind(C, name="lsm_narrowband")
         import :: c_int, c_ptr, c_double, lsm_grid, lsm_params
         type(c_ptr), value :: h
         type(lsm_grid), intent(in) :: g
         type(lsm_params), intent(in) :: p
         real(c_double), intent(in) :: phi_n(*)
         integer(c_int), intent(out) :: nband(*)
      end function

      integer(c_int) function lsm_total_water_volume(h, g, phi, x, y, z, vols, nodes) &
            bind(C, name="lsm_total_water_volume")
         import :: c_int, c_ptr, c_double, lsm_grid
         type(c_ptr), value :: h
         type(lsm_grid), intent(in) :: g
         real(c_double), intent(in) :: phi(*), x(*), y(*), z(*)
         real(c_double), intent(out) :: vols(4)
         integer(c_int), intent(out) :: nodes(*)
      end function

      integer(c_int) function lsm_convergence_volume(h, vol) bind(C, name="lsm_convergence_volume")
         import :: c_int, c_ptr, c_double
         type(c_ptr), value :: h
         real(c_double), intent(out) :: vol
      end function

      ! geometric_reinitialisation (the hybrid path): phicorrected in/out,
      ! interface_nodes_id out (pnode ids, -1, 0)
      integer(c_int) function lsm_geometric_reinitialisation(h, g, p, phizero, x, y, z, total_water_volume, &
            phicorrected, interface_nodes_id, info) bind(C, name="lsm_geometric_reinitialisation")
         import :: c_int, c_ptr, c_double, lsm_grid, lsm_params, lsm_geom_info
         type(c_ptr), value :: h
         type(lsm_grid), intent(in) :: g
         type(lsm_params), intent(in) :: p
         real(c_double), intent(in) :: phizero(*), x(*), y(*), z(*)
         real(c_double), value :: total_water_volume
         real(c_double), intent(inout) :: phicorrected(*)
         integer(c_int), intent(out) :: interface_nodes_id(*)
         type(lsm_geom_info), intent(out) :: info
      end function

      integer(c_int) function lsm_get_gfm_list(h, g, p, phi, count, list, ld) bind(C, name="lsm_get_gfm_list")
         import :: c_int, c_ptr, c_double, lsm_grid, lsm_params
         type(c_ptr), value :: h
         type(lsm_grid), intent(in) :: g
         type(lsm_params), intent(in) :: p
         real(c_double), intent(in) :: phi(*)
         integer(c_int), intent(out) :: count
         integer(c_int), intent(out) :: list(*)
         integer(c_int), value :: ld
      end function

      integer(c_int) function lsm_mg_metrics(h, g, x, y, z, csi, eta, zet, aj) bind(C, name="lsm_mg_metrics")
         import :: c_int, c_ptr, c_double, lsm_grid
         type(c_ptr), value :: h
         type(lsm_grid), intent(in) :: g
         real(c_double), intent(in) :: x(*), y(*), z(*)
         real(c_double), intent(out) :: csi(*), eta(*), zet(*), aj(*)
      end function

      ! ---- batched path (include/lsm_batch.h)
      integer(c_int) function lsm_batch_create(h, device, stream, n, inst, cfg) bind(C, name="lsm_batch_create")
         import :: c_int, c_ptr, lsm_batch_instance, lsm_batch_config
         type(c_ptr), intent(out) :: h
         integer(c_int), value :: device, n
         type(c_ptr), value :: stream
         type(lsm_batch_instance), intent(in) :: inst(*)
         type(lsm_batch_config), intent(in) :: cfg
      end function

      integer(c_int) function lsm_batch_destroy(h) bind(C, name="lsm_batch_destroy")
         import :: c_int, c_ptr
         type(c_ptr), value :: h
      end function

      integer(c_int) function lsm_batch_set_geometry(h, k, x, y, z, csi, eta, zet) bind(C, name="lsm_batch_set_geometry")
         import :: c_int, c_ptr, c_double
         type(c_ptr), value :: h
         integer(c_int), value :: k
         real(c_double), intent(in) :: x(*), y(*), z(*), csi(*), eta(*), zet(*)
      end function

      integer(c_int) function lsm_batch_set_velocity(h, k, q) bind(C, name="lsm_batch_set_velocity")
         import :: c_int, c_ptr, c_double
         type(c_ptr), value :: h
         integer(c_int), value :: k
         real(c_double), intent(in) :: q(*)
      end function

      integer(c_int) function lsm_batch_set_phi(h, k, phi) bind(C, name="lsm_batch_set_phi")
         import :: c_int, c_ptr, c_double
         type(c_ptr), value :: h
         integer(c_int), value :: k
         real(c_double), intent(in) :: phi(*)
      end function

      integer(c_int) function lsm_batch_get_phi(h, k, phi) bind(C, name="lsm_batch_get_phi")
         import :: c_int, c_ptr, c_double
         type(c_ptr), value :: h
         integer(c_int), value :: k
         real(c_double), intent(out) :: phi(*)
      end function

      ! q(k) / phi(k): c_loc of instance k's array, one per instance
      integer(c_int) function lsm_batch_set_velocities(h, q) bind(C, name="lsm_batch_set_velocities")
         import :: c_int, c_ptr
         type(c_ptr), value :: h
         type(c_ptr), intent(in) :: q(*)
      end function

      integer(c_int) function lsm_batch_get_phis(h, phi) bind(C, name="lsm_batch_get_phis")
         import :: c_int, c_ptr
         type(c_ptr), value :: h
         type(c_ptr), intent(in) :: phi(*)
      end function

      integer(c_int) function lsm_batch_step(h, nsteps, vols) bind(C, name="lsm_batch_step")
         import :: c_int, c_ptr, c_double
         type(c_ptr), value :: h
         integer(c_int), value :: nsteps
         real(c_double), intent(out) :: vols(*)
      end function
      integer(c_int) function lsm_batch_water_volume(h, vols) bind(C, name="lsm_batch_water_volume")
         import :: c_int, c_ptr, c_double
         type(c_ptr), value :: h
         real(c_double), intent(out) :: vols(*)
      end function
      integer(c_int) function lsm_batch_set_mass_target(h, inst, volume) bind(C, name="lsm_batch_set_mass_target")
         import :: c_int, c_ptr, c_double
         type(c_ptr), value :: h
         integer(c_int), value :: inst
         real(c_double), value :: volume
      end function
      integer(c_int) function lsm_batch_mass_state(h, state) bind(C, name="lsm_batch_mass_state")
         import :: c_int, c_ptr, c_double
         type(c_ptr), value :: h
         real(c_double), intent(out) :: state(*)
      end function
   end interface

contains

   ! levelsetmethod through the GPU library: `h` from lsm_create (or
   ! c_null_ptr for the library's default handle on the current GPU), the
   ! rank's bounds, ghost planes, grid spacings and physical faces in `g`,
   ! the global_lsm switches in `p` (lsm_params_default + the deck).
   subroutine lsm_levelsetmethod_f(h, g, p, q, csi, eta, zet, aj, phi, phi_n, x, y, z, iteraciontiempo, vols)
      type(c_ptr), intent(in) :: h
      type(lsm_grid), intent(in) :: g
      type(lsm_params), intent(in) :: p
      real(c_double), intent(in) :: q(*), csi(*), eta(*), zet(*), aj(*), phi_n(*), x(*), y(*), z(*)
      real(c_double), intent(inout) :: phi(*)
      integer, intent(in) :: iteraciontiempo
      real(c_double), intent(out) :: vols(4)
      integer(c_int) :: st
      st = lsm_levelsetmethod(h, g, p, q, csi, eta, zet, aj, phi, phi_n, x, y, z, &
                              int(iteraciontiempo, c_int), vols)
      if (st /= LSM_OK) then
         write (*, '(a, i0)') 'lsm_levelsetmethod failed, status ', st
         stop
      end if
   end subroutine lsm_levelsetmethod_f

end module lsm_iso_c
