!! swiftest_gb300_mod.f90 -- iso_c_binding interface to libswiftest_gb300.so, the GB300 (sm_103a)
!! implementation of Swiftest's integrator hot path declared in include/swiftest_gb300.h.
!!
!! Not compiled: no Fortran compiler on this box.  This is the source a Swiftest maintainer adds
!! to the build (any Fortran 2018 compiler; `optional` dummies of bind(C) interfaces arrive as
!! NULL pointers, which is how the C ABI's nullable arrays -- radius, k_plpl, lmask -- are
!! passed).  The C prototypes in include/swiftest_gb300.h are authoritative; a CPU test checks
!! that every interface below names a declared entry point with the same number of arguments.
!!
!! Layout: real(DP) :: r(NDIM, n) arrays pass as-is, since (3,n) column-major is the double[3*n]
!! layout the C ABI expects.  Logical masks pass as integer(c_int32_t) 0/1 arrays (convert with
!! merge(1, 0, lmask)).  Encounter indices come back 1-based.  Every function returns a status:
!! SWG_OK = 0, negative on error; swg_last_error(ctx) returns the message as a C string.
module swiftest_gb300_mod
   use, intrinsic :: iso_c_binding
   implicit none

   integer(c_int), parameter :: SWG_OK = 0, SWG_ERR_ARG = -1, SWG_ERR_CUDA = -2, SWG_ERR_CAPACITY = -3
   integer(c_int), parameter :: SWG_ERR_NOMEM = -4, SWG_ERR_DRIFT = -5, SWG_ERR_RECURSION = -6
   integer(c_int), parameter :: SWG_ERR_STATE = -7
   integer(c_int), parameter :: SWG_MEM_HOST = 0, SWG_MEM_DEVICE = 1
   integer(c_int), parameter :: SWG_FP64 = 0, SWG_MIXED = 1
   integer(c_int), parameter :: SWG_ENC_TRIANGULAR = 0, SWG_ENC_SORTSWEEP = 1
   integer(c_int), parameter :: SWG_WHM = 0, SWG_HELIO = 1, SWG_SYMBA = 2

   interface
      !! ---- context
      integer(c_int) function swg_create(ctx, device) bind(C, name="swg_create")
         import :: c_ptr, c_int
         type(c_ptr), intent(out) :: ctx
         integer(c_int), value :: device
      end function
      integer(c_int) function swg_destroy(ctx) bind(C, name="swg_destroy")
         import :: c_ptr, c_int
         type(c_ptr), value :: ctx
      end function
      integer(c_int) function swg_synchronize(ctx) bind(C, name="swg_synchronize")
         import :: c_ptr, c_int
         type(c_ptr), value :: ctx
      end function
      type(c_ptr) function swg_last_error(ctx) bind(C, name="swg_last_error")
         import :: c_ptr
         type(c_ptr), value :: ctx
      end function

      !! ---- pair-gravity kick (swiftest_kick.f90:69-470)
      integer(c_int) function swg_kick_getacch_int_all_tri_pl(ctx, npl, nplm, r, Gmass, radius, acc, &
                                                               precision, mem) bind(C, name="swg_kick_getacch_int_all_tri_pl")
         import :: c_ptr, c_int, c_int32_t, c_double
         type(c_ptr), value :: ctx
         integer(c_int32_t), value :: npl, nplm
         real(c_double), intent(in) :: r(3,*), Gmass(*)
         real(c_double), intent(in), optional :: radius(*)     ! absent: the norad variant
         real(c_double), intent(inout) :: acc(3,*)
         integer(c_int), value :: precision, mem
      end function
      integer(c_int) function swg_kick_getacch_int_all_flat_pl(ctx, npl, nplm, nplpl, k_plpl, r, Gmass, radius, &
                                                                acc, precision, mem) &
                                                                bind(C, name="swg_kick_getacch_int_all_flat_pl")
         import :: c_ptr, c_int, c_int32_t, c_int64_t, c_double
         type(c_ptr), value :: ctx
         integer(c_int32_t), value :: npl, nplm
         integer(c_int64_t), value :: nplpl
         integer(c_int32_t), intent(in), optional :: k_plpl(2,*)  ! absent: the GPU derives the canonical list
         real(c_double), intent(in) :: r(3,*), Gmass(*)
         real(c_double), intent(in), optional :: radius(*)
         real(c_double), intent(inout) :: acc(3,*)
         integer(c_int), value :: precision, mem
      end function
      !! device pointers and a cudaStream_t; allocates nothing (see the header)
      integer(c_int) function swg_kick_getacch_int_all_tri_pl_noalloc(npl, nplm, r, Gmass, radius, acc, stream) &
                                                                       bind(C, name="swg_kick_getacch_int_all_tri_pl_noalloc")
         import :: c_ptr, c_int, c_int32_t
         integer(c_int32_t), value :: npl, nplm
         type(c_ptr), value :: r, Gmass, radius, acc, stream
      end function
      integer(c_int) function swg_kick_getacch_int_all_tp(ctx, ntp, npl, rtp, rpl, GMpl, lmask, acc, precision, &
                                                           mem) bind(C, name="swg_kick_getacch_int_all_tp")
         import :: c_ptr, c_int, c_int32_t, c_double
         type(c_ptr), value :: ctx
         integer(c_int32_t), value :: ntp, npl
         real(c_double), intent(in) :: rtp(3,*), rpl(3,*), GMpl(*)
         integer(c_int32_t), intent(in), optional :: lmask(*)
         real(c_double), intent(inout) :: acc(3,*)
         integer(c_int), value :: precision, mem
      end function

      !! ---- Danby drift (swiftest_drift.f90:60-580)
      integer(c_int) function swg_drift_all(ctx, mu, x, v, n, lgr, inv_c2, dt, lmask, iflag, mem) &
                                            bind(C, name="swg_drift_all")
         import :: c_ptr, c_int, c_int32_t, c_double
         type(c_ptr), value :: ctx
         real(c_double), intent(in) :: mu(*)
         real(c_double), intent(inout) :: x(3,*), v(3,*)
         integer(c_int32_t), value :: n, lgr
         real(c_double), value :: inv_c2, dt
         integer(c_int32_t), intent(in), optional :: lmask(*)
         integer(c_int32_t), intent(out) :: iflag(*)
         integer(c_int), value :: mem
      end function

      !! ---- encounter checks (encounter_check.f90:14-140), caller-capacity protocol
      integer(c_int) function swg_encounter_check_all_plpl(ctx, mode, npl, r, v, renc, dt, cap, nenc, &
                                                            index1, index2, lvdotr, mem) &
                                                            bind(C, name="swg_encounter_check_all_plpl")
         import :: c_ptr, c_int, c_int32_t, c_int64_t, c_double
         type(c_ptr), value :: ctx
         integer(c_int), value :: mode
         integer(c_int32_t), value :: npl
         real(c_double), intent(in) :: r(3,*), v(3,*), renc(*)
         real(c_double), value :: dt
         integer(c_int64_t), value :: cap
         integer(c_int64_t), intent(out) :: nenc
         integer(c_int32_t), intent(out) :: index1(*), index2(*), lvdotr(*)
         integer(c_int), value :: mem
      end function
      integer(c_int) function swg_encounter_check_all_plplm(ctx, mode, nplm, nplt, rplm, vplm, rplt, vplt, rencm, &
                                                             renct, dt, cap, nenc, index1, index2, lvdotr, mem) &
                                                             bind(C, name="swg_encounter_check_all_plplm")
         import :: c_ptr, c_int, c_int32_t, c_int64_t, c_double
         type(c_ptr), value :: ctx
         integer(c_int), value :: mode
         integer(c_int32_t), value :: nplm, nplt
         real(c_double), intent(in) :: rplm(3,*), vplm(3,*), rplt(3,*), vplt(3,*), rencm(*), renct(*)
         real(c_double), value :: dt
         integer(c_int64_t), value :: cap
         integer(c_int64_t), intent(out) :: nenc
         integer(c_int32_t), intent(out) :: index1(*), index2(*), lvdotr(*)
         integer(c_int), value :: mem
      end function
      integer(c_int) function swg_encounter_check_all_pltp(ctx, mode, npl, ntp, rpl, vpl, rtp, vtp, renc, dt, cap, &
                                                            nenc, index1, index2, lvdotr, mem) &
                                                            bind(C, name="swg_encounter_check_all_pltp")
         import :: c_ptr, c_int, c_int32_t, c_int64_t, c_double
         type(c_ptr), value :: ctx
         integer(c_int), value :: mode
         integer(c_int32_t), value :: npl, ntp
         real(c_double), intent(in) :: rpl(3,*), vpl(3,*), rtp(3,*), vtp(3,*), renc(*)
         real(c_double), value :: dt
         integer(c_int64_t), value :: cap
         integer(c_int64_t), intent(out) :: nenc
         integer(c_int32_t), intent(out) :: index1(*), index2(*), lvdotr(*)
         integer(c_int), value :: mem
      end function

      !! ---- util_sort(arr, ind) (base_module.f90:1361-1472): ind = 1-based ascending permutation
      integer(c_int) function swg_util_sort_index(ctx, n, arr, ind, mem) bind(C, name="swg_util_sort_index")
         import :: c_ptr, c_int, c_int32_t, c_int64_t, c_double
         type(c_ptr), value :: ctx
         integer(c_int64_t), value :: n
         real(c_double), intent(in) :: arr(*)
         integer(c_int32_t), intent(out) :: ind(*)
         integer(c_int), value :: mem
      end function

      !! ---- orbital elements (swiftest_orbel.f90:14-1072)
      integer(c_int) function swg_orbel_el2xv(ctx, n, mu, a, e, inc, capom, omega, capm, rh, vh, mem) &
                                              bind(C, name="swg_orbel_el2xv")
         import :: c_ptr, c_int, c_int32_t, c_double
         type(c_ptr), value :: ctx
         integer(c_int32_t), value :: n
         real(c_double), intent(in) :: mu(*), a(*), e(*), inc(*), capom(*), omega(*), capm(*)
         real(c_double), intent(out) :: rh(3,*), vh(3,*)
         integer(c_int), value :: mem
      end function
      integer(c_int) function swg_orbel_xv2el(ctx, n, mu, rh, vh, a, e, inc, capom, omega, capm, varpi, lam, f, &
                                              cape, capf, mem) bind(C, name="swg_orbel_xv2el")
         import :: c_ptr, c_int, c_int32_t, c_double
         type(c_ptr), value :: ctx
         integer(c_int32_t), value :: n
         real(c_double), intent(in) :: mu(*), rh(3,*), vh(3,*)
         real(c_double), intent(out), optional :: a(*), e(*), inc(*), capom(*), omega(*), capm(*), varpi(*), &
                                                  lam(*), f(*), cape(*), capf(*)
         integer(c_int), value :: mem
      end function

      !! ---- device-resident system and step loops (whm/helio/symba_step.f90)
      integer(c_int) function swg_system_create(ctx, integrator, npl, ntp, sys) bind(C, name="swg_system_create")
         import :: c_ptr, c_int, c_int32_t
         type(c_ptr), value :: ctx
         integer(c_int), value :: integrator
         integer(c_int32_t), value :: npl, ntp
         type(c_ptr), intent(out) :: sys
      end function
      integer(c_int) function swg_system_destroy(sys) bind(C, name="swg_system_destroy")
         import :: c_ptr, c_int
         type(c_ptr), value :: sys
      end function
      integer(c_int) function swg_system_set_cb(sys, GMcb, Rcb) bind(C, name="swg_system_set_cb")
         import :: c_ptr, c_int, c_double
         type(c_ptr), value :: sys
         real(c_double), value :: GMcb, Rcb
      end function
      integer(c_int) function swg_system_set_pl(sys, rh, vh, Gmass, radius, rhill) bind(C, name="swg_system_set_pl")
         import :: c_ptr, c_int, c_double
         type(c_ptr), value :: sys
         real(c_double), intent(in) :: rh(3,*), vh(3,*), Gmass(*), radius(*), rhill(*)
      end function
      integer(c_int) function swg_system_set_tp(sys, rh, vh) bind(C, name="swg_system_set_tp")
         import :: c_ptr, c_int, c_double
         type(c_ptr), value :: sys
         real(c_double), intent(in) :: rh(3,*), vh(3,*)
      end function
      integer(c_int) function swg_system_set_param(sys, dt, loop_mode, enc_plpl, enc_pltp, rhscale, lclose, gmtiny, &
                                                   precision) bind(C, name="swg_system_set_param")
         import :: c_ptr, c_int, c_double
         type(c_ptr), value :: sys
         real(c_double), value :: dt
         integer(c_int), value :: loop_mode, enc_plpl, enc_pltp
         real(c_double), value :: rhscale
         integer(c_int), value :: lclose
         real(c_double), value :: gmtiny
         integer(c_int), value :: precision
      end function
      integer(c_int) function swg_system_initialize(sys) bind(C, name="swg_system_initialize")
         import :: c_ptr, c_int
         type(c_ptr), value :: sys
      end function
      integer(c_int) function swg_system_step(sys, nsteps) bind(C, name="swg_system_step")
         import :: c_ptr, c_int, c_int32_t
         type(c_ptr), value :: sys
         integer(c_int32_t), value :: nsteps
      end function
      integer(c_int) function swg_system_get_pl(sys, rh, vh, status) bind(C, name="swg_system_get_pl")
         import :: c_ptr, c_int, c_int32_t, c_double
         type(c_ptr), value :: sys
         real(c_double), intent(out) :: rh(3,*), vh(3,*)
         integer(c_int32_t), intent(out) :: status(*)
      end function
      integer(c_int) function swg_system_get_tp(sys, rh, vh, status) bind(C, name="swg_system_get_tp")
         import :: c_ptr, c_int, c_int32_t, c_double
         type(c_ptr), value :: sys
         real(c_double), intent(out) :: rh(3,*), vh(3,*)
         integer(c_int32_t), intent(out) :: status(*)
      end function
      integer(c_int) function swg_system_get_pl_masses(sys, Gmass, radius, rhill) &
                                                       bind(C, name="swg_system_get_pl_masses")
         import :: c_ptr, c_int, c_double
         type(c_ptr), value :: sys
         real(c_double), intent(out) :: Gmass(*), radius(*), rhill(*)
      end function
      integer(c_int) function swg_system_energy(sys, out) bind(C, name="swg_system_energy")
         import :: c_ptr, c_int, c_double
         type(c_ptr), value :: sys
         real(c_double), intent(out) :: out(*)
      end function
      !! out(4): E_collisions, L_escape(3) (G*m units)
      integer(c_int) function swg_system_collision_terms(sys, out) bind(C, name="swg_system_collision_terms")
         import :: c_ptr, c_int, c_double
         type(c_ptr), value :: sys
         real(c_double), intent(out) :: out(*)
      end function
      integer(c_int) function swg_system_stats(sys, out) bind(C, name="swg_system_stats")
         import :: c_ptr, c_int, c_int64_t
         type(c_ptr), value :: sys
         integer(c_int64_t), intent(out) :: out(*)
      end function
      integer(c_int) function swg_system_plpl_list(sys, cap, n, i1, i2) bind(C, name="swg_system_plpl_list")
         import :: c_ptr, c_int, c_int32_t, c_int64_t
         type(c_ptr), value :: sys
         integer(c_int64_t), value :: cap
         integer(c_int64_t), intent(out) :: n
         integer(c_int32_t), intent(out) :: i1(*), i2(*)
      end function
      integer(c_int) function swg_system_pltp_list(sys, cap, n, i1, i2) bind(C, name="swg_system_pltp_list")
         import :: c_ptr, c_int, c_int32_t, c_int64_t
         type(c_ptr), value :: sys
         integer(c_int64_t), value :: cap
         integer(c_int64_t), intent(out) :: n
         integer(c_int32_t), intent(out) :: i1(*), i2(*)
      end function
      integer(c_int) function swg_system_set_state(sys, rh, vh, trh, tvh) bind(C, name="swg_system_set_state")
         import :: c_ptr, c_int, c_double
         type(c_ptr), value :: sys
         real(c_double), intent(in), optional :: rh(3,*), vh(3,*), trh(3,*), tvh(3,*)
      end function
      integer(c_int) function swg_system_get_state_async(sys, rh, vh, trh, tvh) &
                                                         bind(C, name="swg_system_get_state_async")
         import :: c_ptr, c_int, c_double
         type(c_ptr), value :: sys
         real(c_double), intent(out), optional :: rh(3,*), vh(3,*), trh(3,*), tvh(3,*)
      end function

      !! ---- batched ensembles of independent systems (no single counterpart in the reference)
      integer(c_int) function swg_ensemble_create(ctx, integrator, nsys, npl, ntp, ens) &
                                                  bind(C, name="swg_ensemble_create")
         import :: c_ptr, c_int, c_int32_t
         type(c_ptr), value :: ctx
         integer(c_int), value :: integrator
         integer(c_int32_t), value :: nsys
         integer(c_int32_t), intent(in) :: npl(*), ntp(*)
         type(c_ptr), intent(out) :: ens
      end function
      integer(c_int) function swg_ensemble_destroy(ens) bind(C, name="swg_ensemble_destroy")
         import :: c_ptr, c_int
         type(c_ptr), value :: ens
      end function
      integer(c_int) function swg_ensemble_set_cb(ens, GMcb, Rcb) bind(C, name="swg_ensemble_set_cb")
         import :: c_ptr, c_int, c_double
         type(c_ptr), value :: ens
         real(c_double), intent(in) :: GMcb(*)
         real(c_double), intent(in), optional :: Rcb(*)
      end function
      integer(c_int) function swg_ensemble_set_pl(ens, rh, vh, Gmass, radius, rhill) bind(C, name="swg_ensemble_set_pl")
         import :: c_ptr, c_int, c_double
         type(c_ptr), value :: ens
         real(c_double), intent(in) :: rh(3,*), vh(3,*), Gmass(*), radius(*), rhill(*)
      end function
      integer(c_int) function swg_ensemble_set_tp(ens, rh, vh) bind(C, name="swg_ensemble_set_tp")
         import :: c_ptr, c_int, c_double
         type(c_ptr), value :: ens
         real(c_double), intent(in) :: rh(3,*), vh(3,*)
      end function
      integer(c_int) function swg_ensemble_set_param(ens, dt, rhscale, lclose, precision) &
                                                     bind(C, name="swg_ensemble_set_param")
         import :: c_ptr, c_int, c_double
         type(c_ptr), value :: ens
         real(c_double), value :: dt, rhscale
         integer(c_int), value :: lclose, precision
      end function
      integer(c_int) function swg_ensemble_set_encounter_modes(ens, enc_plpl, enc_pltp) &
                                                               bind(C, name="swg_ensemble_set_encounter_modes")
         import :: c_ptr, c_int
         type(c_ptr), value :: ens
         integer(c_int), value :: enc_plpl, enc_pltp
      end function
      integer(c_int) function swg_ensemble_set_kick_strip(ens, strip) bind(C, name="swg_ensemble_set_kick_strip")
         import :: c_ptr, c_int
         type(c_ptr), value :: ens
         integer(c_int), value :: strip
      end function
      integer(c_int) function swg_ensemble_set_kick_warps(ens, warps) bind(C, name="swg_ensemble_set_kick_warps")
         import :: c_ptr, c_int
         type(c_ptr), value :: ens
         integer(c_int), value :: warps
      end function
      integer(c_int) function swg_ensemble_set_kick_tile(ens, tile) bind(C, name="swg_ensemble_set_kick_tile")
         import :: c_ptr, c_int
         type(c_ptr), value :: ens
         integer(c_int), value :: tile
      end function
      integer(c_int) function swg_ensemble_set_kick_group(ens, group) bind(C, name="swg_ensemble_set_kick_group")
         import :: c_ptr, c_int
         type(c_ptr), value :: ens
         integer(c_int), value :: group
      end function
      integer(c_int) function swg_ensemble_set_gmtiny(ens, gmtiny) bind(C, name="swg_ensemble_set_gmtiny")
         import :: c_ptr, c_int, c_double
         type(c_ptr), value :: ens
         real(c_double), value :: gmtiny
      end function
      integer(c_int) function swg_ensemble_initialize(ens) bind(C, name="swg_ensemble_initialize")
         import :: c_ptr, c_int
         type(c_ptr), value :: ens
      end function
      integer(c_int) function swg_ensemble_step(ens, nsteps) bind(C, name="swg_ensemble_step")
         import :: c_ptr, c_int, c_int32_t
         type(c_ptr), value :: ens
         integer(c_int32_t), value :: nsteps
      end function
      integer(c_int) function swg_ensemble_get_pl(ens, rh, vh, status) bind(C, name="swg_ensemble_get_pl")
         import :: c_ptr, c_int, c_int32_t, c_double
         type(c_ptr), value :: ens
         real(c_double), intent(out) :: rh(3,*), vh(3,*)
         integer(c_int32_t), intent(out) :: status(*)
      end function
      integer(c_int) function swg_ensemble_get_tp(ens, rh, vh, status) bind(C, name="swg_ensemble_get_tp")
         import :: c_ptr, c_int, c_int32_t, c_double
         type(c_ptr), value :: ens
         real(c_double), intent(out) :: rh(3,*), vh(3,*)
         integer(c_int32_t), intent(out) :: status(*)
      end function
      integer(c_int) function swg_ensemble_get_pl_masses(ens, Gmass, radius, rhill) &
                                                         bind(C, name="swg_ensemble_get_pl_masses")
         import :: c_ptr, c_int, c_double
         type(c_ptr), value :: ens
         real(c_double), intent(out) :: Gmass(*), radius(*), rhill(*)
      end function
      integer(c_int) function swg_ensemble_energy(ens, out) bind(C, name="swg_ensemble_energy")
         import :: c_ptr, c_int, c_double
         type(c_ptr), value :: ens
         real(c_double), intent(out) :: out(*)
      end function
      integer(c_int) function swg_ensemble_collision_terms(ens, out) bind(C, name="swg_ensemble_collision_terms")
         import :: c_ptr, c_int, c_double
         type(c_ptr), value :: ens
         real(c_double), intent(out) :: out(*)
      end function
      integer(c_int) function swg_ensemble_stats(ens, out) bind(C, name="swg_ensemble_stats")
         import :: c_ptr, c_int, c_int64_t
         type(c_ptr), value :: ens
         integer(c_int64_t), intent(out) :: out(*)
      end function
      integer(c_int) function swg_ensemble_plpl_list(ens, sys, cap, n, i1, i2) bind(C, name="swg_ensemble_plpl_list")
         import :: c_ptr, c_int, c_int32_t, c_int64_t
         type(c_ptr), value :: ens
         integer(c_int32_t), value :: sys
         integer(c_int64_t), value :: cap
         integer(c_int64_t), intent(out) :: n
         integer(c_int32_t), intent(out) :: i1(*), i2(*)
      end function
      integer(c_int) function swg_ensemble_set_state(ens, rh, vh, trh, tvh) bind(C, name="swg_ensemble_set_state")
         import :: c_ptr, c_int, c_double
         type(c_ptr), value :: ens
         real(c_double), intent(in), optional :: rh(3,*), vh(3,*), trh(3,*), tvh(3,*)
      end function
      integer(c_int) function swg_ensemble_get_state_async(ens, rh, vh, trh, tvh) &
                                                           bind(C, name="swg_ensemble_get_state_async")
         import :: c_ptr, c_int, c_double
         type(c_ptr), value :: ens
         real(c_double), intent(out), optional :: rh(3,*), vh(3,*), trh(3,*), tvh(3,*)
      end function
      integer(c_int) function swg_ensemble_reset_first_step(ens) bind(C, name="swg_ensemble_reset_first_step")
         import :: c_ptr, c_int
         type(c_ptr), value :: ens
      end function
      integer(c_int) function swg_system_reset_first_step(sys) bind(C, name="swg_system_reset_first_step")
         import :: c_ptr, c_int
         type(c_ptr), value :: sys
      end function
      integer(c_int) function swg_ensemble_use_graphs(ens, enable) bind(C, name="swg_ensemble_use_graphs")
         import :: c_ptr, c_int
         type(c_ptr), value :: ens
         integer(c_int), value :: enable
      end function
   end interface
end module swiftest_gb300_mod
