! ocean_gpu_mod.f90 -- iso_c_binding interface to libocean_gpu.so for ocean.x.
!
! A maintainer adds this module to OCEAN2/ and calls the wrappers from
! OCEAN_action.f90 / OCEAN_haydock.f90 / OCEAN_gmres.f90 in place of the CPU calls.
! Not compiled in this repository (no Fortran compiler here); the C ABI it binds
! is tested from C/Python.
module ocean_gpu_mod
  use iso_c_binding
  implicit none
  private

  integer(c_int), parameter, public :: OCN_PREC_FP64 = 0, OCN_PREC_MIXED = 1

  type, bind(C), public :: ocn_dims
    integer(c_int) :: num_bands
    integer(c_int) :: kmesh(3)
    integer(c_int) :: xmesh(3)
    integer(c_int) :: nalpha
    integer(c_int) :: nspn
    integer(c_int) :: core_l
    integer(c_int) :: precision
    integer(c_int) :: device
    integer(c_int) :: nvec
  end type

  type, bind(C), public :: ocn_system
    real(c_double) :: celvol
    real(c_double) :: interaction_scale
    integer(c_int) :: e0, long_range, mult
    integer(c_int) :: nhflag(6)
  end type

  type, bind(C), public :: ocn_lr_params
    real(c_double) :: avec(9)
    real(c_double) :: tau(3)
    real(c_double) :: epsilon0
    real(c_double) :: interaction_scale
    integer(c_int) :: nptab
    type(c_ptr) :: rtab, ptab
    integer(c_int) :: isolated
    real(c_double) :: iso_cut
    integer(c_int) :: pbc(3)
    integer(c_int) :: have_eps3d
    real(c_double) :: epsilon3d(3)
    integer(c_int) :: xshift_override(3)
  end type

  type, bind(C), public :: ocn_cf_params
    real(c_double) :: el, eh, gam0, ebase, gam_gauss
    integer(c_int) :: ne
    real(c_double) :: ucvol
    integer(c_int) :: old_broaden
    real(c_double) :: nval, eps
  end type

  type, bind(C), public :: ocn_gmres_params
    integer(c_int) :: depth
    real(c_double) :: resolution, preconditioner, convergence
    integer(c_int) :: max_restarts
  end type

  public :: ocn_ctx_create, ocn_ctx_destroy, ocn_set_system, ocn_set_energies, ocn_set_allow
  public :: ocn_set_bloch, ocn_lr_init, ocn_soprep, ocn_apply_H, ocn_haydock, ocn_spectrum_cf
  public :: ocn_gmres, ocn_redtrid, ocn_gmres_set_lanes, ocn_set_haydock_conv, ocn_mult_exchange

  type, bind(C), public :: ocn_haydock_conv
    real(c_double) :: threshold
    integer(c_int) :: spacing, ne
    real(c_double) :: el, eh, gam0, kpref
  end type

  type, bind(C) :: ocn_val_dims
    integer(c_int) :: nc, nv, kmesh(3), xmesh(3), precision, device, nspn, vspin
  end type

  interface
    integer(c_int) function ocn_ctx_create(dims, ctx) bind(C, name="ocn_ctx_create")
      import :: c_int, c_ptr, ocn_dims
      type(ocn_dims), intent(in) :: dims
      type(c_ptr), intent(out) :: ctx
    end function
    integer(c_int) function ocn_ctx_destroy(ctx) bind(C, name="ocn_ctx_destroy")
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx
    end function
    integer(c_int) function ocn_set_system(ctx, sys) bind(C, name="ocn_set_system")
      import :: c_int, c_ptr, ocn_system
      type(c_ptr), value :: ctx
      type(ocn_system), intent(in) :: sys
    end function
    integer(c_int) function ocn_set_energies(ctx, re, im) bind(C, name="ocn_set_energies")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: ctx
      real(c_double), intent(in) :: re(*), im(*)
    end function
    integer(c_int) function ocn_set_allow(ctx, allow) bind(C, name="ocn_set_allow")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: ctx
      real(c_double), intent(in) :: allow(*)
    end function
    integer(c_int) function ocn_set_bloch(ctx, re, im) bind(C, name="ocn_set_bloch")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: ctx
      real(c_double), intent(in) :: re(*), im(*)
    end function
    integer(c_int) function ocn_lr_init(ctx, p) bind(C, name="ocn_lr_init")
      import :: c_int, c_ptr, ocn_lr_params
      type(c_ptr), value :: ctx
      type(ocn_lr_params), intent(in) :: p
    end function
    integer(c_int) function ocn_soprep(ctx, xi) bind(C, name="ocn_soprep")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: ctx
      real(c_double), value :: xi
    end function
    integer(c_int) function ocn_apply_H(ctx, in_r, in_i, out_r, out_i, hflag, backwards) &
        bind(C, name="ocn_apply_H")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: ctx
      real(c_double), intent(in) :: in_r(*), in_i(*)
      real(c_double), intent(out) :: out_r(*), out_i(*)
      integer(c_int), intent(in) :: hflag(6)
      integer(c_int), value :: backwards
    end function
    integer(c_int) function ocn_haydock(ctx, p0r, p0i, niter, real_a, imag_a, real_b, ndone) &
        bind(C, name="ocn_haydock")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: ctx
      real(c_double), intent(in) :: p0r(*), p0i(*)
      integer(c_int), value :: niter
      real(c_double), intent(out) :: real_a(0:*), imag_a(0:*), real_b(0:*)
      integer(c_int), intent(out) :: ndone
    end function
    integer(c_int) function ocn_haydock_block(ctx, nv, p0r, p0i, niter, real_a, imag_a, real_b, &
        ndone) bind(C, name="ocn_haydock_block")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: ctx
      integer(c_int), value :: nv
      real(c_double), intent(in) :: p0r(*), p0i(*)
      integer(c_int), value :: niter
      real(c_double), intent(out) :: real_a(0:*), imag_a(0:*), real_b(0:*)
      integer(c_int), intent(out) :: ndone(*)
    end function
    integer(c_int) function ocn_apply_H_block(ctx, nv, in_r, in_i, out_r, out_i, hflag, backwards) &
        bind(C, name="ocn_apply_H_block")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: ctx
      integer(c_int), value :: nv
      real(c_double), intent(in) :: in_r(*), in_i(*)
      real(c_double), intent(out) :: out_r(*), out_i(*)
      integer(c_int), intent(in) :: hflag(6)
      integer(c_int), value :: backwards
    end function
    integer(c_int) function ocn_spectrum_cf(real_a, imag_a, real_b, iter, kpref, p, out) &
        bind(C, name="ocn_spectrum_cf")
      import :: c_int, c_double, ocn_cf_params
      real(c_double), intent(in) :: real_a(0:*), imag_a(0:*), real_b(0:*)
      integer(c_int), value :: iter
      real(c_double), value :: kpref
      type(ocn_cf_params), intent(in) :: p
      real(c_double), intent(out) :: out(9, *)
    end function
    integer(c_int) function ocn_gmres(ctx, hay_r, hay_i, kpref, energies, nomega, p, out_re, &
        out_im, rel_err, iters) bind(C, name="ocn_gmres")
      import :: c_int, c_ptr, c_double, ocn_gmres_params
      type(c_ptr), value :: ctx
      real(c_double), intent(in) :: hay_r(*), hay_i(*)
      real(c_double), value :: kpref
      real(c_double), intent(in) :: energies(*)
      integer(c_int), value :: nomega
      type(ocn_gmres_params), intent(in) :: p
      real(c_double), intent(out) :: out_re(*), out_im(*), rel_err(*)
      integer(c_int), intent(out) :: iters(*)
    end function
    integer(c_int) function ocn_gmres_set_lanes(ctx, nlanes) bind(C, name="ocn_gmres_set_lanes")
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx
      integer(c_int), value :: nlanes
    end function
    ! haydockconv.ipt present (sys%earlyExit): set before OCEAN_haydock_do's run
    integer(c_int) function ocn_set_haydock_conv(ctx, p) bind(C, name="ocn_set_haydock_conv")
      import :: c_int, c_ptr, ocn_haydock_conv
      type(c_ptr), value :: ctx
      type(ocn_haydock_conv), intent(in) :: p
    end function
    ! nbsemhsetup2 for one lv: mhr_l / mhi_l(mham, mham) in Hartree
    integer(c_int) function ocn_mult_exchange(lc, lv, np, kfl, kfh, fk, scfk, kgl, kgh, gk, scgk, scfac, &
        mhr, mhi) bind(C, name="ocn_mult_exchange")
      import :: c_int, c_double
      integer(c_int), value :: lc, lv, np, kfl, kfh, kgl, kgh
      real(c_double), intent(in) :: fk(*), scfk(*), gk(*), scgk(*)
      real(c_double), value :: scfac
      real(c_double), intent(out) :: mhr(*), mhi(*)
    end function
    integer(c_int) function ocn_redtrid(n, real_a, real_b, w) bind(C, name="ocn_redtrid")
      import :: c_int, c_double
      integer(c_int), value :: n
      real(c_double), intent(in) :: real_a(0:*), real_b(0:*)
      real(c_double), intent(out) :: w(*)
    end function
    ! ---- valence BSE (one spin channel, resonant pairs)
    integer(c_int) function ocn_val_create(dims, ctx) bind(C, name="ocn_val_create")
      import :: c_int, c_ptr, ocn_val_dims
      type(ocn_val_dims), intent(in) :: dims
      type(c_ptr), intent(out) :: ctx
    end function
    integer(c_int) function ocn_val_destroy(ctx) bind(C, name="ocn_val_destroy")
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx
    end function
    integer(c_int) function ocn_val_set_energies(ctx, re, im) bind(C, name="ocn_val_set_energies")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: ctx
      real(c_double), intent(in) :: re(*), im(*)
    end function
    integer(c_int) function ocn_val_set_allow(ctx, allow) bind(C, name="ocn_val_set_allow")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: ctx
      real(c_double), intent(in) :: allow(*)
    end function
    integer(c_int) function ocn_val_set_states(ctx, con_r, con_i, val_r, val_i) bind(C, name="ocn_val_set_states")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: ctx
      real(c_double), intent(in) :: con_r(*), con_i(*), val_r(*), val_i(*)
    end function
    integer(c_int) function ocn_val_set_bubble(ctx, bubble) bind(C, name="ocn_val_set_bubble")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: ctx
      real(c_double), intent(in) :: bubble(*)
    end function
    integer(c_int) function ocn_val_set_ladder(ctx, ladder) bind(C, name="ocn_val_set_ladder")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: ctx
      real(c_double), intent(in) :: ladder(*)
    end function
    integer(c_int) function ocn_val_set_fxc(ctx, fxc) bind(C, name="ocn_val_set_fxc")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: ctx
      real(c_double), intent(in) :: fxc(*)
    end function
    integer(c_int) function ocn_val_apply_H(ctx, in_r, in_i, out_r, out_i, flags, backwards) &
        bind(C, name="ocn_val_apply_H")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: ctx
      real(c_double), intent(in) :: in_r(*), in_i(*)
      real(c_double), intent(out) :: out_r(*), out_i(*)
      integer(c_int), intent(in) :: flags(3)
      integer(c_int), value :: backwards
    end function
    integer(c_int) function ocn_val_haydock(ctx, psi0_r, psi0_i, niter, flags, real_a, imag_a, real_b, &
        niter_done) bind(C, name="ocn_val_haydock")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: ctx
      real(c_double), intent(in) :: psi0_r(*), psi0_i(*)
      integer(c_int), value :: niter
      integer(c_int), intent(in) :: flags(3)
      real(c_double), intent(out) :: real_a(0:*), imag_a(0:*), real_b(0:*)
      integer(c_int), intent(out) :: niter_done
    end function
  end interface
end module ocean_gpu_mod
