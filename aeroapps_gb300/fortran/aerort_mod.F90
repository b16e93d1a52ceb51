! ISO_C_BINDING shim between the AeroApps Fortran drivers and libaerort.so.
!
! A maintainer adds this module next to geo_vlidort/VLIDORT_LAMBERT.F90 and
! links with -L<repo>/aeroapps_gb300/_build -laerort -lcudart.  The drop-in
! subroutines keep the reference's argument lists, so a call site changes
! only the routine name:
!   geo_vlidort.F90:598-603   call VLIDORT_Scalar_Lambert(...)  -> VLIDORT_Scalar_Lambert_GPU(...)
!   geo_vlidort.F90:612-619   call VLIDORT_Vector_Lambert(...)  -> VLIDORT_Vector_Lambert_GPU(...)
!   geo_vlidort.F90:640-646   call VLIDORT_Scalar_LandMODIS(...) -> VLIDORT_Scalar_LandMODIS_GPU(...)
!   geo_vlidort_ocean.F90:536-544 call VLIDORT_Scalar_GissCX(...) -> VLIDORT_Scalar_GissCX_GPU(...)
!   (VLIDORT_Scalar_CX, VLIDORT_BRDF_CX.F90:420-584, has VLIDORT_Scalar_CX_GPU)
!   geo_vlidort.F90:558-560   call VLIDORT_ROT_CALC(...)        -> VLIDORT_ROT_CALC_GPU(...)
! The C prototypes are include/aerort.h; arrays pass by address in Fortran
! (column-major) order with the reference's shapes, scalars by value.  Every
! entry point returns the reference's rc (plus 1001 CUDA error, 1002 invalid
! argument, 1003 stream count not built); the message of a nonzero rc is
! available from aerort_last_error().
module aerort_mod
  use iso_c_binding
  implicit none
  private
  public :: VLIDORT_Scalar_Lambert_GPU, VLIDORT_Vector_Lambert_GPU, VLIDORT_Scalar_LandMODIS_GPU
  public :: VLIDORT_Scalar_CX_GPU, VLIDORT_Scalar_GissCX_GPU
  public :: VLIDORT_ROT_CALC_GPU, getEdgeVars_GPU
  public :: aerort_mie_table_desc, aerort_mie_create, aerort_mie_destroy, aerort_get_aop_vector
  public :: aerort_get_aop_scalar, aerort_mie_table_interp, aerort_last_error_string

  ! mirrors aerort_mie_table_desc of include/aerort.h: one Chem_MieTable,
  ! already on the requested channels (REAL*4 arrays, c_loc of each)
  type, bind(C) :: aerort_mie_table_desc
    integer(c_int) :: nrh, nbin, nmom, npol
    type(c_ptr)    :: rh, bext, bsca, g, pmom
  end type

  interface
    integer(c_int) function aerort_vlidort_scalar_lambert(km, nch, nobs, channels, nstreams, plane_parallel, &
        nMom, nPol, ROT, depol, tau, ssa, g, pmom, pe, he, te, albedo, solar_zenith, relat_azymuth,          &
        sensor_zenith, MISSING, verbose, radiance_VL, reflectance_VL) bind(C, name="aerort_vlidort_scalar_lambert")
      import :: c_int, c_double
      integer(c_int), value :: km, nch, nobs, nstreams, plane_parallel, nMom, nPol, verbose
      real(c_double), intent(in) :: channels(*), ROT(*), depol(*), tau(*), ssa(*), g(*), pmom(*)
      real(c_double), intent(in) :: pe(*), he(*), te(*), albedo(*), solar_zenith(*), relat_azymuth(*)
      real(c_double), intent(in) :: sensor_zenith(*)
      real(c_double), value :: MISSING
      real(c_double), intent(out) :: radiance_VL(*), reflectance_VL(*)
    end function

    integer(c_int) function aerort_vlidort_vector_lambert(km, nch, nobs, channels, nstreams, plane_parallel, &
        nMom, nPol, ROT, depol, alpha, tau, ssa, pmom, pe, he, te, albedo, solar_zenith, relat_azymuth,      &
        sensor_zenith, flux_factor, MISSING, verbose, radiance_VL, reflectance_VL, Q, U)                    &
        bind(C, name="aerort_vlidort_vector_lambert")
      import :: c_int, c_double
      integer(c_int), value :: km, nch, nobs, nstreams, plane_parallel, nMom, nPol, verbose
      real(c_double), intent(in) :: channels(*), ROT(*), depol(*), alpha(*), tau(*), ssa(*), pmom(*)
      real(c_double), intent(in) :: pe(*), he(*), te(*), albedo(*), solar_zenith(*), relat_azymuth(*)
      real(c_double), intent(in) :: sensor_zenith(*), flux_factor(*)
      real(c_double), value :: MISSING
      real(c_double), intent(out) :: radiance_VL(*), reflectance_VL(*), Q(*), U(*)
    end function

    integer(c_int) function aerort_vlidort_scalar_landmodis(km, nch, nobs, channels, nstreams, plane_parallel, &
        nMom, nPol, ROT, depol, tau, ssa, g, pmom, pe, he, te, kernel_wt, param, solar_zenith, relat_azymuth,    &
        sensor_zenith, MISSING, verbose, radiance_VL_SURF, reflectance_VL_SURF, BR)                             &
        bind(C, name="aerort_vlidort_scalar_landmodis")
      import :: c_int, c_double
      integer(c_int), value :: km, nch, nobs, nstreams, plane_parallel, nMom, nPol, verbose
      real(c_double), intent(in) :: channels(*), ROT(*), depol(*), tau(*), ssa(*), g(*), pmom(*)
      real(c_double), intent(in) :: pe(*), he(*), te(*), kernel_wt(*), param(*), solar_zenith(*)
      real(c_double), intent(in) :: relat_azymuth(*), sensor_zenith(*)
      real(c_double), value :: MISSING
      real(c_double), intent(out) :: radiance_VL_SURF(*), reflectance_VL_SURF(*), BR(*)
    end function

    integer(c_int) function aerort_vlidort_scalar_cx(km, nch, nobs, channels, nstreams, plane_parallel, &
        nMom, nPol, ROT, depol, tau, ssa, g, pmom, pe, he, te, U10m, V10m, mr, solar_zenith, relat_azymuth, &
        sensor_zenith, MISSING, verbose, radiance_VL_SURF, reflectance_VL_SURF, BRDF)                      &
        bind(C, name="aerort_vlidort_scalar_cx")
      import :: c_int, c_double
      integer(c_int), value :: km, nch, nobs, nstreams, plane_parallel, nMom, nPol, verbose
      real(c_double), intent(in) :: channels(*), ROT(*), depol(*), tau(*), ssa(*), g(*), pmom(*)
      real(c_double), intent(in) :: pe(*), he(*), te(*), U10m(*), V10m(*), mr(*), solar_zenith(*)
      real(c_double), intent(in) :: relat_azymuth(*), sensor_zenith(*)
      real(c_double), value :: MISSING
      real(c_double), intent(out) :: radiance_VL_SURF(*), reflectance_VL_SURF(*), BRDF(*)
    end function

    integer(c_int) function aerort_vlidort_scalar_gisscx(km, nch, nobs, channels, nstreams, plane_parallel, &
        nMom, nPol, ROT, depol, tau, ssa, g, pmom, pe, he, te, U10m, V10m, mr, solar_zenith, relat_azymuth,    &
        sensor_zenith, MISSING, verbose, radiance_VL_SURF, reflectance_VL_SURF, BRDF)                         &
        bind(C, name="aerort_vlidort_scalar_gisscx")
      import :: c_int, c_double
      integer(c_int), value :: km, nch, nobs, nstreams, plane_parallel, nMom, nPol, verbose
      real(c_double), intent(in) :: channels(*), ROT(*), depol(*), tau(*), ssa(*), g(*), pmom(*)
      real(c_double), intent(in) :: pe(*), he(*), te(*), U10m(*), V10m(*), mr(*), solar_zenith(*)
      real(c_double), intent(in) :: relat_azymuth(*), sensor_zenith(*)
      real(c_double), value :: MISSING
      real(c_double), intent(out) :: radiance_VL_SURF(*), reflectance_VL_SURF(*), BRDF(*)
    end function

    integer(c_int) function aerort_vlidort_rot_calc(km, nch, nobs, channels, pe, he, te, MISSING, verbose, &
        ROT, depol) bind(C, name="aerort_vlidort_rot_calc")
      import :: c_int, c_double
      integer(c_int), value :: km, nch, nobs, verbose
      real(c_double), intent(in) :: channels(*), pe(*), he(*), te(*)
      real(c_double), value :: MISSING
      real(c_double), intent(out) :: ROT(*), depol(*)
    end function

    integer(c_int) function aerort_get_edge_vars(km, nobs, airdens, delp, ptop, pe, ze, te) &
        bind(C, name="aerort_get_edge_vars")
      import :: c_int, c_float
      integer(c_int), value :: km, nobs
      real(c_float), intent(in)  :: airdens(*), delp(*)
      real(c_float), value :: ptop
      real(c_float), intent(out) :: pe(*), ze(*), te(*)
    end function

    integer(c_int) function aerort_mie_create(ntables, tables, nch, channels_m, mie) bind(C, name="aerort_mie_create")
      import :: c_int, c_float, c_ptr, aerort_mie_table_desc
      integer(c_int), value :: ntables, nch
      type(aerort_mie_table_desc), intent(in) :: tables(*)
      real(c_float), intent(in) :: channels_m(*)
      type(c_ptr), intent(out) :: mie
    end function

    integer(c_int) function aerort_mie_destroy(mie) bind(C, name="aerort_mie_destroy")
      import :: c_int, c_ptr
      type(c_ptr), value :: mie
    end function

    integer(c_int) function aerort_get_aop_vector(mie, km, nobs, nch, nq, channels_nm, q_table, q_bin, qm, rh, &
        nMom, nPol, tau, ssa, g, pmom) bind(C, name="aerort_get_aop_vector")
      import :: c_int, c_float, c_ptr
      type(c_ptr), value :: mie
      integer(c_int), value :: km, nobs, nch, nq, nMom, nPol
      real(c_float), intent(in) :: channels_nm(*), qm(*), rh(*)
      integer(c_int), intent(in) :: q_table(*), q_bin(*)
      real(c_float), intent(out) :: tau(*), ssa(*), g(*), pmom(*)
    end function

    integer(c_int) function aerort_get_aop_scalar(mie, km, nobs, nch, nq, channels_nm, q_table, q_bin, qm, rh, &
        tau, ssa, g) bind(C, name="aerort_get_aop_scalar")
      import :: c_int, c_float, c_ptr
      type(c_ptr), value :: mie
      integer(c_int), value :: km, nobs, nch, nq
      real(c_float), intent(in) :: channels_nm(*), qm(*), rh(*)
      integer(c_int), intent(in) :: q_table(*), q_bin(*)
      real(c_float), intent(out) :: tau(*), ssa(*), g(*)
    end function

    integer(c_int) function aerort_mie_table_interp(nlam, lambda_table, nrh, rh_table, nbin, nmom_table, npol, &
        bext_table, bsca_table, g_table, pmom_table, nch, channels_m, nmom, rh, bext, bsca, g, pmom, nout)     &
        bind(C, name="aerort_mie_table_interp")
      import :: c_int, c_double, c_float
      integer(c_int), value :: nlam, nrh, nbin, nmom_table, npol, nch, nmom
      real(c_double), intent(in) :: lambda_table(*), rh_table(*), bext_table(*), bsca_table(*), g_table(*)
      real(c_double), intent(in) :: pmom_table(*)
      real(c_float), intent(in)  :: channels_m(*)
      real(c_float), intent(out) :: rh(*), bext(*), bsca(*), g(*), pmom(*)
      integer(c_int), intent(out) :: nout
    end function

    type(c_ptr) function aerort_last_error() bind(C, name="aerort_last_error")
      import :: c_ptr
    end function
  end interface

contains

  ! Drop-in for VLIDORT_Scalar_Lambert (geo_vlidort/VLIDORT_LAMBERT.F90:34-168)
  subroutine VLIDORT_Scalar_Lambert_GPU(km, nch, nobs, channels, nstreams, plane_parallel, nMom, nPol, ROT, depol, &
      tau, ssa, g, pmom, pe, he, te, albedo, solar_zenith, relat_azymuth, sensor_zenith, MISSING, verbose,        &
      radiance_VL, reflectance_VL, rc)
    integer, intent(in) :: km, nch, nobs, nstreams, nMom, nPol, verbose
    logical, intent(in) :: plane_parallel
    real*8, intent(in)  :: channels(nch), ROT(km,nobs,nch), depol(nch), tau(km,nch,nobs), ssa(km,nch,nobs)
    real*8, intent(in)  :: g(km,nch,nobs), pmom(km,nch,nobs,nMom,nPol), pe(km+1,nobs), he(km+1,nobs)
    real*8, intent(in)  :: te(km+1,nobs), albedo(nobs,nch), solar_zenith(nobs), relat_azymuth(nobs)
    real*8, intent(in)  :: sensor_zenith(nobs), MISSING
    real*8, intent(out) :: radiance_VL(nobs,nch), reflectance_VL(nobs,nch)
    integer, intent(out) :: rc
    rc = aerort_vlidort_scalar_lambert(km, nch, nobs, channels, nstreams, merge(1, 0, plane_parallel), nMom, nPol, &
         ROT, depol, tau, ssa, g, pmom, pe, he, te, albedo, solar_zenith, relat_azymuth, sensor_zenith, MISSING,   &
         verbose, radiance_VL, reflectance_VL)
  end subroutine

  ! Drop-in for VLIDORT_Vector_Lambert_SingleGeom (geo_vlidort/VLIDORT_LAMBERT.F90:172-342), NSTOKES = 3,
  ! without the optional DO_2OS_CORRECTION / DO_BOA arguments (both off at the
  ! geo_vlidort.F90:612-619 call site)
  subroutine VLIDORT_Vector_Lambert_GPU(km, nch, nobs, channels, nstreams, plane_parallel, nMom, nPol, ROT, depol, &
      alpha, tau, ssa, pmom, pe, he, te, albedo, solar_zenith, relat_azymuth, sensor_zenith, flux_factor, MISSING,   &
      verbose, radiance_VL, reflectance_VL, Q, U, rc)
    integer, intent(in) :: km, nch, nobs, nstreams, nMom, nPol, verbose
    logical, intent(in) :: plane_parallel
    real*8, intent(in)  :: channels(nch), ROT(km,nobs,nch), depol(nch), alpha(km,nobs,nch), tau(km,nch,nobs)
    real*8, intent(in)  :: ssa(km,nch,nobs), pmom(km,nch,nobs,nMom,nPol), pe(km+1,nobs), he(km+1,nobs)
    real*8, intent(in)  :: te(km+1,nobs), albedo(nobs,nch), solar_zenith(nobs), relat_azymuth(nobs)
    real*8, intent(in)  :: sensor_zenith(nobs), flux_factor(nch,nobs), MISSING
    real*8, intent(out) :: radiance_VL(nobs,nch), reflectance_VL(nobs,nch), Q(nobs,nch), U(nobs,nch)
    integer, intent(out) :: rc
    rc = aerort_vlidort_vector_lambert(km, nch, nobs, channels, nstreams, merge(1, 0, plane_parallel), nMom, nPol, &
         ROT, depol, alpha, tau, ssa, pmom, pe, he, te, albedo, solar_zenith, relat_azymuth, sensor_zenith,         &
         flux_factor, MISSING, verbose, radiance_VL, reflectance_VL, Q, U)
  end subroutine

  ! Drop-in for VLIDORT_Scalar_LandMODIS (geo_vlidort/VLIDORT_BRDF_MODIS.F90:34-200),
  ! MODIS RTLS BRDF surface: kernel_wt = (fiso, fgeo, fvol), param = Li-sparse (h/b, b/r)
  subroutine VLIDORT_Scalar_LandMODIS_GPU(km, nch, nobs, channels, nstreams, plane_parallel, nMom, nPol, ROT, depol, &
      tau, ssa, g, pmom, pe, he, te, kernel_wt, param, solar_zenith, relat_azymuth, sensor_zenith, MISSING, verbose, &
      radiance_VL_SURF, reflectance_VL_SURF, BR, rc)
    integer, intent(in) :: km, nch, nobs, nstreams, nMom, nPol, verbose
    logical, intent(in) :: plane_parallel
    real*8, intent(in)  :: channels(nch), ROT(km,nobs,nch), depol(nch), tau(km,nch,nobs), ssa(km,nch,nobs)
    real*8, intent(in)  :: g(km,nch,nobs), pmom(km,nch,nobs,nMom,nPol), pe(km+1,nobs), he(km+1,nobs)
    real*8, intent(in)  :: te(km+1,nobs), kernel_wt(3,nch,nobs), param(2,nch,nobs), solar_zenith(nobs)
    real*8, intent(in)  :: relat_azymuth(nobs), sensor_zenith(nobs), MISSING
    real*8, intent(out) :: radiance_VL_SURF(nobs,nch), reflectance_VL_SURF(nobs,nch), BR(nobs,nch)
    integer, intent(out) :: rc
    rc = aerort_vlidort_scalar_landmodis(km, nch, nobs, channels, nstreams, merge(1, 0, plane_parallel), nMom, nPol, &
         ROT, depol, tau, ssa, g, pmom, pe, he, te, kernel_wt, param, solar_zenith, relat_azymuth, sensor_zenith,    &
         MISSING, verbose, radiance_VL_SURF, reflectance_VL_SURF, BR)
  end subroutine

  ! Drop-in for VLIDORT_Scalar_CX (geo_vlidort/VLIDORT_BRDF_CX.F90:420-584),
  ! Cox-Munk ocean glint: 10 m winds U10m, V10m (nobs), refractive index mr (nch)
  subroutine VLIDORT_Scalar_CX_GPU(km, nch, nobs, channels, nstreams, plane_parallel, nMom, nPol, ROT, depol, &
      tau, ssa, g, pmom, pe, he, te, U10m, V10m, mr, solar_zenith, relat_azymuth, sensor_zenith, MISSING,     &
      verbose, radiance_VL_SURF, reflectance_VL_SURF, BRDF, rc)
    integer, intent(in) :: km, nch, nobs, nstreams, nMom, nPol, verbose
    logical, intent(in) :: plane_parallel
    real*8, intent(in)  :: channels(nch), ROT(km,nobs,nch), depol(nch), tau(km,nch,nobs), ssa(km,nch,nobs)
    real*8, intent(in)  :: g(km,nch,nobs), pmom(km,nch,nobs,nMom,nPol), pe(km+1,nobs), he(km+1,nobs)
    real*8, intent(in)  :: te(km+1,nobs), U10m(nobs), V10m(nobs), mr(nch), solar_zenith(nobs)
    real*8, intent(in)  :: relat_azymuth(nobs), sensor_zenith(nobs), MISSING
    real*8, intent(out) :: radiance_VL_SURF(nobs,nch), reflectance_VL_SURF(nobs,nch), BRDF(1,nobs,nch)
    integer, intent(out) :: rc
    rc = aerort_vlidort_scalar_cx(km, nch, nobs, channels, nstreams, merge(1, 0, plane_parallel), nMom, nPol, &
         ROT, depol, tau, ssa, g, pmom, pe, he, te, U10m, V10m, mr, solar_zenith, relat_azymuth, sensor_zenith,  &
         MISSING, verbose, radiance_VL_SURF, reflectance_VL_SURF, BRDF)
  end subroutine

  ! Drop-in for VLIDORT_Scalar_GissCX (geo_vlidort/VLIDORT_BRDF_CX.F90:1553-1716),
  ! GISS Cox-Munk ocean glint, the call of geo_vlidort_ocean.F90:536
  subroutine VLIDORT_Scalar_GissCX_GPU(km, nch, nobs, channels, nstreams, plane_parallel, nMom, nPol, ROT, depol, &
      tau, ssa, g, pmom, pe, he, te, U10m, V10m, mr, solar_zenith, relat_azymuth, sensor_zenith, MISSING,         &
      verbose, radiance_VL_SURF, reflectance_VL_SURF, BRDF, rc)
    integer, intent(in) :: km, nch, nobs, nstreams, nMom, nPol, verbose
    logical, intent(in) :: plane_parallel
    real*8, intent(in)  :: channels(nch), ROT(km,nobs,nch), depol(nch), tau(km,nch,nobs), ssa(km,nch,nobs)
    real*8, intent(in)  :: g(km,nch,nobs), pmom(km,nch,nobs,nMom,nPol), pe(km+1,nobs), he(km+1,nobs)
    real*8, intent(in)  :: te(km+1,nobs), U10m(nobs), V10m(nobs), mr(nch), solar_zenith(nobs)
    real*8, intent(in)  :: relat_azymuth(nobs), sensor_zenith(nobs), MISSING
    real*8, intent(out) :: radiance_VL_SURF(nobs,nch), reflectance_VL_SURF(nobs,nch), BRDF(1,nobs,nch)
    integer, intent(out) :: rc
    rc = aerort_vlidort_scalar_gisscx(km, nch, nobs, channels, nstreams, merge(1, 0, plane_parallel), nMom, nPol, &
         ROT, depol, tau, ssa, g, pmom, pe, he, te, U10m, V10m, mr, solar_zenith, relat_azymuth, sensor_zenith,      &
         MISSING, verbose, radiance_VL_SURF, reflectance_VL_SURF, BRDF)
  end subroutine

  ! Drop-in for VLIDORT_ROT_CALC (geo_vlidort/VLIDORT_ROT.F90:19-86)
  subroutine VLIDORT_ROT_CALC_GPU(km, nch, nobs, channels, pe, he, te, MISSING, verbose, ROT, depol, rc)
    integer, intent(in) :: km, nch, nobs, verbose
    real*8, intent(in)  :: channels(nch), pe(km+1,nobs), he(km+1,nobs), te(km+1,nobs), MISSING
    real*8, intent(out) :: ROT(km,nobs,nch), depol(nch)
    integer, intent(out) :: rc
    rc = aerort_vlidort_rot_calc(km, nch, nobs, channels, pe, he, te, MISSING, verbose, ROT, depol)
  end subroutine

  ! Drop-in for getEdgeVars (Chem_Base/MieObs_py.F90:27-83)
  subroutine getEdgeVars_GPU(km, nobs, airdens, delp, ptop, pe, ze, te, rc)
    integer, intent(in) :: km, nobs
    real, intent(in)    :: airdens(km,nobs), delp(km,nobs), ptop
    real, intent(out)   :: pe(km+1,nobs), ze(km+1,nobs), te(km+1,nobs)
    integer, intent(out) :: rc
    rc = aerort_get_edge_vars(km, nobs, airdens, delp, ptop, pe, ze, te)
  end subroutine

  ! The message of the calling thread's last nonzero rc
  function aerort_last_error_string() result(msg)
    character(len=:), allocatable :: msg
    character(kind=c_char), pointer :: p(:)
    type(c_ptr) :: cp
    integer :: n
    cp = aerort_last_error()
    call c_f_pointer(cp, p, [4096])
    n = 0
    do while (n < 4096)
      if (p(n + 1) == c_null_char) exit
      n = n + 1
    end do
    allocate(character(len=n) :: msg)
    msg = transfer(p(1:n), msg)
  end function
end module aerort_mod
