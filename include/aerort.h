/* aerort: GB300-native aerosol optics + scalar VLIDORT-style radiative transfer.
 *
 * C ABI of the drop-in replacement for AeroApps' per-column hot path.  Every
 * entry point takes plain pointers and sizes, Fortran column-major arrays with
 * exactly the shapes of the reference routine it replaces, and returns the
 * reference's integer rc.  Reference paths are relative to the AeroApps tree.
 *
 * Host-pointer entry points copy inputs to the GPU, run, and copy results
 * back (a drop-in for the Fortran/f2py caller).  The *_dev variants take
 * device pointers and a cudaStream_t (passed as void*) and never synchronise
 * the host; they are the building blocks of batched/fused pipelines.
 */
#ifndef AERORT_H
#define AERORT_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* rc values shared with the reference */
#define AERORT_OK 0
#define AERORT_RC_NSTREAMS 2       /* VLIDORT_Mod.F90:366  NSTREAMS > MAXSTREAMS (25)  */
#define AERORT_RC_NLAYERS 3        /* VLIDORT_Mod.F90:367  NLAYERS  > MAXLAYERS  (72)  */
#define AERORT_RC_NMOMENTS 5       /* VLIDORT_ScatMod.F90:1050  nmom > MAXMOMENTS_INPUT */
#define AERORT_RC_CHANNEL 99       /* VLIDORT_MieMod.F90:219-224 channel not in the Mie table */
#define AERORT_RC_MOMENTS 666      /* VLIDORT_MieMod.F90:237-241 table has too few moments */
#define AERORT_RC_NPOL 777         /* VLIDORT_MieMod.F90:243-255 inconsistent nPol */
/* rc values of this library (not produced by the reference) */
#define AERORT_RC_CUDA 1001        /* CUDA runtime error (message via aerort_last_error) */
#define AERORT_RC_ARG 1002         /* invalid argument (null pointer, non-positive size) */
#define AERORT_RC_UNSUPPORTED 1003 /* configuration not built (e.g. nstreams not in {4,6,8,12,16}) */

/* working precision of the RT solve */
#define AERORT_PREC_FP64 0         /* plain method: FP64 throughout (parity 1e-9 with the reference)            */
#define AERORT_PREC_MIXED 1        /* mixed method: FP64 set-up and single scatter, FP32 Fourier series (1e-4)  */

/* per-pixel status written by the *_ex / *_dev RT entry points */
#define AERORT_ST_OK 0
#define AERORT_ST_EIGEN 1          /* layer eigenproblem failed (reference: ASYMTX error, rc 4)   */
#define AERORT_ST_BVP 2            /* singular boundary-value system (reference: DGBTRF info > 0) */
#define AERORT_ST_INPUT 3          /* non-positive extinction / scattering optical depth          */

/* ------------------------------------------------------------------------------------------
 * Mie tables (Chem_Mie object).
 * Replaces Chem_MieCreate / Chem_MieTableRead (Chem_Base/Chem_MieMod.F90:124-411,
 * Chem_MieTableMod.F90:238-719) once the tables are in memory: uploads the
 * per-species tables, already on the requested channels, and builds the RH map
 * (Chem_MieTableMod.F90:612-627).  Arrays are REAL*4, Fortran order:
 *   rh(nrh); bext,bsca,g (nrh,nch,nbin); pmom (nrh,nch,nbin,nmom,npol).
 * channels_m(nch): table wavelengths in metres (as Chem_Mie%channels).
 */
typedef struct aerort_mie aerort_mie;

typedef struct {
  int nrh, nbin, nmom, npol;
  const float* rh;
  const float* bext;
  const float* bsca;
  const float* g;
  const float* pmom;
} aerort_mie_table_desc;

int aerort_mie_create(int ntables, const aerort_mie_table_desc* tables, int nch, const float* channels_m,
                      aerort_mie** out);
int aerort_mie_destroy(aerort_mie* mie);

/* Chem_MieTableRead after the netCDF read (Chem_MieTableMod.F90:557-627):
 * brings one species table from its file wavelengths to the requested
 * channels with the reference's polint (:671-717) — linear in wavelength,
 * REAL*8 in, REAL*4 slope/offset/result; below the first table wavelength it
 * extrapolates the first segment, above the last it holds the last value —
 * and converts the RH grid to REAL*4.  Host code; no GPU needed.
 * Inputs in file (Fortran) order, wavelength fastest:
 *   lambda_table(nlam) [m], rh_table(nrh), bext/bsca/g_table(nlam,nrh,nbin),
 *   pmom_table(nlam,nrh,nbin,nmom_table,npol) (may be NULL when nmom = 0).
 * Outputs in the aerort_mie_table_desc order:
 *   rh(nrh), bext/bsca/g(nrh,nch,nbin), pmom(nrh,nch,nbin,nmom,npol) (the
 *   first nmom moments).
 * channels_m(nch) [m] as Chem_Mie%channels.  nout (optional) receives the
 * number of channels outside the table's wavelength range (the reference
 * prints a warning for each interpolation there).
 * rc: 0; 99 when nmom > nmom_table (Chem_MieTableMod.F90:331-335);
 * AERORT_RC_ARG for bad sizes, NULL pointers or NaN wavelengths. */
int aerort_mie_table_interp(int nlam, const double* lambda_table, int nrh, const double* rh_table, int nbin,
                            int nmom_table, int npol, const double* bext_table, const double* bsca_table,
                            const double* g_table, const double* pmom_table, int nch, const float* channels_m,
                            int nmom, float* rh, float* bext, float* bsca, float* g, float* pmom, int* nout);

/* VLIDORT_getAOPvector (geo_vlidort/VLIDORT_MieMod.F90:124-336) with
 * Chem_MieQuery (Chem_MieMod.F90:789-965) for every tracer.  The tracer names
 * vname(nq,16) of the reference are resolved by the caller (Chem_MieQueryIdx,
 * Chem_MieMod.F90:720-777) into q_table(nq) (species table index, -1 = tracer
 * without optics, skipped like the reference's idxTable == -1) and q_bin(nq)
 * (0-based size bin).  Shapes: channels_nm(nch) [nm], qm(km,nq,nobs),
 * rh(km,nobs), tau/ssa/g(km,nch,nobs), pmom(km,nch,nobs,nMom,nPol).  FP32,
 * bit-identical to the reference arithmetic. */
int aerort_get_aop_vector(aerort_mie* mie, int km, int nobs, int nch, int nq, const float* channels_nm,
                          const int* q_table, const int* q_bin, const float* qm, const float* rh, int nMom,
                          int nPol, float* tau, float* ssa, float* g, float* pmom);
int aerort_get_aop_vector_dev(aerort_mie* mie, int km, int nobs, int nch, int nq, const float* channels_nm_host,
                              const int* q_table_host, const int* q_bin_host, const float* qm_dev,
                              const float* rh_dev, int nMom, int nPol, float* tau_dev, float* ssa_dev,
                              float* g_dev, float* pmom_dev, void* stream);

/* VLIDORT_getAOPscalar (geo_vlidort/VLIDORT_MieMod.F90:10-120): tau, ssa, g
 * (km,nch,nobs) without phase-function moments; otherwise as
 * aerort_get_aop_vector (rc 0 or 99). */
int aerort_get_aop_scalar(aerort_mie* mie, int km, int nobs, int nch, int nq, const float* channels_nm,
                          const int* q_table, const int* q_bin, const float* qm, const float* rh, float* tau,
                          float* ssa, float* g);
int aerort_get_aop_scalar_dev(aerort_mie* mie, int km, int nobs, int nch, int nq, const float* channels_nm_host,
                              const int* q_table_host, const int* q_bin_host, const float* qm_dev,
                              const float* rh_dev, float* tau_dev, float* ssa_dev, float* g_dev, void* stream);

/* ------------------------------------------------------------------------------------------
 * VLIDORT_Scalar_Lambert (geo_vlidort/VLIDORT_LAMBERT.F90:34-168): scalar TOA
 * radiance and reflectance for nobs pixels x nch channels, observation
 * geometry, Lambertian surface, with the VLIDORT_Init settings of
 * VLIDORT2p8p3/VLIDORT_Mod.F90:65-383 (FO outgoing correction, delta-M,
 * pseudo-spherical, double convergence test at accuracy 1e-4) and the layer
 * mixing of VLIDORT_Run_Scalar (VLIDORT_ScatMod.F90:975-1247).
 * Shapes: channels(nch) [nm], ROT(km,nobs,nch), depol(nch), tau/ssa/g(km,nch,nobs),
 * pmom(km,nch,nobs,nMom,nPol), pe/he/te(km+1,nobs) [Pa, m, K], albedo(nobs,nch),
 * solar_zenith/relat_azymuth/sensor_zenith(nobs) [deg], radiance_VL/reflectance_VL(nobs,nch).
 * Pixels whose angles or albedo are MISSING (|x/MISSING-1| < 1e-3), or whose
 * solve fails, get MISSING, as in the reference.  FP64.  nstreams must be one
 * of 4, 6, 8, 12, 16 (the compiled stream counts).  Every RT entry point
 * rejects nobs * nch above 2,130,706,432 solves with AERORT_RC_ARG. */
int aerort_vlidort_scalar_lambert(int km, int nch, int nobs, const double* channels, int nstreams,
                                  int plane_parallel, int nMom, int nPol, const double* ROT, const double* depol,
                                  const double* tau, const double* ssa, const double* g, const double* pmom,
                                  const double* pe, const double* he, const double* te, const double* albedo,
                                  const double* solar_zenith, const double* relat_azymuth,
                                  const double* sensor_zenith, double MISSING, int verbose, double* radiance_VL,
                                  double* reflectance_VL);

/* Same, plus per-pixel diagnostics: nfourier(nobs,nch) = last Fourier term
 * summed, status(nobs,nch) = AERORT_ST_* (either may be NULL). */
int aerort_vlidort_scalar_lambert_ex(int km, int nch, int nobs, const double* channels, int nstreams,
                                     int plane_parallel, int nMom, int nPol, const double* ROT,
                                     const double* depol, const double* tau, const double* ssa, const double* g,
                                     const double* pmom, const double* pe, const double* he, const double* te,
                                     const double* albedo, const double* solar_zenith,
                                     const double* relat_azymuth, const double* sensor_zenith, double MISSING,
                                     int verbose, double* radiance_VL, double* reflectance_VL, int* nfourier,
                                     int* status);

/* Device-pointer form of aerort_vlidort_scalar_lambert_ex (all array arguments
 * are device pointers, channels/pe/te unused).  Enqueued on `stream`. */
int aerort_vlidort_scalar_lambert_dev(int km, int nch, int nobs, int nstreams, int plane_parallel, int nMom,
                                      const double* ROT, const double* depol, const double* tau,
                                      const double* ssa, const double* pmom, const double* he,
                                      const double* albedo, const double* solar_zenith,
                                      const double* relat_azymuth, const double* sensor_zenith, double MISSING,
                                      double* radiance_VL, double* reflectance_VL, int* nfourier, int* status,
                                      void* stream);

/* Batched device form for mixed column shapes (one launch per stream count):
 * nlay(nobs) (device, may be NULL = all km) gives the layer count of each
 * column, which uses the first nlay entries of its km-dimensioned arrays
 * (layer 1 = top); the optics may be given as FP32 device arrays straight
 * from aerort_get_aop_vector_dev (tau_f, ssa_f, pmom_f; pass NULL for the FP64
 * tau, ssa, pmom), in which case the FP64 conversion the reference driver does
 * (dble(), geo_vlidort.F90:598-601) happens on load.  No counterpart routine in
 * the reference: it batches many VLIDORT_Scalar_Lambert calls into one launch.
 * Calls on different streams use different library scratch (one pad per
 * stream, up to 16 streams at once), so groups of different stream counts may
 * be enqueued on separate streams and run concurrently.  The calls may be
 * captured into a CUDA graph once an eager call of the same size on the same
 * stream has sized the scratch (no allocation is allowed during capture); a
 * pad used by captured work then stays with its stream for good, so graph
 * replays never share scratch with other streams. */
int aerort_vlidort_scalar_lambert_batch_dev(int km, int nch, int nobs, int nstreams, int plane_parallel, int nMom,
                                            const int* nlay, const double* ROT, const double* depol,
                                            const double* tau, const double* ssa, const double* pmom,
                                            const float* tau_f, const float* ssa_f, const float* pmom_f,
                                            const double* he, const double* albedo, const double* solar_zenith,
                                            const double* relat_azymuth, const double* sensor_zenith, double MISSING,
                                            double* radiance_VL, double* reflectance_VL, int* nfourier, int* status,
                                            void* stream);

/* Mixed-precision forms of the two batched calls (same arguments).  No
 * counterpart in the reference.  The per-column set-up (layer mixing, delta-M,
 * Chapman factors, first-order single scatter) stays FP64; the Fourier series
 * runs in FP32 with formulations chosen for FP32: the layer eigenproblem by
 * one-sided Jacobi on a graded factor (k to relative accuracy), the
 * conservative mode of Fourier term 0 split off exactly, and the
 * Green's-function multipliers as divided differences of exp(-x tau).
 * A radiance whose Fourier sum cancels (sum of |terms| > 10 |radiance|, e.g.
 * unconverged series near backscatter) would inherit the FP32 term error
 * amplified; such solves are listed on the device and re-solved in FP64 by a
 * second launch on the same stream.  Radiance error against the FP64 method:
 * <= 1e-5 on the synthetic configs, <= 1e-4 with layer SSA in [0.999, 1). */
int aerort_vlidort_scalar_lambert_mixed_batch_dev(int km, int nch, int nobs, int nstreams, int plane_parallel,
                                                  int nMom, const int* nlay, const double* ROT, const double* depol,
                                                  const double* tau, const double* ssa, const double* pmom,
                                                  const float* tau_f, const float* ssa_f, const float* pmom_f,
                                                  const double* he, const double* albedo, const double* solar_zenith,
                                                  const double* relat_azymuth, const double* sensor_zenith,
                                                  double MISSING, double* radiance_VL, double* reflectance_VL,
                                                  int* nfourier, int* status, void* stream);
int aerort_vlidort_scalar_lambert_mixed_batch(int km, int nch, int nobs, int nstreams, int plane_parallel, int nMom,
                                              const int* nlay, const double* ROT, const double* depol,
                                              const double* tau, const double* ssa, const double* pmom,
                                              const double* he, const double* albedo, const double* solar_zenith,
                                              const double* relat_azymuth, const double* sensor_zenith,
                                              double MISSING, double* radiance_VL, double* reflectance_VL,
                                              int* nfourier, int* status);

/* VLIDORT_Vector_Lambert (geo_vlidort/VLIDORT_LAMBERT.F90:172-342, single
 * geometry per pixel; f2py VECTOR_LAMBERT, leo_vlidort/VLIDORT_POLAR_py.F90
 * :457-526): TOA radiance, reflectance and Stokes Q, U for nobs pixels x nch
 * channels with NSTOKES = 3, the VLIDORT_Init settings of the scalar call and
 * the 16-entry Greek-matrix mixing of VLIDORT_Run_Vector_SingleGeom
 * (VLIDORT_ScatMod.F90:284-617).  Same arguments as the reference:
 * alpha(km,nobs,nch) trace-gas absorption (may be NULL = 0),
 * pmom(km,nch,nobs,nMom,nPol) with nPol = 6 elements P11, P12, P33, P34, P22,
 * P44 (as aerort_get_aop_vector with nPol = 6 writes them), flux_factor(nch,nobs)
 * solar flux F0 (reflectance = pi I / (cos(sza) F0), single-precision pi),
 * radiance_VL, reflectance_VL, Q, U (nobs,nch).  A pixel with MISSING angles
 * or albedo, or whose solve fails, gets MISSING in all four outputs (the
 * reference writes Q, U of a missing-angle pixel only at a stale channel
 * index).  FP64 with a real eigen-decomposition per layer (the reference's
 * real eigensolver mask is always set for NSTOKES = 3); nstreams one of 4, 6,
 * 8, 12, 16.  rc: 0; 2, 3, 5 as the scalar call; AERORT_RC_ARG for nPol != 6. */
int aerort_vlidort_vector_lambert(int km, int nch, int nobs, const double* channels, int nstreams,
                                  int plane_parallel, int nMom, int nPol, const double* ROT, const double* depol,
                                  const double* alpha, const double* tau, const double* ssa, const double* pmom,
                                  const double* pe, const double* he, const double* te, const double* albedo,
                                  const double* solar_zenith, const double* relat_azymuth,
                                  const double* sensor_zenith, const double* flux_factor, double MISSING,
                                  int verbose, double* radiance_VL, double* reflectance_VL, double* Q, double* U);
/* Same, plus nfourier(nobs,nch) (last Fourier term) and status(nobs,nch)
 * (AERORT_ST_*); either may be NULL. */
int aerort_vlidort_vector_lambert_ex(int km, int nch, int nobs, const double* channels, int nstreams,
                                     int plane_parallel, int nMom, int nPol, const double* ROT, const double* depol,
                                     const double* alpha, const double* tau, const double* ssa, const double* pmom,
                                     const double* pe, const double* he, const double* te, const double* albedo,
                                     const double* solar_zenith, const double* relat_azymuth,
                                     const double* sensor_zenith, const double* flux_factor, double MISSING,
                                     int verbose, double* radiance_VL, double* reflectance_VL, double* Q, double* U,
                                     int* nfourier, int* status);
/* Batched device form (no counterpart routine in the reference): every array
 * a device pointer, nlay(nobs) per-column layer counts (may be NULL), optics
 * either FP64 (tau, ssa, pmom) or FP32 straight from aerort_get_aop_vector_dev
 * with nPol = 6 (tau_f, ssa_f, pmom_f), flux_factor may be NULL (1).  Enqueued
 * on `stream` with the library's scratch pad of that stream. */
int aerort_vlidort_vector_lambert_batch_dev(int km, int nch, int nobs, int nstreams, int plane_parallel, int nMom,
                                            const int* nlay, const double* ROT, const double* depol,
                                            const double* alpha, const double* tau, const double* ssa,
                                            const double* pmom, const float* tau_f, const float* ssa_f,
                                            const float* pmom_f, const double* he, const double* albedo,
                                            const double* solar_zenith, const double* relat_azymuth,
                                            const double* sensor_zenith, const double* flux_factor, double MISSING,
                                            double* radiance_VL, double* reflectance_VL, double* Q, double* U,
                                            int* nfourier, int* status, void* stream);

/* VLIDORT_Scalar_LandMODIS (geo_vlidort/VLIDORT_BRDF_MODIS.F90:34-200): the
 * scalar solve of aerort_vlidort_scalar_lambert over the MODIS RTLS BRDF of
 * VLIDORT_LANDMODIS_SingleGeom (RTSI/VLIDORT2p8p3/VLIDORT_SurfaceMod.F90
 * :1376-1596) -- Lambertian, Ross-thick and Li-sparse kernels with amplitudes
 * kernel_wt(3, nch, nobs) = (fiso, fgeo, fvol) and Li-sparse parameters
 * param(2, nch, nobs) = (h/b, b/r), 50 azimuth streams -- in place of the
 * albedo; same argument list as the reference (BR(nobs, nch): the exact
 * direct-bounce BRDF of each pixel and channel).  A pixel with MISSING angles
 * gets MISSING radiance, reflectance and BR; a negative BR gives -500 in all
 * three and no solve (as the reference).  The reference's MISSING checks of
 * kernel_wt and param never skip a pixel (their CYCLE ends only their own
 * loop), so none is made here either.  FP64; at most 256 distinct param pairs
 * per call (AERORT_RC_ARG beyond).  rc as aerort_vlidort_scalar_lambert. */
int aerort_vlidort_scalar_landmodis(int km, int nch, int nobs, const double* channels, int nstreams,
                                    int plane_parallel, int nMom, int nPol, const double* ROT, const double* depol,
                                    const double* tau, const double* ssa, const double* g, const double* pmom,
                                    const double* pe, const double* he, const double* te, const double* kernel_wt,
                                    const double* param, const double* solar_zenith, const double* relat_azymuth,
                                    const double* sensor_zenith, double MISSING, int verbose,
                                    double* radiance_VL_SURF, double* reflectance_VL_SURF, double* BR);
/* Same, plus nfourier(nobs,nch) and status(nobs,nch) (either may be NULL). */
int aerort_vlidort_scalar_landmodis_ex(int km, int nch, int nobs, const double* channels, int nstreams,
                                       int plane_parallel, int nMom, int nPol, const double* ROT, const double* depol,
                                       const double* tau, const double* ssa, const double* g, const double* pmom,
                                       const double* pe, const double* he, const double* te, const double* kernel_wt,
                                       const double* param, const double* solar_zenith, const double* relat_azymuth,
                                       const double* sensor_zenith, double MISSING, int verbose,
                                       double* radiance_VL_SURF, double* reflectance_VL_SURF, double* BR,
                                       int* nfourier, int* status);
/* Batched device form (no counterpart routine in the reference): arrays on
 * the device as aerort_vlidort_scalar_lambert_batch_dev (nlay and FP32
 * optics optional), kernel_wt(3, nch, nobs) on the device, param_host(2, nch,
 * nobs) on the HOST (the launch builds one Fourier table per distinct pair),
 * BR(nobs, nch) out on the device.  Enqueued on `stream`; the table upload
 * is a pageable-memory copy, so this call does not belong in a stream capture. */
int aerort_vlidort_scalar_landmodis_batch_dev(int km, int nch, int nobs, int nstreams, int plane_parallel, int nMom,
                                              const int* nlay, const double* ROT, const double* depol,
                                              const double* tau, const double* ssa, const double* pmom,
                                              const float* tau_f, const float* ssa_f, const float* pmom_f,
                                              const double* he, const double* kernel_wt, const double* param_host,
                                              const double* solar_zenith, const double* relat_azymuth,
                                              const double* sensor_zenith, double MISSING, double* radiance_VL_SURF,
                                              double* reflectance_VL_SURF, double* BR, int* nfourier, int* status,
                                              void* stream);

/* VLIDORT_Scalar_CX (geo_vlidort/VLIDORT_BRDF_CX.F90:420-584): the scalar
 * solve of aerort_vlidort_scalar_lambert over the Cox-Munk ocean glint of
 * VLIDORT_CoxMunk_SingleGeom (RTSI/VLIDORT2p8p3/VLIDORT_SurfaceMod.F90
 * :816-1042) -- one Cox-Munk kernel with shadowing, slope variance
 * 0.003 + 0.00512 W from the wind speed W = |(U10m, V10m)| clamped to
 * [0, 50] m/s, refractive index squared mr(ch)^2, 100 azimuth streams -- in
 * place of the albedo; same argument list as the reference (BRDF(nobs, nch):
 * the exact direct-bounce BRDF of each pixel and channel).  A pixel with
 * MISSING angles, or a channel with a MISSING wind component or refractive
 * index, gets MISSING radiance and reflectance (and BRDF, which the reference
 * leaves unset there).  FP64.  rc as aerort_vlidort_scalar_lambert. */
int aerort_vlidort_scalar_cx(int km, int nch, int nobs, const double* channels, int nstreams, int plane_parallel,
                             int nMom, int nPol, const double* ROT, const double* depol, const double* tau,
                             const double* ssa, const double* g, const double* pmom, const double* pe,
                             const double* he, const double* te, const double* U10m, const double* V10m,
                             const double* mr, const double* solar_zenith, const double* relat_azymuth,
                             const double* sensor_zenith, double MISSING, int verbose, double* radiance_VL_SURF,
                             double* reflectance_VL_SURF, double* BRDF);
/* Same, plus nfourier(nobs,nch) and status(nobs,nch) (either may be NULL). */
int aerort_vlidort_scalar_cx_ex(int km, int nch, int nobs, const double* channels, int nstreams, int plane_parallel,
                                int nMom, int nPol, const double* ROT, const double* depol, const double* tau,
                                const double* ssa, const double* g, const double* pmom, const double* pe,
                                const double* he, const double* te, const double* U10m, const double* V10m,
                                const double* mr, const double* solar_zenith, const double* relat_azymuth,
                                const double* sensor_zenith, double MISSING, int verbose, double* radiance_VL_SURF,
                                double* reflectance_VL_SURF, double* BRDF, int* nfourier, int* status);
/* Batched device form (no counterpart routine in the reference): arrays on
 * the device as aerort_vlidort_scalar_lambert_batch_dev (nlay and FP32
 * optics optional), U10m, V10m (nobs) and mr (nch) on the device, BRDF(nobs,
 * nch) out on the device.  Each solve's quadrature-to-quadrature Cox-Munk
 * components are formed on the device (they depend on its wind and
 * refractive index).  Enqueued on `stream`; an azimuth-weight table goes up
 * by a pageable-memory copy, so this call does not belong in a stream capture. */
int aerort_vlidort_scalar_cx_batch_dev(int km, int nch, int nobs, int nstreams, int plane_parallel, int nMom,
                                       const int* nlay, const double* ROT, const double* depol, const double* tau,
                                       const double* ssa, const double* pmom, const float* tau_f, const float* ssa_f,
                                       const float* pmom_f, const double* he, const double* U10m,
                                       const double* V10m, const double* mr, const double* solar_zenith,
                                       const double* relat_azymuth, const double* sensor_zenith, double MISSING,
                                       double* radiance_VL_SURF, double* reflectance_VL_SURF, double* BRDF,
                                       int* nfourier, int* status, void* stream);

/* VLIDORT_Scalar_GissCX (geo_vlidort/VLIDORT_BRDF_CX.F90:1553-1716), the
 * Cox-Munk call of the ocean driver (geo_vlidort_ocean.F90:536): the same
 * wrapper and arguments as aerort_vlidort_scalar_cx over the GISS Cox-Munk
 * kernel of VLIDORT_GissCoxMunk_SingleGeom (VLIDORT_SurfaceMod.F90:586-814):
 * kernel 10 with slope parameter sigma2 / 2 and refractive index mr(ch),
 * shadowing, 100 azimuth streams.  For a real refractive index its scalar
 * element is the Cox-Munk kernel's (to ~1e-13). */
int aerort_vlidort_scalar_gisscx(int km, int nch, int nobs, const double* channels, int nstreams,
                                 int plane_parallel, int nMom, int nPol, const double* ROT, const double* depol,
                                 const double* tau, const double* ssa, const double* g, const double* pmom,
                                 const double* pe, const double* he, const double* te, const double* U10m,
                                 const double* V10m, const double* mr, const double* solar_zenith,
                                 const double* relat_azymuth, const double* sensor_zenith, double MISSING,
                                 int verbose, double* radiance_VL_SURF, double* reflectance_VL_SURF, double* BRDF);
int aerort_vlidort_scalar_gisscx_ex(int km, int nch, int nobs, const double* channels, int nstreams,
                                    int plane_parallel, int nMom, int nPol, const double* ROT, const double* depol,
                                    const double* tau, const double* ssa, const double* g, const double* pmom,
                                    const double* pe, const double* he, const double* te, const double* U10m,
                                    const double* V10m, const double* mr, const double* solar_zenith,
                                    const double* relat_azymuth, const double* sensor_zenith, double MISSING,
                                    int verbose, double* radiance_VL_SURF, double* reflectance_VL_SURF, double* BRDF,
                                    int* nfourier, int* status);
int aerort_vlidort_scalar_gisscx_batch_dev(int km, int nch, int nobs, int nstreams, int plane_parallel, int nMom,
                                           const int* nlay, const double* ROT, const double* depol,
                                           const double* tau, const double* ssa, const double* pmom,
                                           const float* tau_f, const float* ssa_f, const float* pmom_f,
                                           const double* he, const double* U10m, const double* V10m,
                                           const double* mr, const double* solar_zenith, const double* relat_azymuth,
                                           const double* sensor_zenith, double MISSING, double* radiance_VL_SURF,
                                           double* reflectance_VL_SURF, double* BRDF, int* nfourier, int* status,
                                           void* stream);

/* Edge pressure pe (Pa), height above the surface ze (m) and temperature te
 * (K), each (km+1,nobs), from layer air density airdens (kg m-3) and pressure
 * thickness delp (Pa), each (km,nobs), and the top pressure ptop (Pa).
 * Replaces getEdgeVars (Chem_Base/MieObs_py.F90:27-83), same argument list
 * with rc as the return value.  FP32 like the reference: pe and ze
 * bit-identical, te within a few units in the last place (logf/powf).
 * rc: 0; AERORT_RC_ARG; AERORT_RC_NLAYERS when km > 532.  _dev: every array on
 * the device, enqueued on `stream`. */
int aerort_get_edge_vars(int km, int nobs, const float* airdens, const float* delp, float ptop, float* pe, float* ze,
                         float* te);
int aerort_get_edge_vars_dev(int km, int nobs, const float* airdens, const float* delp, float ptop, float* pe,
                             float* ze, float* te, void* stream);

/* Rayleigh optical thickness ROT(km,nobs,nch) and depolarisation ratio
 * depol(nch) from the edge profiles pe (Pa), he (m), te (K), each
 * (km+1,nobs), at channels(nch) nm.  Replaces VLIDORT_ROT_CALC
 * (geo_vlidort/VLIDORT_ROT.F90:19-86, with VLIDORT_Rayleigh / coef_depol /
 * F_air of RTSI/VLIDORT2p8p3/VLIDORT_ScatMod.F90:145-283), same argument list
 * with rc as the return value; bit-identical to the reference arithmetic.
 * MISSING and verbose are accepted for the drop-in and unused (the reference
 * calculator cannot fail).  _dev: every array on the device, enqueued on
 * `stream`. */
int aerort_vlidort_rot_calc(int km, int nch, int nobs, const double* channels, const double* pe, const double* he,
                            const double* te, double MISSING, int verbose, double* ROT, double* depol);
int aerort_vlidort_rot_calc_dev(int km, int nch, int nobs, const double* channels, const double* pe,
                                const double* he, const double* te, double* ROT, double* depol, void* stream);

/* Caller-owned RT workspace (device scratch for one launch at a time).  No
 * counterpart in the reference.  aerort_workspace_create allocates `bytes` of
 * device memory once; launches through aerort_vlidort_scalar_lambert_ws_dev
 * then allocate nothing, and launches on different workspaces may overlap on
 * different streams (the batched entry points above keep one library
 * scratch pad per stream, for up to 16 streams at once, and allocate it on
 * first use).  The grid is capped to the threads whose
 * scratch fits: bytes_per_thread(km, nstreams, precision) x threads; one
 * block (32-128 threads) must fit.  The precision argument selects
 * AERORT_PREC_FP64 or AERORT_PREC_MIXED; the other arguments are those of
 * aerort_vlidort_scalar_lambert_batch_dev. */
typedef struct aerort_workspace aerort_workspace;
int aerort_workspace_create(size_t bytes, aerort_workspace** ws);
int aerort_workspace_destroy(aerort_workspace* ws);
long aerort_workspace_bytes_per_thread(int km, int nstreams, int precision);
int aerort_vlidort_scalar_lambert_ws_dev(aerort_workspace* ws, int precision, int km, int nch, int nobs, int nstreams,
                                         int plane_parallel, int nMom, const int* nlay, const double* ROT,
                                         const double* depol, const double* tau, const double* ssa,
                                         const double* pmom, const float* tau_f, const float* ssa_f,
                                         const float* pmom_f, const double* he, const double* albedo,
                                         const double* solar_zenith, const double* relat_azymuth,
                                         const double* sensor_zenith, double MISSING, double* radiance_VL,
                                         double* reflectance_VL, int* nfourier, int* status, void* stream);

/* Number of solves that the last mixed call enqueued on `stream` through the
 * library's batched entry points re-solved in FP64; with stream = NULL, the
 * last mixed call on any stream (this is how to ask after the host-pointer
 * entry points, which run on the library's own stream).  Synchronises the
 * stream of that call.  No counterpart in the reference. */
int aerort_refined_count(void* stream, int* count);

/* Launch schedule of the RT kernel per (stream count, precision): threads per
 * block (32, 64, 96 or 128) and resident blocks per SM (0 = occupancy limit).
 * Set by the autotuner (aeroapps_gb300/autotune.py); no counterpart in the
 * reference. */
int aerort_set_schedule(int nstreams, int precision, int threads_per_block, int blocks_per_sm);
int aerort_get_schedule(int nstreams, int precision, int* threads_per_block, int* blocks_per_sm);

/* RT kernel per (stream count, precision): AERORT_KERNEL_THREAD runs each
 * solve on one thread; AERORT_KERNEL_TEAM runs the set-up thread per solve and
 * the Fourier series on a whole warp per solve with the layer matrices in
 * shared memory (the better choice where the per-solve working set is large).
 * AERORT_KERNEL_AUTO (the default) takes the thread kernel only where it was
 * measured faster on GB300: FP64 at 4, 6 and 8 streams and mixed at 4 and 8
 * streams, for batches that give every SM 2-4 warps of 32 solves or more;
 * otherwise the team kernel.  The FP64 re-solve of a mixed launch's refinement list always runs
 * on the team kernel.  Results agree to round-off.  aerort_get_kernel returns
 * the setting, or a negative rc. */
#define AERORT_KERNEL_THREAD 0
#define AERORT_KERNEL_TEAM 1
#define AERORT_KERNEL_AUTO 2
/* AERORT_KERNEL_TERMS (FP64; the team kernel for mixed): the team solve with
 * each solve's Fourier terms spread over the warps of a block, for batches too
 * small to fill the GPU one warp per solve.  The FP64 re-solve of a mixed
 * launch's refinement list always runs in this form. */
#define AERORT_KERNEL_TERMS 3
int aerort_set_kernel(int nstreams, int precision, int kernel);
int aerort_get_kernel(int nstreams, int precision);

/* How the FP32 (mixed) team solve forms the moment contraction of its layer
 * matrices, sum_l omega beta_l P_l^m(mu_i) P_l^m(mu_j) (the SAB/DAB sums of
 * vlidort_solutions.f90:436-476): AERORT_CONTRACT_FMA (the default) on the
 * CUDA cores; AERORT_CONTRACT_TF32X3 on the tensor cores, mma.sync m16n8k8
 * with TF32 operands split as hi + lo (three products per pair, FP32
 * accumulation; an error of order 2^-22 relative).  FP64 solves and the
 * thread kernel always use the CUDA cores.  Process-wide; read when an entry
 * point is called.  No counterpart in the reference.  aerort_get_moment_
 * contraction returns the setting. */
#define AERORT_CONTRACT_FMA 0
#define AERORT_CONTRACT_TF32X3 1
int aerort_set_moment_contraction(int mode);
int aerort_get_moment_contraction(void);

/* Allocation-free form of aerort_vlidort_scalar_lambert_batch_dev (same
 * arguments, same results).  No counterpart in the reference: it exists for
 * callers that must not have the library allocate or free device memory
 * during a run (a model whose pool allocator owns the device memory, a loop
 * with other streams in flight that cudaFree would synchronise).  It calls no
 * cudaMalloc/cudaFree: its scratch is a static 256 MiB device arena (plus two
 * ints) reserved when the library's CUDA module for it is loaded.  The first
 * call on a device, made with that device current, does the set-up (symbol
 * lookup, which may load that module); make it before any stream capture.
 * The arena is reserved on every device where that module is loaded: with
 * lazy module loading (the CUDA default) only when a process first calls this
 * entry point, with CUDA_MODULE_LOADING=EAGER by every process that loads the
 * library.  After cudaDeviceReset (or any teardown of the primary context)
 * call aerort_release before the next call, so that the arena address is
 * looked up again.
 * Limits: the kernel's resident blocks are capped so their scratch fits the
 * arena (throughput drops at 12-16 streams); nobs * nch is at most
 * 2,130,706,432 (as for every RT entry point); a configuration of which not
 * even one block fits (32 threads for the thread-per-solve kernel, two warps
 * with their 64 set-up scratches for the team kernel) is rejected with
 * AERORT_RC_ARG.  Nothing needs zeroing beforehand: the work counter is reset
 * on the stream by each call and every output element is written.  Calls
 * share the arena: two calls that may overlap (different streams, or threads
 * on the same device) race; order them on one stream or with events. */
int aerort_vlidort_scalar_lambert_batch_dev_noalloc(int km, int nch, int nobs, int nstreams, int plane_parallel,
                                                    int nMom, const int* nlay, const double* ROT, const double* depol,
                                                    const double* tau, const double* ssa, const double* pmom,
                                                    const float* tau_f, const float* ssa_f, const float* pmom_f,
                                                    const double* he, const double* albedo,
                                                    const double* solar_zenith, const double* relat_azymuth,
                                                    const double* sensor_zenith, double MISSING, double* radiance_VL,
                                                    double* reflectance_VL, int* nfourier, int* status, void* stream);

/* Host-pointer form of the batched call (same extension as above, FP64
 * optics, nlay(nobs) host array or NULL).  No counterpart routine in the
 * reference: it replaces a loop of VLIDORT_Scalar_Lambert calls over columns
 * of different layer counts with one launch. */
int aerort_vlidort_scalar_lambert_batch(int km, int nch, int nobs, int nstreams, int plane_parallel, int nMom,
                                        const int* nlay, const double* ROT, const double* depol, const double* tau,
                                        const double* ssa, const double* pmom, const double* he,
                                        const double* albedo, const double* solar_zenith,
                                        const double* relat_azymuth, const double* sensor_zenith, double MISSING,
                                        double* radiance_VL, double* reflectance_VL, int* nfourier, int* status);

/* ------------------------------------------------------------------------------------------ misc */
/* Diagnostic, no counterpart in the reference: enqueue blocks x threads
 * threads each running 8 independent FP64 FMA chains for `iters` rounds
 * (16 * iters flops per thread); timing it gives the FP64 pipe rate. */
int aerort_probe_dfma(int blocks, int threads, int iters, double* out_dev, void* stream);
/* Same with FP32 FMA chains (the FP32 pipe rate that bounds the mixed solve). */
int aerort_probe_ffma(int blocks, int threads, int iters, float* out_dev, void* stream);

/* Number of kernels the library has launched since it was loaded (all entry
 * points, all streams); a diagnostic for launch accounting. */
unsigned long long aerort_launch_count(void);
const char* aerort_last_error(void);  /* last error message of the calling thread */
int aerort_version(void);             /* 100 * major + minor */
/* Release the library's cached device buffers and streams (optional). */
int aerort_release(void);

#ifdef __cplusplus
}
#endif
#endif /* AERORT_H */
