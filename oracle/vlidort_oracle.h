// Test infrastructure only: declarations shared by the CPU oracle's scalar
// (vlidort_oracle.cpp) and polarized (vlidort_vector_oracle.cpp) VLIDORT
// restatements.  Paths are relative to the reference project root
// (src/Components/rtms/RTSI/VLIDORT2p8p3/...).
#pragma once
#include <vector>

namespace orc {

// vlidort_def/vlidort_pars.f90:386-444 (truncated DEG_TO_RAD is reproduced on purpose)
constexpr double DTR = 1.7453292519943e-02;
constexpr double PIE = 180.0 * DTR;
constexpr double PI4 = 4.0 * PIE;
constexpr double TAYLOR_SMALL = 1.0e-4;
constexpr double MAX_TAU_SPATH = 32.0, MAX_TAU_UPATH = 32.0, MAX_TAU_QPATH = 32.0;
constexpr double FO_CUTOFF = 88.0;  // vlidort_focode/FO_VectorSS_RTCalcs_I.f90:325

// Options of one VLIDORT master call (the subset of VLIDORT_FixIn/ModIn that the
// AeroApps wrapper VLIDORT2p8p3/VLIDORT_Mod.F90:65-383 and the solar testers use).
struct OracleOpts {
  int do_focorr;           // DO_FOCORR (FO single scatter + direct bounce)
  int do_focorr_nadir;     // DO_FOCORR_NADIR (regular pseudo-spherical FO)
  int do_focorr_outgoing;  // DO_FOCORR_OUTGOING (enhanced pseudo-spherical FO)
  int do_deltam;           // DO_DELTAM_SCALING
  int do_plane_parallel;   // DO_PLANE_PARALLEL
  int do_double_convtest;  // DO_DOUBLE_CONVTEST
  int nfinelayers;         // NFINELAYERS
  int taylor_order;        // TAYLOR_ORDER
  double accuracy;         // VLIDORT_ACCURACY
  double asymtx_tol;       // ASYMTX_TOLERANCE
  double earth_radius;     // EARTH_RADIUS [km]
  double flux_factor;      // FLUX_FACTOR
};

// Status codes shared with the CUDA path.
enum { ORC_OK = 0, ORC_EIGEN_FAIL = 1, ORC_BVP_SINGULAR = 2, ORC_BAD_INPUT = 3 };

// vlidort_aux.f90:960-1042 GETQUAD2
void getquad2(double a, double b, int n, double* roots, double* wgts);
// vlidort_Taylor.f90 Taylor_series_1 / Taylor_Series_2
double taylor1(int order, double eps, double delta, double udel, double sm);
double taylor2(int order, double eps, double y, double delta, double fac1, double fac2, double sm);
// vlidort_aux.f90:386-956 ASYMTX (column-major, leading dimension ia)
int asymtx(double tol, double* aad, int m, int ia, double* evecd, double* evald, double* wkd, bool* bad);
// DGBTRF/DGBTRS semantics (lapack_tools.f90:6683, 7354)
int band_lu(int n, int kl, int ku, double* ab, int ldab, int* ipiv);
void band_solve(int n, int kl, int ku, const double* ab, int ldab, const int* ipiv, double* b);

struct FoGeom {
  double mu0, mu1, cosscat;
  std::vector<double> atten, lostrans, mult;  // atten[0..L], lostrans[L], mult[L]
};

// FO single-scatter geometry of one (sza, vza, raa) observation, upwelling
// (VFO_Master.f90:652 -> FO_SSWPgeometry_master.f90:101; regular pseudo-spherical
// or plane-parallel: FO_WPgeometry_Routines.f90:776; enhanced pseudo-spherical:
// :1511/:1700/:2409).  radii = earth radius + heights, ext = extinction per km
// (delta-M scaled when delta-M is on), dts = layer optical depths used on the
// line of sight.  Outputs: mu0, mu1, the scattering cosine, the solar
// attenuation at every level (atten[L] at BOA), line-of-sight transmittances and
// the layer source multipliers of SSV_Integral_I_UP (FO_VectorSS_RTCalcs_I.f90:116).
void fo_geometry(const OracleOpts* o, int L, const double* heights, const std::vector<double>& radii,
                 const std::vector<double>& ext, const std::vector<double>& dts, double sza, double vza,
                 double raa, FoGeom& G);

// One VBRDF kernel value (brdf_oracle.cpp): incident (xi, sxi), reflected
// (xj, sxj), azimuth cosine/sine; `which` as vlidort_pars.f90:466-474.
double brdf_kernel(int which, const double* pars, double xi, double sxi, double xj, double sxj, double cphi,
                   double sphi);

}  // namespace orc

extern "C" int oracle_brdf_supplement(int nk, const int* which, const double* factors, const double* pars_in,
                                      int do_shadow, int nstreams_brdf, int N, int nmom, double sza, int nvza,
                                      const double* vza, int nraa, const double* raa, double* f, double* f0,
                                      double* uf, double* uf0, double* exactdb);
