// Test harness: the per-thread solver of the CUDA kernel compiled for the host, so
// that the CPU test suite can check its numerics against the oracle.  Never
// linked by the package (which has no CPU path).
#include "../../aeroapps_gb300/csrc/rt_solve.cuh"
#include <vector>
#include <cstdio>
using namespace aerort;
static void gl(int n, double* x, double* w) {  // own Gauss-Legendre on (0,1) by Newton
  for (int i = 0; i < n; ++i) {
    double z = std::cos(M_PI * (i + 0.75) / (n + 0.5)), pp = 0;
    for (int it = 0; it < 100; ++it) {
      double p1 = 1, p2 = 0;
      for (int j = 1; j <= n; ++j) { double p3 = p2; p2 = p1; p1 = ((2.0*j-1)*z*p2 - (j-1.0)*p3)/j; }
      pp = n * (z*p1 - p2) / (z*z - 1);
      double z1 = z; z = z1 - p1/pp; if (std::fabs(z-z1) < 1e-15) break;
    }
    x[n-1-i] = 0.5 - 0.5*z; w[n-1-i] = 1.0/((1-z*z)*pp*pp);
  }
}
template <int NS, typename T>
static int run(const RtOptions& opt, const LambertInputs& in, double* rad, double* refl, int* nf, int* st) {
  double qx[NS], qw[NS], tu[4], wu[4];
  gl(NS, qx, qw);
  gl(opt.nfine > 0 ? opt.nfine : 1, tu, wu);
  ScratchLayout<NS> lay(in.km);
  std::vector<double> scr((lay.template bytes<T>() + 7) / 8);
  const SolveScratch<T> S = make_scratch<NS, T>(scr.data(), 0, 1, in.km);
  for (int s = 0; s < in.nobs * in.nch; ++s) solve_lambert<NS, T>(opt, in, s, qx, qw, tu, wu, S, rad, refl, nf, st);
  return 0;
}
static int g_plane_parallel = 0;  // VLIDORT_Scalar_Lambert's plane_parallel flag for the next calls
extern "C" void host_set_plane_parallel(int on) { g_plane_parallel = on ? 1 : 0; }
template <typename T>
static int dispatch(int km, int nch, int nobs, int nstreams, int nmom, const double* rot, const double* depol,
    const double* tau, const double* ssa, const double* pmom, const double* he, const double* albedo, const double* sza,
    const double* raa, const double* vza, const int* nadir, double missing, int max_fourier,
    double* rad, double* refl, int* nf, int* st) {
  RtOptions opt{1, 1, g_plane_parallel, 1, 3, 3, kAccuracySingle, 6371.0, 1.0, max_fourier};
  LambertInputs in{km, nch, nobs, nmom, rot, depol, tau, ssa, pmom, he, albedo, sza, raa, vza, nullptr, nullptr, nullptr, nullptr, nadir, missing};
  switch (nstreams) {
    case 4: return run<4, T>(opt, in, rad, refl, nf, st);
    case 6: return run<6, T>(opt, in, rad, refl, nf, st);
    case 8: return run<8, T>(opt, in, rad, refl, nf, st);
    case 12: return run<12, T>(opt, in, rad, refl, nf, st);
    case 16: return run<16, T>(opt, in, rad, refl, nf, st);
  }
  return -1;
}
// FP64 (plain method) solver
extern "C" int host_scalar_lambert(int km, int nch, int nobs, int nstreams, int nmom, const double* rot, const double* depol,
    const double* tau, const double* ssa, const double* pmom, const double* he, const double* albedo, const double* sza,
    const double* raa, const double* vza, const int* nadir, double missing, int max_fourier,
    double* rad, double* refl, int* nf, int* st) {
  return dispatch<double>(km, nch, nobs, nstreams, nmom, rot, depol, tau, ssa, pmom, he, albedo, sza, raa, vza, nadir,
                          missing, max_fourier, rad, refl, nf, st);
}
// mixed method: FP32 Fourier series
extern "C" int host_scalar_lambert_mixed(int km, int nch, int nobs, int nstreams, int nmom, const double* rot, const double* depol,
    const double* tau, const double* ssa, const double* pmom, const double* he, const double* albedo, const double* sza,
    const double* raa, const double* vza, const int* nadir, double missing, int max_fourier,
    double* rad, double* refl, int* nf, int* st) {
  return dispatch<float>(km, nch, nobs, nstreams, nmom, rot, depol, tau, ssa, pmom, he, albedo, sza, raa, vza, nadir,
                         missing, max_fourier, rad, refl, nf, st);
}
// The mixed method's refinement decision for one Fourier series: terms sf[0..n)
// (before the azimuth factor), relative azimuth raa; returns 1 when the solve
// would be handed to the FP64 pass, and the last term in *mlast.
extern "C" int host_refine_flag(int n, const double* sf, double raa, int* mlast) {
  RtOptions opt{0, 1, 0, 1, 3, 3, kAccuracySingle, 6371.0, 1.0, -1};
  SetupRecord r{};
  r.raa = raa;
  FourierSum sum;
  int m = 0;
  for (m = 0; m < n; ++m)
    if (sum.add(opt, r, m, sf[m])) break;
  *mlast = m;
  int count = 0, list[1];
  Worklist wl;
  wl.out_list = list;
  wl.out_count = &count;
  wl.ratio = kRefineRatio;
  wl.flag(sum, RT_OK, 0);
  return count;
}
