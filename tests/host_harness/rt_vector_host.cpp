// Test harness: the polarized warp solve of the CUDA kernel (rt_vector.cuh)
// run on the host, one std::thread per lane with a barrier for the warp
// synchronisation, so that the CPU test suite can compare it with the oracle.
// Never linked by the package.
#include "../../aeroapps_gb300/csrc/rt_vector.cuh"
#include <barrier>
#include <memory>
#include <thread>
#include <vector>
using namespace aerort;
static void gl(int n, double* x, double* w) {
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
static void bar_sync(void* b) { static_cast<std::barrier<>*>(b)->arrive_and_wait(); }
template <int N>
static int run(const RtOptions& opt, const VectorInputs& vin, double* rad, double* refl, double* Q, double* U, int* nf,
               int* st) {
  double qx[N], qw[N], tu[4] = {0, 0, 0, 0}, wu[4] = {0, 0, 0, 0};
  gl(N, qx, qw);
  gl(opt.nfine > 0 ? opt.nfine : 1, tu, wu);
  const VecLayout<N> lay(vin.base.km);
  std::vector<double> ws(lay.total, 0.0);
  auto sh = std::make_unique<VecShared<N>>();
  const int nsolve = vin.base.nobs * vin.base.nch;
  for (int s = 0; s < nsolve; ++s) {
    std::barrier<> bar(kTeam);
    std::vector<std::thread> th;
    for (int lane = 0; lane < kTeam; ++lane)
      th.emplace_back([&, lane] {
        const Team tm{lane, bar_sync, &bar};
        vec_solve<N>(tm, *sh, opt, vin, s, qx, qw, tu, wu, ws.data(), rad, refl, Q, U, nf, st);
      });
    for (auto& t : th) t.join();
  }
  return 0;
}
extern "C" int host_vector_lambert(int km, int nch, int nobs, int nstreams, int nmom, const double* rot,
                                   const double* depol, const double* alpha, const double* tau, const double* ssa,
                                   const double* pmom, const double* he, const double* albedo, const double* sza,
                                   const double* raa, const double* vza, const double* flux, const int* nadir_first,
                                   const int* nlay, double missing, int max_fourier, double* rad, double* refl,
                                   double* Q, double* U, int* nf, int* st) {
  RtOptions opt{1, 1, 0, 1, 3, 3, kAccuracySingle, 6371.0, 1.0, max_fourier};
  VectorInputs vin;
  vin.base = LambertInputs{km, nch, nobs, nmom, rot, depol, tau, ssa, pmom, he, albedo, sza, raa, vza, nlay, nullptr,
                           nullptr, nullptr, nadir_first, missing, alpha};
  vin.flux_factor = flux;
  switch (nstreams) {
    case 4: return run<4>(opt, vin, rad, refl, Q, U, nf, st);
    case 6: return run<6>(opt, vin, rad, refl, Q, U, nf, st);
    case 8: return run<8>(opt, vin, rad, refl, Q, U, nf, st);
    case 12: return run<12>(opt, vin, rad, refl, Q, U, nf, st);
  }
  return -1;
}
