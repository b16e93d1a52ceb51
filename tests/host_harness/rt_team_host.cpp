// Test harness: the team-cooperative Fourier series of the CUDA kernel run on
// the host, one std::thread per lane with a barrier for the warp
// synchronisation, so that the CPU test suite can compare it with the
// thread-per-solve solver.  Never linked by the package.
#include "../../aeroapps_gb300/csrc/rt_team.cuh"
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
template <int NS, typename T>
static int run(const RtOptions& opt, const LambertInputs& in, double* rad, double* refl, int* nf, int* st) {
  double qx[NS], qw[NS], tu[4], wu[4];
  gl(NS, qx, qw);
  gl(opt.nfine > 0 ? opt.nfine : 1, tu, wu);
  ScratchLayout<NS> lay(in.km, false);
  std::vector<double> scr((lay.template bytes<T>() + 7) / 8);
  auto M = std::make_unique<TeamMem<NS, T>>();
  const SolveScratch<T> S = make_scratch<NS, T>(scr.data(), 0, 1, in.km, false);
  for (int s = 0; s < in.nobs * in.nch; ++s) {
    SetupRecord r;
    if (!solve_setup<NS, T>(opt, in, s, tu, wu, S, rad, refl, nf, st, r)) continue;
    r.store(S.D, lay.rec);
    SetupRecord rb;
    rb.load(S.D, lay.rec);
    std::barrier<> bar(kTeam);
    std::vector<std::thread> th;
    for (int lane = 0; lane < kTeam; ++lane)
      th.emplace_back([&, lane] {
        const Team tm{lane, bar_sync, &bar};
        team_fourier_series<NS, T>(tm, *M, opt, in, rb, qx, qw, S.W, lay, rad, refl, nf, st);
      });
    for (auto& t : th) t.join();
  }
  return 0;
}
static int g_plane_parallel = 0;  // VLIDORT_Scalar_Lambert's plane_parallel flag for the next calls
extern "C" void team_set_plane_parallel(int on) { g_plane_parallel = on ? 1 : 0; }
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
extern "C" int team_scalar_lambert(int km, int nch, int nobs, int nstreams, int nmom, const double* rot, const double* depol,
    const double* tau, const double* ssa, const double* pmom, const double* he, const double* albedo, const double* sza,
    const double* raa, const double* vza, const int* nadir, double missing, int max_fourier,
    double* rad, double* refl, int* nf, int* st) {
  return dispatch<double>(km, nch, nobs, nstreams, nmom, rot, depol, tau, ssa, pmom, he, albedo, sza, raa, vza, nadir,
                          missing, max_fourier, rad, refl, nf, st);
}
extern "C" int team_scalar_lambert_mixed(int km, int nch, int nobs, int nstreams, int nmom, const double* rot, const double* depol,
    const double* tau, const double* ssa, const double* pmom, const double* he, const double* albedo, const double* sza,
    const double* raa, const double* vza, const int* nadir, double missing, int max_fourier,
    double* rad, double* refl, int* nf, int* st) {
  return dispatch<float>(km, nch, nobs, nstreams, nmom, rot, depol, tau, ssa, pmom, he, albedo, sza, raa, vza, nadir,
                         missing, max_fourier, rad, refl, nf, st);
}

// The RTLS BRDF surface (VLIDORT_Scalar_LandMODIS) through the same team
// solve: Fourier tables and per-solve blocks built as the CUDA entry point
// builds them, one solve at a time.  kw (3, nch, nobs), param (2, nch, nobs).
template <int NS>
static int run_brdf(const RtOptions& opt, const LambertInputs& in, const double* kw, const double* param,
                    double* rad, double* refl, double* br, int* nf, int* st) {
  double qx[NS], qw[NS], tu[4], wu[4];
  gl(NS, qx, qw);
  gl(opt.nfine > 0 ? opt.nfine : 1, tu, wu);
  BrdfInputs b{};
  b.kind = kBrdfRTLS;
  b.q.nb = kBrdfAzimuth;
  double ax[kBrdfAzimuth], aw[kBrdfAzimuth];
  gl(kBrdfAzimuth, ax, aw);
  for (int k = 0; k < kBrdfAzimuth; ++k) {
    b.q.phi[k] = kPIE * ax[k];
    b.q.a[k] = aw[k];
    b.q.c[k] = std::cos(b.q.phi[k]);
    b.q.s[k] = std::sin(b.q.phi[k]);
  }
  for (int q = 0; q < NS; ++q) b.qx[q] = qx[q];
  // one Li-sparse table per (pixel, channel): tab[w] = w
  const int nsolve = in.nobs * in.nch;
  std::vector<double> tpar(2 * nsolve), qq((size_t)(1 + nsolve) * 2 * NS * NS * NS);
  std::vector<int> tab(nsolve);
  brdf_qq_table(NS, qx, b.q, false, 0.0, 0.0, qq.data());
  for (int w = 0; w < nsolve; ++w) {
    tab[w] = w;
    tpar[2 * w] = param[2 * w];
    tpar[2 * w + 1] = param[2 * w + 1];
    brdf_qq_table(NS, qx, b.q, true, tpar[2 * w], tpar[2 * w + 1], qq.data() + (size_t)(1 + w) * 2 * NS * NS * NS);
  }
  std::vector<double> terms(BrdfBlock<NS>::total);
  b.kw = kw; b.tab = tab.data(); b.tpar = tpar.data(); b.qq = qq.data(); b.br = br;
  b.terms = terms.data(); b.stride = 1;
  ScratchLayout<NS> lay(in.km, false);
  std::vector<double> scr((lay.template bytes<double>() + 7) / 8);
  auto M = std::make_unique<TeamMem<NS, double>>();
  const SolveScratch<double> S = make_scratch<NS, double>(scr.data(), 0, 1, in.km, false);
  for (int s = 0; s < nsolve; ++s) {
    SetupRecord r;
    if (!solve_setup<NS, double>(opt, in, s, tu, wu, S, rad, refl, nf, st, r, &b, 0)) continue;
    r.store(S.D, lay.rec);
    SetupRecord rb;
    rb.load(S.D, lay.rec);
    std::barrier<> bar(kTeam);
    std::vector<std::thread> th;
    for (int lane = 0; lane < kTeam; ++lane)
      th.emplace_back([&, lane] {
        const Team tm{lane, bar_sync, &bar};
        team_fourier_series<NS, double, true>(tm, *M, opt, in, rb, qx, qw, S.W, lay, rad, refl, nf, st, Worklist(), 0,
                                              &b, 0);
      });
    for (auto& t : th) t.join();
  }
  return 0;
}
extern "C" int team_scalar_landmodis(int km, int nch, int nobs, int nstreams, int nmom, const double* rot,
    const double* depol, const double* tau, const double* ssa, const double* pmom, const double* he,
    const double* kw, const double* param, const double* sza, const double* raa, const double* vza,
    const int* nadir, double missing, double* rad, double* refl, double* br, int* nf, int* st) {
  RtOptions opt{1, 1, g_plane_parallel, 1, 3, 3, kAccuracySingle, 6371.0, 1.0, -1};
  LambertInputs in{km, nch, nobs, nmom, rot, depol, tau, ssa, pmom, he, nullptr, sza, raa, vza, nullptr, nullptr,
                   nullptr, nullptr, nadir, missing};
  switch (nstreams) {
    case 4: return run_brdf<4>(opt, in, kw, param, rad, refl, br, nf, st);
    case 6: return run_brdf<6>(opt, in, kw, param, rad, refl, br, nf, st);
    case 8: return run_brdf<8>(opt, in, kw, param, rad, refl, br, nf, st);
    case 12: return run_brdf<12>(opt, in, kw, param, rad, refl, br, nf, st);
    case 16: return run_brdf<16>(opt, in, kw, param, rad, refl, br, nf, st);
  }
  return -1;
}

// The Cox-Munk glint (VLIDORT_Scalar_CX) through the same team solve: each
// solve's terms built as the CUDA set-up builds them.  U10m, V10m (nobs), mr (nch).
template <int NS>
static int run_cx(int kind, const RtOptions& opt, const LambertInputs& in, const double* u10, const double* v10,
                  const double* mr, double* rad, double* refl, double* br, int* nf, int* st) {
  double qx[NS], qw[NS], tu[4], wu[4];
  gl(NS, qx, qw);
  gl(opt.nfine > 0 ? opt.nfine : 1, tu, wu);
  BrdfInputs b{};
  b.kind = kind;
  b.q.nb = kBrdfAzimuthCX;
  double ax[kBrdfAzimuthCX], aw[kBrdfAzimuthCX];
  gl(kBrdfAzimuthCX, ax, aw);
  for (int k = 0; k < kBrdfAzimuthCX; ++k) {
    b.q.phi[k] = kPIE * ax[k];
    b.q.a[k] = aw[k];
    b.q.c[k] = std::cos(b.q.phi[k]);
    b.q.s[k] = std::sin(b.q.phi[k]);
  }
  for (int q = 0; q < NS; ++q) b.qx[q] = qx[q];
  std::vector<double> cf((size_t)2 * NS * kBrdfAzimuthCX);
  for (int m = 0; m < 2 * NS; ++m)
    for (int k = 0; k < kBrdfAzimuthCX; ++k)
      cf[(size_t)m * kBrdfAzimuthCX + k] = (m == 0) ? b.q.a[k] : b.q.a[k] * std::cos((double)m * b.q.phi[k]);
  std::vector<double> terms(BrdfBlock<NS>::total_cx);
  b.u10 = u10; b.v10 = v10; b.mr = mr; b.cf = cf.data(); b.br = br;
  b.terms = terms.data(); b.stride = 1;
  const int nsolve = in.nobs * in.nch;
  ScratchLayout<NS> lay(in.km, false);
  std::vector<double> scr((lay.template bytes<double>() + 7) / 8);
  auto M = std::make_unique<TeamMem<NS, double>>();
  const SolveScratch<double> S = make_scratch<NS, double>(scr.data(), 0, 1, in.km, false);
  for (int s = 0; s < nsolve; ++s) {
    SetupRecord r;
    if (!solve_setup<NS, double>(opt, in, s, tu, wu, S, rad, refl, nf, st, r, &b, 0)) continue;
    r.store(S.D, lay.rec);
    SetupRecord rb;
    rb.load(S.D, lay.rec);
    std::barrier<> bar(kTeam);
    std::vector<std::thread> th;
    for (int lane = 0; lane < kTeam; ++lane)
      th.emplace_back([&, lane] {
        const Team tm{lane, bar_sync, &bar};
        team_fourier_series<NS, double, true>(tm, *M, opt, in, rb, qx, qw, S.W, lay, rad, refl, nf, st, Worklist(), 0,
                                              &b, 0);
      });
    for (auto& t : th) t.join();
  }
  return 0;
}
static int dispatch_cx(int kind, int km, int nch, int nobs, int nstreams, int nmom, const double* rot,
    const double* depol, const double* tau, const double* ssa, const double* pmom, const double* he,
    const double* u10, const double* v10, const double* mr, const double* sza, const double* raa, const double* vza,
    const int* nadir, double missing, double* rad, double* refl, double* br, int* nf, int* st) {
  RtOptions opt{1, 1, g_plane_parallel, 1, 3, 3, kAccuracySingle, 6371.0, 1.0, -1};
  LambertInputs in{km, nch, nobs, nmom, rot, depol, tau, ssa, pmom, he, nullptr, sza, raa, vza, nullptr, nullptr,
                   nullptr, nullptr, nadir, missing};
  switch (nstreams) {
    case 4: return run_cx<4>(kind, opt, in, u10, v10, mr, rad, refl, br, nf, st);
    case 6: return run_cx<6>(kind, opt, in, u10, v10, mr, rad, refl, br, nf, st);
    case 8: return run_cx<8>(kind, opt, in, u10, v10, mr, rad, refl, br, nf, st);
    case 12: return run_cx<12>(kind, opt, in, u10, v10, mr, rad, refl, br, nf, st);
    case 16: return run_cx<16>(kind, opt, in, u10, v10, mr, rad, refl, br, nf, st);
  }
  return -1;
}
// giss = 0: VLIDORT_Scalar_CX's Cox-Munk kernel; 1: VLIDORT_Scalar_GissCX's GISS kernel
extern "C" int team_scalar_cx(int giss, int km, int nch, int nobs, int nstreams, int nmom, const double* rot,
    const double* depol, const double* tau, const double* ssa, const double* pmom, const double* he,
    const double* u10, const double* v10, const double* mr, const double* sza, const double* raa, const double* vza,
    const int* nadir, double missing, double* rad, double* refl, double* br, int* nf, int* st) {
  return dispatch_cx(giss ? kBrdfGissCoxMunk : kBrdfCoxMunk, km, nch, nobs, nstreams, nmom, rot, depol, tau, ssa,
                     pmom, he, u10, v10, mr, sza, raa, vza, nadir, missing, rad, refl, br, nf, st);
}

// The term-parallel FP64 re-solve of the mixed method's refinement list
// (k_refine_terms) emulated on the host: W teams per solve, team w running the
// terms m0 + w of each round with its own shared memory, the Fourier sum
// taken in term order after each round.  Each round's teams run one after
// another (they share nothing but the solve's scratch).
template <int NS>
static int run_termpar(int W, const RtOptions& opt, const LambertInputs& in, double* rad, double* refl, int* nf,
                       int* st) {
  double qx[NS], qw[NS], tu[4], wu[4];
  gl(NS, qx, qw);
  gl(opt.nfine > 0 ? opt.nfine : 1, tu, wu);
  ScratchLayout<NS> lay(in.km, false);
  std::vector<double> scr((lay.template bytes<double>() + 7) / 8);
  std::vector<std::unique_ptr<TeamMem<NS, double>>> M(W);
  for (auto& m : M) m = std::make_unique<TeamMem<NS, double>>();
  std::vector<SolveCtx<NS, double>> ctx((size_t)W * kTeam);
  const SolveScratch<double> S = make_scratch<NS, double>(scr.data(), 0, 1, in.km, false);
  for (int s = 0; s < in.nobs * in.nch; ++s) {
    SetupRecord r;
    if (!solve_setup<NS, double>(opt, in, s, tu, wu, S, rad, refl, nf, st, r)) continue;
    r.store(S.D, lay.rec);
    SetupRecord rb;
    rb.load(S.D, lay.rec);
    std::vector<int> last(W, -1);
    FourierSum sum;
    int mfin = 0, stfin = RT_OK;
    for (int m0 = 0;; m0 += W) {
      std::vector<double> sf(W, 0.0);
      std::vector<int> tst(W, RT_OK);
      for (int w = 0; w < W; ++w) {
        const int m = m0 + w;
        if (m > rb.n_fouriers) continue;
        std::barrier<> bar(kTeam);
        std::vector<std::thread> th;
        std::vector<double> out(kTeam, 0.0);
        std::vector<int> rc(kTeam, RT_OK);
        for (int lane = 0; lane < kTeam; ++lane)
          th.emplace_back([&, lane] {
            const Team tm{lane, bar_sync, &bar};
            SolveCtx<NS, double>& c = ctx[(size_t)w * kTeam + lane];
            if (m0 == 0) team_series_init<NS, double>(tm, *M[w], rb, qx, qw, c);
            team_skip_terms<NS, double>(tm, *M[w], c, last[w], m);
            double x = 0.0;
            rc[lane] = team_fourier_term<NS, double>(tm, *M[w], c, opt, m, S.W, lay, &x);
            out[lane] = x;
          });
        for (auto& t : th) t.join();
        last[w] = m;
        sf[w] = out[0];
        tst[w] = rc[0];
      }
      int stop = 0;
      for (int k = 0; k < W && !stop; ++k) {
        const int mk = m0 + k;
        if (mk > rb.n_fouriers) { stop = 1; mfin = mk; stfin = RT_OK; }
        else if (tst[k] != RT_OK) { stop = 1; mfin = mk; stfin = tst[k]; }
        else if (sum.add(opt, rb, mk, sf[k])) { stop = 1; mfin = mk; stfin = RT_OK; }
      }
      if (stop) break;
    }
    solve_finish(opt, in, rb, stfin, mfin, sum.stokes, rad, refl, nf, st);
  }
  return 0;
}
extern "C" int team_scalar_lambert_termpar(int W, int km, int nch, int nobs, int nstreams, int nmom,
    const double* rot, const double* depol, const double* tau, const double* ssa, const double* pmom,
    const double* he, const double* albedo, const double* sza, const double* raa, const double* vza,
    const int* nadir, double missing, double* rad, double* refl, int* nf, int* st) {
  RtOptions opt{1, 1, g_plane_parallel, 1, 3, 3, kAccuracySingle, 6371.0, 1.0, -1};
  LambertInputs in{km, nch, nobs, nmom, rot, depol, tau, ssa, pmom, he, albedo, sza, raa, vza, nullptr, nullptr,
                   nullptr, nullptr, nadir, missing};
  switch (nstreams) {
    case 4: return run_termpar<4>(W, opt, in, rad, refl, nf, st);
    case 6: return run_termpar<6>(W, opt, in, rad, refl, nf, st);
    case 8: return run_termpar<8>(W, opt, in, rad, refl, nf, st);
    case 12: return run_termpar<12>(W, opt, in, rad, refl, nf, st);
    case 16: return run_termpar<16>(W, opt, in, rad, refl, nf, st);
  }
  return -1;
}
