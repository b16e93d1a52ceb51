// Test infrastructure only: the CPU oracle for the polarized (NSTOKES = 1 or 3)
// VLIDORT 2.8.3 solar path.
//
// Restates, routine by routine and in FP64, the reference's vector forward model
// for one column seen in one solar geometry (observation geometry, or a one-SZA
// lattice of user zenith/azimuth angles): Lambertian surface, pseudo-spherical
// beam, Green's-function particular integral (the 2.8.3 default for NSTOKES <= 3),
// real eigensolver (DO_REAL_EIGENSOLVER is always set for NSTOKES = 3,
// vlidort_inputs.f90:4425-4456), TOA upwelling Stokes vector, first-order
// single-scatter + direct-bounce correction.  It is the checker for the CUDA
// polarized kernel; no product code links it.  Paths are relative to the
// reference project root (src/Components/rtms/RTSI/VLIDORT2p8p3/...).
//
// Parity pin: tests/test_oracle_golden_vector.py compares this oracle with the
// reference's saved gfortran results vlidort_v_test/saved_results/gfortran/
// nstokes3/results_solar_tester_IQU0.all (I, Q, U) and
// results_solar_tester_I000.all (NSTOKES = 1 through this vector code).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include <omp.h>

#include "vlidort_oracle.h"

using namespace orc;

namespace {
// Greek-matrix entry of Stokes element pair (o1, o2), 0-based (MUELLER_INDEX,
// vlidort_inputs.f90: MAXSTOKES*(O1-1)+O2).
inline int mueller(int o1, int o2) { return 4 * o1 + o2; }
// DMAT = diag(1, 1, -1, -1) (vlidort_inputs.f90:4184-4190)
inline double dmat(int o) { return o < 2 ? 1.0 : -1.0; }
}  // namespace

extern "C" {

// One polarized VLIDORT solve for a single solar beam with nvza user zenith
// angles and nraa azimuths.  NS = NSTOKES (1 or 3).  greek_in holds the 16
// Greek-matrix entries of GREEKMAT_TOTAL_INPUT: entry k (0..15, row-major 4x4)
// of moment l in layer n at greek_in[l + (ngreek+1) * (n + L * k)].
// out[o + NS * (ua + nraa * um)] is TOA upwelling STOKES(1, geom, o, UPIDX).
// nfourier_out = last Fourier term summed.  Returns a status code.
int oracle_vlidort_vector_solve(const OracleOpts* o, int NS, int L, int N, int ngreek, const double* heights,
                                const double* deltau_in, const double* omega_in, const double* greek_in,
                                double albedo, double sza, int nvza, const double* vza, int nraa, const double* raa,
                                double* out, int* nfourier_out) {
  if (NS != 1 && NS != 3) return ORC_BAD_INPUT;
  const int order = o->taylor_order;
  const int NM = std::min(2 * N - 1, ngreek);  // vlidort_inputs.f90:4141
  const int G1 = ngreek + 1;
  const int N2 = 2 * N;
  const int NSN = NS * N, NSN2 = 2 * NSN;  // NSTKS_NSTRMS, NSTKS_NSTRMS_2
  const int NM1 = NM + 1;
  auto GIN = [&](int l, int n, int k) { return greek_in[l + G1 * (n + L * k)]; };
  // ---------------------------------------------------------------- derive input (vlidort_inputs.f90)
  std::vector<double> qx(N), qw(N), strmwts(N), halfwts(N);
  if (N == 1) { qx[0] = std::sqrt(1.0 / 3.0); qw[0] = 1.0; }
  else getquad2(0.0, 1.0, N, qx.data(), qw.data());
  for (int i = 0; i < N; ++i) { strmwts[i] = qx[i] * qw[i]; halfwts[i] = 0.5 * qw[i]; }
  std::vector<double> mu_u(nvza), sec_u(nvza);
  for (int u = 0; u < nvza; ++u) { mu_u[u] = std::cos(DTR * vza[u]); sec_u[u] = 1.0 / mu_u[u]; }
  const double cos_sza = std::cos(sza * DTR);
  // DO_LAYER_SCATTERING(M,N) from the (1,1) entries, vlidort_inputs.f90:4321-4330
  std::vector<char> laysc((NM + 1) * L, 1);
  for (int m = 3; m <= NM; ++m) {
    int qc = NM - m + 1;
    for (int n = 0; n < L; ++n) {
      int q = 0;
      for (int l = m; l <= NM; ++l)
        if (GIN(l, n, 0) == 0.0) q++;
      laysc[m + (NM + 1) * n] = (q < qc);
    }
  }
  // ---------------------------------------------------------------- Chapman factors (vlidort_geometry.f90:119-317)
  std::vector<double> chap(L * L, 0.0);
  {
    double mu_toa = std::cos(sza * DTR);
    double sn_toa = std::sqrt(1.0 - mu_toa * mu_toa);
    std::vector<double> radii(L + 1), delz(L + 1);
    radii[0] = heights[0] + o->earth_radius;
    for (int n = 1; n <= L; ++n) { radii[n] = heights[n] + o->earth_radius; delz[n] = heights[n - 1] - heights[n]; }
    if (o->do_plane_parallel) {
      for (int n = 0; n < L; ++n) for (int k = 0; k <= n; ++k) chap[n * L + k] = 1.0 / mu_toa;
    } else if (sn_toa == 0.0) {
      for (int n = 0; n < L; ++n) for (int k = 0; k <= n; ++k) chap[n * L + k] = 1.0;
    } else {
      for (int n = 1; n <= L; ++n) {
        double sinth1 = sn_toa * radii[n] / radii[0];
        double sth1 = std::asin(sinth1);
        double re_upper = radii[0];
        for (int k = 1; k <= n; ++k) {
          double re_lower = re_upper - delz[k];
          double sinth2 = re_upper * sinth1 / re_lower;
          double sth2 = std::asin(sinth2);
          double phi = sth2 - sth1;
          double dist = re_upper * std::sin(phi) / sinth2;
          chap[(n - 1) * L + (k - 1)] = dist / delz[k];
          re_upper = re_lower; sinth1 = sinth2; sth1 = sth2;
        }
      }
    }
  }
  // ---------------------------------------------------------------- delta-M scaling (vlidort_miscsetups.f90:370-758)
  // greek[l + NM1*(n + L*k)]: scaled entries KTYPE1 = 1,6,11,16 and KTYPE2 = 2,5,12,15 (vector), entry 1 (scalar)
  static const int KT1[4] = {0, 5, 10, 15}, KT2[4] = {1, 4, 11, 14};
  std::vector<double> dtau(L), omg(L), fac1(L), trunc(L), greek((size_t)NM1 * L * 16, 0.0);
  auto GR = [&](int l, int n, int k) -> double& { return greek[l + (size_t)NM1 * (n + (size_t)L * k)]; };
  for (int n = 0; n < L; ++n) {
    double fdel = 0.0;
    if (o->do_deltam) fdel = (NM1 <= ngreek ? GIN(NM1, n, 0) : 0.0) / (double)(2 * NM1 + 1);
    double fac2 = 1.0 - fdel;
    fac1[n] = o->do_deltam ? 1.0 - fdel * omega_in[n] : 1.0;
    trunc[n] = o->do_deltam ? fdel : 0.0;
    for (int l = 0; l <= NM; ++l) {
      double fdnl1 = fdel * (double)(2 * l + 1);
      if (NS > 1) {
        for (int kk = 0; kk < 4; ++kk) {
          if (o->do_deltam) {
            GR(l, n, KT1[kk]) = (GIN(l, n, KT1[kk]) - fdnl1) / fac2;
            GR(l, n, KT2[kk]) = GIN(l, n, KT2[kk]) / fac2;
          } else {
            GR(l, n, KT1[kk]) = GIN(l, n, KT1[kk]);
            GR(l, n, KT2[kk]) = GIN(l, n, KT2[kk]);
          }
        }
      } else {
        GR(l, n, 0) = o->do_deltam ? (GIN(l, n, 0) - fdnl1) / fac2 : GIN(l, n, 0);
      }
    }
    if (o->do_deltam) {
      GR(0, n, 0) = 1.0;
      dtau[n] = deltau_in[n] * fac1[n];
      omg[n] = omega_in[n] * fac2 / fac1[n];
    } else {
      dtau[n] = deltau_in[n];
      omg[n] = omega_in[n];
    }
  }
  for (int n = 0; n < L; ++n) {  // singularity busters :627-651
    if (omg[n] > 0.999999999) omg[n] = 0.999999999;
    else if (omg[n] < 1.0e-9) omg[n] = 1.0e-9;
    double g1 = GR(1, n, 0) / 3.0;
    if (g1 > 0.999999999) g1 = 0.999999999;
    else if (g1 < -0.999999999) g1 = -0.999999999;
    else if (g1 >= 0.0 && g1 < 1.0e-9) g1 = 1.0e-9;
    else if (g1 < 0.0 && g1 > -1.0e-9) g1 = -1.0e-9;
    GR(1, n, 0) = 3.0 * g1;
  }
  std::vector<double> tauslant(L + 1, 0.0);
  for (int n = 0; n < L; ++n) {
    double tau = 0.0;
    for (int k = 0; k <= n; ++k) tau += (deltau_in[k] * chap[n * L + k]) * (o->do_deltam ? fac1[k] : 1.0);
    tauslant[n + 1] = tau;
  }
  // SSALBINIT :762 -- OMEGA_GREEK(l, n, o1, o2) at og[l + NM1*(n + L*(o1 + 4*o2))]
  std::vector<double> og((size_t)NM1 * L * 16, 0.0);
  auto OG = [&](int l, int n, int o1, int o2) -> double& {
    return og[l + (size_t)NM1 * (n + (size_t)L * (o1 + 4 * o2))];
  };
  for (int n = 0; n < L; ++n)
    for (int l = 0; l <= NM; ++l)
      for (int o1 = 0; o1 < NS; ++o1)
        for (int o2 = 0; o2 < NS; ++o2) OG(l, n, o1, o2) = omg[n] * GR(l, n, mueller(o1, o2));
  // ---------------------------------------------------------------- QSPREP :813-1010
  int cutoff = L;
  std::vector<double> avsec(L, 0.0), itrans(L, 0.0);
  double trans_solar_beam = 0.0;
  bool refl_directbeam = false;
  {
    std::vector<double> taugrid(L + 1, 0.0);
    for (int n = 0; n < L; ++n) taugrid[n + 1] = taugrid[n] + dtau[n];
    double tau_solar;
    if (o->do_plane_parallel) {
      double sec0 = 1.0 / cos_sza;
      for (int n = 1; n <= L; ++n) {
        double ts = taugrid[n] * sec0;
        if (n <= cutoff) {
          if (ts > MAX_TAU_SPATH) cutoff = n;
          avsec[n - 1] = sec0;
          itrans[n - 1] = std::exp(-taugrid[n - 1] * sec0);
        }
      }
      tau_solar = taugrid[L] * sec0;
    } else {
      tau_solar = tauslant[L];
      double s_t_1 = 0.0, s_t_0 = 1.0;
      for (int n = 1; n <= L; ++n) {
        if (n <= cutoff) {
          if (tauslant[n] > MAX_TAU_SPATH) cutoff = n;
          else s_t_1 = std::exp(-tauslant[n]);
          avsec[n - 1] = (tauslant[n] - tauslant[n - 1]) / dtau[n - 1];
          itrans[n - 1] = s_t_0;
          s_t_0 = s_t_1;
        }
      }
    }
    if (tau_solar < MAX_TAU_SPATH) { trans_solar_beam = std::exp(-tau_solar); refl_directbeam = true; }
  }
  // ---------------------------------------------------------------- PREPTRANS :1014-1292, EMULT :3187
  std::vector<double> t_mubar(L, 0.0), t_user(L * nvza, 0.0), itrans_u(L * nvza, 0.0);
  for (int n = 0; n < L; ++n) {
    if (n + 1 <= cutoff) {
      double sp = dtau[n] * avsec[n];
      t_mubar[n] = sp > MAX_TAU_SPATH ? 0.0 : std::exp(-sp);
    }
    for (int u = 0; u < nvza; ++u) {
      itrans_u[n + L * u] = itrans[n] * sec_u[u];
      double sp = dtau[n] * sec_u[u];
      t_user[n + L * u] = sp > MAX_TAU_UPATH ? 0.0 : std::exp(-sp);
    }
  }
  std::vector<double> sigma_p(L * nvza), emult_up(L * nvza, 0.0);
  for (int n = 0; n < L; ++n)
    for (int u = 0; u < nvza; ++u) {
      sigma_p[n + L * u] = avsec[n] + sec_u[u];
      if (n + 1 <= cutoff) {
        double wudel = t_mubar[n] * t_user[n + L * u];
        double su = (1.0 - wudel) / sigma_p[n + L * u];
        emult_up[n + L * u] = itrans_u[n + L * u] * su;
      }
    }
  // ---------------------------------------------------------------- FO single scatter + direct bounce
  // vlidort_vfo_interface.f90:128 -> VFO_Master.f90:123; FO_VectorSS_Spherfuncs.f90:93 (NSTOKES > 1
  // with sunlight: P00 and P02 functions and the rotation C2, S2), FO_VectorSS_RTCalcs_I.f90:116
  // (exactscat = tms * (F11, -F12 C2, F12 S2); Lambertian direct bounce in I only)
  const int NG = nvza * nraa;
  std::vector<double> ss((size_t)NG * NS, 0.0), db((size_t)NG * NS, 0.0);
  if (o->do_focorr) {
    const double flux = o->flux_factor / PI4;
    std::vector<double> radii(L + 1), ext(L), dts(L), tms(L);
    for (int n = 0; n <= L; ++n) radii[n] = o->earth_radius + heights[n];
    for (int n = 0; n < L; ++n) {
      double dz = heights[n] - heights[n + 1];
      dts[n] = o->do_deltam ? dtau[n] : deltau_in[n];
      ext[n] = dts[n] / dz;
      tms[n] = o->do_deltam ? omega_in[n] / (1.0 - trunc[n] * omega_in[n]) : omega_in[n];
    }
    for (int u = 0; u < nvza; ++u)
      for (int a = 0; a < nraa; ++a) {
        const int g = a + nraa * u;
        FoGeom G;
        fo_geometry(o, L, heights, radii, ext, dts, sza, vza[u], raa[a], G);
        const double mus = G.cosscat;
        // generalized spherical functions at the scattering angle
        std::vector<double> p00(ngreek + 1, 0.0), p02(ngreek + 1, 0.0);
        p00[0] = 1.0;
        if (ngreek >= 1) p00[1] = mus;
        for (int l = 2; l <= ngreek; ++l)
          p00[l] = ((double)(2 * l - 1) / (double)l) * mus * p00[l - 1] - ((double)(l - 1) / (double)l) * p00[l - 2];
        if (NS > 1 && ngreek >= 2) {
          const double qroot6 = -0.25 * std::sqrt(6.0);
          p02[2] = qroot6 * (1.0 - mus) * (1.0 + mus);
          double sql41 = 0.0;
          for (int l = 3; l <= ngreek; ++l) {
            double sql4 = sql41;
            double dl = (double)l;
            sql41 = std::sqrt(dl * dl - 4.0);
            double g3 = (double)(2 * l - 1) / sql41, g4 = sql4 / sql41;
            p02[l] = g3 * mus * p02[l - 1] - g4 * p02[l - 2];
          }
        }
        // rotation angles (H/VDM eqs. 89-101), VSIGN = +1 upwelling
        double c2 = 0.0, s2 = 0.0;
        if (NS > 1) {
          const double small = 1.0e-12, vsign = 1.0;
          double th_r = DTR * sza, ctheta = std::cos(th_r), stheta = std::sin(th_r);
          double al_r = DTR * vza[u], calpha = std::cos(al_r), salpha = std::sin(al_r);
          double cphi = std::cos(DTR * raa[a]);
          double hs = 1.0 - mus * mus, sinscat = hs <= 0.0 ? small : std::sqrt(hs);
          double csig2;
          if (std::fabs(sinscat) <= small) csig2 = 0.0;
          else if (salpha == 0.0) csig2 = -cphi;
          else csig2 = (-ctheta - vsign * calpha * mus) / sinscat / salpha;
          if (csig2 > 1.0) csig2 = 1.0;
          if (csig2 < -1.0) csig2 = -1.0;
          double csig2_2 = 2.0 * csig2;
          double ssig2 = std::fabs(csig2 - 1.0) < small ? 0.0 : std::sqrt(1.0 - csig2 * csig2);
          c2 = csig2_2 * csig2 - 1.0;
          s2 = raa[a] <= 180.0 ? csig2_2 * ssig2 : -csig2_2 * ssig2;
        }
        double cum[3] = {0.0, 0.0, 0.0};
        double cumdb = 4.0 * G.mu0 * albedo * G.atten[L] * 1.0;
        for (int n = L; n >= 1; --n) {
          double f11 = 0.0, f12 = 0.0;
          for (int l = 0; l <= ngreek; ++l) f11 += p00[l] * GIN(l, n - 1, 0);
          if (NS > 1)
            for (int l = 0; l <= ngreek; ++l) f12 += p02[l] * GIN(l, n - 1, 1);
          double ex[3] = {f11, -f12 * c2, f12 * s2};
          cumdb = G.lostrans[n - 1] * cumdb;
          for (int s = 0; s < NS; ++s) {
            double source = (tms[n - 1] * ex[s]) * G.mult[n - 1];
            cum[s] = G.lostrans[n - 1] * cum[s] + source;
          }
        }
        for (int s = 0; s < NS; ++s) ss[s + NS * g] = flux * cum[s];
        db[0 + NS * g] = flux * cumdb;
      }
  }
  // ---------------------------------------------------------------- Fourier loop
  const bool do_dbcorr = o->do_focorr != 0;
  const bool msmode = o->do_focorr != 0;
  std::vector<double> stokes((size_t)NG * NS, 0.0);
  int testconv = 0;
  bool iterate = true;
  int fourier = -1;
  // generalized spherical functions: PI(l, i, s1, s2) for quadrature (0..N-1), user (N..N+nvza-1), solar
  const int NA = N + nvza + 1;
  auto PIX = [&](std::vector<double>& v, int l, int i, int s1, int s2) -> double& {
    return v[l + (size_t)NM1 * (i + (size_t)NA * (s1 + 4 * s2))];
  };
  std::vector<double> pimat((size_t)NM1 * NA * 16), xqp, xqp_pre, xqm_pre, xqm_post, xqm, xup, xup_pre, xum_post, xum,
      x0p;
  std::vector<double> xm(NA);
  for (int i = 0; i < N; ++i) xm[i] = qx[i];
  for (int u = 0; u < nvza; ++u) xm[N + u] = mu_u[u];
  xm[N + nvza] = cos_sza;
  std::vector<double> pimm11(NA, 0.0), pimmkm(NA, 0.0);
  // layer solutions
  std::vector<double> xpos((size_t)N2 * NS * NSN * L), xneg((size_t)N2 * NS * NSN * L), keig(NSN * L), teig(NSN * L),
      norm(NSN * L);
  auto XP = [&](int i, int s, int k, int n) -> double& { return xpos[i + N2 * (s + NS * (k + (size_t)NSN * n))]; };
  auto XN = [&](int i, int s, int k, int n) -> double& { return xneg[i + N2 * (s + NS * (k + (size_t)NSN * n))]; };
  std::vector<double> uhom_updn((size_t)nvza * NS * NSN * L), uhom_upup((size_t)nvza * NS * NSN * L);
  auto UDN = [&](int u, int s, int k, int n) -> double& { return uhom_updn[u + nvza * (s + NS * (k + (size_t)NSN * n))]; };
  auto UUP = [&](int u, int s, int k, int n) -> double& { return uhom_upup[u + nvza * (s + NS * (k + (size_t)NSN * n))]; };
  std::vector<double> hm1((size_t)nvza * NSN * L), hm2((size_t)nvza * NSN * L), zeta_m((size_t)nvza * NSN * L),
      zeta_p((size_t)nvza * NSN * L);
  std::vector<char> hsingo((size_t)nvza * NSN * L);
  std::vector<double> aterm(NSN * L), bterm(NSN * L), gam_p(NSN * L), gam_m(NSN * L);
  std::vector<double> wupper((size_t)N2 * NS * L), wlower((size_t)N2 * NS * L), upar1((size_t)nvza * NS * L);
  auto WU = [&](int i, int s, int n) -> double& { return wupper[i + N2 * (s + NS * n)]; };
  auto WL = [&](int i, int s, int n) -> double& { return wlower[i + N2 * (s + NS * n)]; };
  const int NT = NSN2 * L;
  const int KL = (L == 1) ? (2 * NSN - 1) : (3 * NSN - 1), KU = KL;
  const int LDAB = 2 * KL + KU + 1;
  std::vector<double> ab((size_t)LDAB * NT), col(NT);
  std::vector<int> ipiv(NT);
  std::vector<double> sab((size_t)NSN * NSN), dab((size_t)NSN * NSN), emat((size_t)NSN * NSN), evec((size_t)NSN * NSN),
      eval(NSN), wk(4 * NSN), esave((size_t)NSN * NSN);
  // SAB(i, j, o1, o2) at sab[(NS*i + o1) + NSN * (NS*j + o2)]
  auto SAB = [&](int i, int j, int o1, int o2) -> double& { return sab[(NS * i + o1) + (size_t)NSN * (NS * j + o2)]; };
  auto DAB = [&](int i, int j, int o1, int o2) -> double& { return dab[(NS * i + o1) + (size_t)NSN * (NS * j + o2)]; };
  // DO_NO_AZIMUTH (vlidort_inputs.f90:3953): scalar only, nadir-only view, no FO correction
  const int n_fouriers = (NS == 1 && nvza == 1 && vza[0] == 0.0 && !o->do_focorr) ? 0 : NM;
  while (iterate && fourier < n_fouriers) {
    fourier++;
    const int m = fourier;
    const bool incl_surface = (m == 0) && (albedo != 0.0);
    const double surface_factor = (m == 0) ? 2.0 : 1.0;
    const double delta_factor = (m == 0) ? 1.0 : 2.0;
    const double flux_multiplier = delta_factor;
    double direct_beam = 0.0;
    bool localbeam = incl_surface ? refl_directbeam : false;
    if (incl_surface && refl_directbeam) {
      double x0_flux = 4.0 * cos_sza / delta_factor;
      x0_flux = o->flux_factor * x0_flux / PI4;
      double attn = x0_flux * trans_solar_beam;
      direct_beam = attn * albedo;
    }
    // ---------------------------------------------- PIMATRIX_SETUP_OMP, miscsetups :2273-2935
    {
      std::fill(pimat.begin(), pimat.end(), 0.0);
      std::vector<double> phiv(NM1, 0.0), pinorm(NM1, 0.0);
      double fac = 1.0;
      for (int l = 1; l <= 2 * m; ++l) fac *= (double)l;
      phiv[m] = 1.0 / fac;
      for (int l = m + 1; l <= NM; ++l) phiv[l] = phiv[l - 1] * ((double)(l - m) / (double)(l + m));
      for (int l = m; l <= NM; ++l) pinorm[l] = std::sqrt(phiv[l]);
      const double rc20 = 0.25 * std::sqrt(6.0), rc21 = 2.0 * rc20;
      std::vector<double> xlm((size_t)NM1 * 4, 0.0), ylm((size_t)NM1 * 4, 0.0), zlm((size_t)NM1 * 16, 0.0);
      auto XL = [&](int l, int s) -> double& { return xlm[l + NM1 * s]; };
      auto YL = [&](int l, int s) -> double& { return ylm[l + NM1 * s]; };
      auto ZL = [&](int l, int s1, int s2) -> double& { return zlm[l + NM1 * (s1 + 4 * s2)]; };
      auto df_lsqm4 = [](int l) { return l >= 3 ? std::sqrt((double)(l * l - 4)) : 0.0; };
      auto df_rt = [](int l) { return std::sqrt((double)((l + 3) * (l - 1))); };
      if (m == 0) {
        for (int l = 2; l <= NM; ++l) {
          XL(l, 0) = (double)(l + 1); XL(l, 1) = df_rt(l); XL(l, 2) = XL(l, 1); XL(l, 3) = XL(l, 0);
          for (int s = 0; s < NS; ++s) XL(l, s) = 1.0 / XL(l, s);
          YL(l, 0) = (double)l; YL(l, 1) = df_lsqm4(l); YL(l, 2) = YL(l, 1); YL(l, 3) = YL(l, 0);
        }
      } else {
        for (int l = m; l <= NM; ++l) {
          double dlp1mm = (double)(l + 1 - m);
          XL(l, 0) = 1.0 / dlp1mm;
          if (l == 1) XL(l, 1) = 0.0;
          else XL(l, 1) = 1.0 / (df_rt(l) * dlp1mm / (double)(l + 1));
          XL(l, 2) = XL(l, 1); XL(l, 3) = XL(l, 0);
        }
        for (int s = 0; s < NS; ++s) YL(m, s) = 0.0;
        for (int l = m + 1; l <= NM; ++l) {
          double dlpm = (double)(l + m);
          YL(l, 0) = dlpm; YL(l, 1) = dlpm * df_lsqm4(l) / (double)l; YL(l, 2) = YL(l, 1); YL(l, 3) = YL(l, 0);
        }
        for (int l = 2; l <= NM; ++l) {
          double zhelp = 2.0 * (double)(2 * l + 1) / (double)(l + 1) / (double)l;
          double zv = (double)m * zhelp;
          ZL(l, 1, 2) = zv; ZL(l, 2, 1) = zv;
        }
      }
      for (int i = 0; i < NA; ++i) {
        const double x = xm[i], xsq = x * x;
        const double pleg20 = 0.5 * (3.0 * xsq - 1.0), umxsq = 1.0 - xsq;
        double rt_umxsq, x_rt_umxsq, upxsq_d_umxsq, m2x_d_umxsq;
        if (x == 1.0) { rt_umxsq = 0.0; x_rt_umxsq = 0.0; upxsq_d_umxsq = 0.0; m2x_d_umxsq = 0.0; }
        else {
          rt_umxsq = std::sqrt(umxsq); x_rt_umxsq = rt_umxsq * x;
          upxsq_d_umxsq = (1.0 + xsq) / umxsq; m2x_d_umxsq = -2.0 * x / umxsq;
        }
        auto P = [&](int l, int s1, int s2) -> double& { return PIX(pimat, l, i, s1, s2); };
        auto x2lp1 = [&](int l) { return x * (double)(2 * l + 1); };
        if (m == 0) {
          P(0, 0, 0) += 1.0; if (NS == 4) P(0, 3, 3) += 1.0;
          if (NM >= 1) { P(1, 0, 0) += x; if (NS == 4) P(1, 3, 3) += x; }
          if (NM >= 2) {
            P(2, 0, 0) += pleg20;
            if (NS > 1) { P(2, 1, 1) += rc20 * umxsq; P(2, 2, 2) = P(2, 1, 1); }
          }
          for (int l = 2; l <= NM - 1; ++l)
            for (int s1 = 0; s1 < NS; ++s1)
              for (int s2 = 0; s2 < NS; ++s2) {
                double hx = x2lp1(l) * P(l, s1, s2), hy = YL(l, s1) * P(l - 1, s1, s2);
                P(l + 1, s1, s2) = (hx - hy) * XL(l, s1);
              }
        } else if (m == 1) {
          P(1, 0, 0) += rt_umxsq;
          if (NM >= 2) {
            P(2, 0, 0) += 3.0 * x_rt_umxsq;
            if (NS > 1) {
              P(2, 1, 1) += -rc21 * x_rt_umxsq;
              P(2, 1, 2) += rc21 * rt_umxsq;
              P(2, 2, 2) = P(2, 1, 1);
              P(2, 2, 1) = P(2, 1, 2);
            }
          }
          for (int l = 2; l <= NM - 1; ++l)
            for (int s1 = 0; s1 < NS; ++s1)
              for (int s2 = 0; s2 < NS; ++s2) {
                double hx = x2lp1(l) * P(l, s1, s2), hy = YL(l, s1) * P(l - 1, s1, s2), hz = 0.0;
                for (int s3 = 0; s3 < NS; ++s3) hz += ZL(l, s1, s3) * P(l, s3, s2);
                P(l + 1, s1, s2) = (hx - hy + hz) * XL(l, s1);
              }
        } else {
          if (m == 2) {
            pimm11[i] = 3.0 * umxsq;
            pimmkm[i] = (x == 1.0) ? rc21 : rc21 * umxsq;
          } else {
            double h1 = (double)(2 * (m - 1) + 1);
            double h2 = (double)m * h1 / df_rt(m - 1);
            pimm11[i] = h1 * rt_umxsq * pimm11[i];
            pimmkm[i] = (x == 1.0) ? 0.0 : h2 * rt_umxsq * pimmkm[i];
          }
          P(m, 0, 0) += pimm11[i];
          if (NS > 1) {
            if (x == 1.0) { P(m, 1, 1) += pimmkm[i] * 2.0; P(m, 1, 2) -= pimmkm[i] * 2.0; }
            else { P(m, 1, 1) += pimmkm[i] * upxsq_d_umxsq; P(m, 1, 2) += pimmkm[i] * m2x_d_umxsq; }
            P(m, 2, 2) = P(m, 1, 1);
            P(m, 2, 1) = P(m, 1, 2);
          }
          if (m < NM)
            for (int s1 = 0; s1 < NS; ++s1)
              for (int s2 = 0; s2 < NS; ++s2) {
                double hx = x2lp1(m) * P(m, s1, s2), hz = 0.0;
                for (int s3 = 0; s3 < NS; ++s3) hz += ZL(m, s1, s3) * P(m, s3, s2);
                P(m + 1, s1, s2) = (hx + hz) * XL(m, s1);
              }
          for (int l = m + 1; l <= NM - 1; ++l)
            for (int s1 = 0; s1 < NS; ++s1)
              for (int s2 = 0; s2 < NS; ++s2) {
                double hx = x2lp1(l) * P(l, s1, s2), hy = YL(l, s1) * P(l - 1, s1, s2), hz = 0.0;
                for (int s3 = 0; s3 < NS; ++s3) hz += ZL(l, s1, s3) * P(l, s3, s2);
                P(l + 1, s1, s2) = (hx - hy + hz) * XL(l, s1);
              }
        }
      }
      // normalised outputs and their D-matrix products (only l >= m is used)
      xqp.assign(pimat.size(), 0.0); xqp_pre.assign(pimat.size(), 0.0); xqm_pre.assign(pimat.size(), 0.0);
      xqm_post.assign(pimat.size(), 0.0); xqm.assign(pimat.size(), 0.0);
      xup.assign(pimat.size(), 0.0); xup_pre.assign(pimat.size(), 0.0); xum_post.assign(pimat.size(), 0.0);
      xum.assign(pimat.size(), 0.0); x0p.assign(pimat.size(), 0.0);
      for (int l = m; l <= NM; ++l) {
        const double sgn = ((l - m) % 2 == 0) ? 1.0 : -1.0;
        for (int i = 0; i < NA; ++i)
          for (int s1 = 0; s1 < NS; ++s1)
            for (int s2 = 0; s2 < NS; ++s2) PIX(xqp, l, i, s1, s2) = PIX(pimat, l, i, s1, s2) * pinorm[l];
        for (int i = 0; i < NA; ++i)
          for (int s1 = 0; s1 < NS; ++s1)
            for (int s2 = 0; s2 < NS; ++s2) {
              double p = PIX(xqp, l, i, s1, s2);
              double pre = dmat(s1) * p, post = p * dmat(s2), both = dmat(s1) * (p * dmat(s2));
              if (i < N) {
                PIX(xqp_pre, l, i, s1, s2) = pre;
                PIX(xqm_pre, l, i, s1, s2) = pre * sgn;
                PIX(xqm_post, l, i, s1, s2) = post * sgn;
                PIX(xqm, l, i, s1, s2) = both * sgn;
              } else if (i < N + nvza) {
                PIX(xup, l, i, s1, s2) = p;
                PIX(xup_pre, l, i, s1, s2) = pre;
                PIX(xum_post, l, i, s1, s2) = post * sgn;
                PIX(xum, l, i, s1, s2) = both * sgn;
              } else {
                PIX(x0p, l, i, s1, s2) = p;
              }
            }
      }
    }
    const int I0 = N + nvza;  // solar index in the PI arrays
    // ---------------------------------------------- homogeneous solutions per layer
    for (int n = 0; n < L; ++n) {
      // QHOM_SOLUTION, solutions.f90:150-1050 (sum and difference matrices :436-476, eigenmatrix :484-496)
      std::vector<double> h2p((size_t)NS * NM1 * NS * N), h2m((size_t)NS * NM1 * NS * N);
      auto H2P = [&](int o3, int l, int o2, int j) -> double& { return h2p[o3 + NS * (l + NM1 * (o2 + NS * j))]; };
      auto H2M = [&](int o3, int l, int o2, int j) -> double& { return h2m[o3 + NS * (l + NM1 * (o2 + NS * j))]; };
      for (int j = 0; j < N; ++j)
        for (int o2 = 0; o2 < NS; ++o2)
          for (int l = m; l <= NM; ++l)
            for (int o3 = 0; o3 < NS; ++o3) {
              double sp = 0.0, sm = 0.0;
              for (int s = 0; s < NS; ++s) {
                sp += OG(l, n, o3, s) * PIX(xqp, l, j, s, o2);
                sm += OG(l, n, o3, s) * PIX(xqm_pre, l, j, s, o2);
              }
              H2P(o3, l, o2, j) = sp;
              H2M(o3, l, o2, j) = sm;
            }
      for (int i = 0; i < N; ++i) {
        double xinv = -1.0 / qx[i];
        for (int j = 0; j < N; ++j) {
          double f = xinv * halfwts[j];
          for (int o1 = 0; o1 < NS; ++o1)
            for (int o2 = 0; o2 < NS; ++o2) {
              double dp = 0.0, dm = 0.0;
              for (int l = m; l <= NM; ++l) {
                double sp = 0.0, sm = 0.0;
                for (int s = 0; s < NS; ++s) {
                  sp += PIX(xqp, l, i, o1, s) * H2P(s, l, o2, j);
                  sm += PIX(xqp, l, i, o1, s) * H2M(s, l, o2, j);
                }
                dp += sp; dm += sm;
              }
              SAB(i, j, o1, o2) = f * (dp + dm);
              DAB(i, j, o1, o2) = f * (dp - dm);
            }
        }
        for (int o1 = 0; o1 < NS; ++o1) { SAB(i, i, o1, o1) -= xinv; DAB(i, i, o1, o1) -= xinv; }
      }
      for (int r = 0; r < NSN; ++r)
        for (int c = 0; c < NSN; ++c) {
          double s = 0.0;
          for (int k = 0; k < NSN; ++k) s += dab[r + (size_t)NSN * k] * sab[k + (size_t)NSN * c];
          emat[r + (size_t)NSN * c] = s;
        }
      esave = emat;
      bool bad;
      int ier = asymtx(o->asymtx_tol, emat.data(), NSN, NSN, evec.data(), eval.data(), wk.data(), &bad);
      if (bad) return ORC_EIGEN_FAIL;
      if (ier > 0) {
        emat = esave;
        ier = asymtx(1.0e-10, emat.data(), NSN, NSN, evec.data(), eval.data(), wk.data(), &bad);
        if (ier > 0) {
          emat = esave;
          ier = asymtx(1.0e-8, emat.data(), NSN, NSN, evec.data(), eval.data(), wk.data(), &bad);
          if (ier > 0 || bad) return ORC_EIGEN_FAIL;
        }
      }
      for (int a = 0; a < NSN; ++a) {
        double s = 0.0;
        for (int r = 0; r < NSN; ++r) s += evec[r + (size_t)NSN * a] * evec[r + (size_t)NSN * a];
        s = std::sqrt(s);
        for (int r = 0; r < NSN; ++r) evec[r + (size_t)NSN * a] /= s;
      }
      for (int k = 0; k < NSN; ++k) {
        if (!(eval[k] > 0.0)) return ORC_EIGEN_FAIL;
        double kv = std::sqrt(eval[k]);
        keig[k + NSN * n] = kv;
        double sc = 1.0 / kv;
        double nr = 0.0;
        for (int r = 0; r < NSN; ++r) nr += evec[r + (size_t)NSN * k] * evec[r + (size_t)NSN * k];
        nr = std::sqrt(nr);
        std::vector<double> sumv(NSN), difv(NSN);
        for (int r = 0; r < NSN; ++r) sumv[r] = evec[r + (size_t)NSN * k] / nr;  // (NS*i + o)
        for (int i = 0; i < N; ++i)
          for (int o1 = 0; o1 < NS; ++o1) {
            double h = 0.0;
            for (int j = 0; j < N; ++j)
              for (int s = 0; s < NS; ++s) h += SAB(i, j, o1, s) * sumv[NS * j + s];
            difv[NS * i + o1] = h * sc;
          }
        for (int i = 0; i < N; ++i)
          for (int s = 0; s < NS; ++s) {
            double fpd = 0.5 * (sumv[NS * i + s] + difv[NS * i + s]);
            double fnd = 0.5 * (sumv[NS * i + s] - difv[NS * i + s]);
            XP(i, s, k, n) = fpd;
            XN(i, s, k, n) = fnd;
            XP(i + N, s, k, n) = s < 2 ? fnd : -fnd;
            XN(i + N, s, k, n) = s < 2 ? fpd : -fpd;
          }
        double help = kv * dtau[n];
        teig[k + NSN * n] = help > MAX_TAU_QPATH ? 0.0 : std::exp(-help);
      }
      // UHOM_SOLUTION, solutions.f90:1167-1508 (upwelling user streams)
      for (int u = 0; u < nvza; ++u)
        for (int k = 0; k < NSN; ++k) {
          size_t idx = u + nvza * (k + (size_t)NSN * n);
          double rho_p = sec_u[u] + keig[k + NSN * n];
          double rho_m = sec_u[u] - keig[k + NSN * n];
          zeta_p[idx] = 1.0 / rho_p;
          hsingo[idx] = std::fabs(rho_m) < TAYLOR_SMALL;
          zeta_m[idx] = hsingo[idx] ? rho_m : 1.0 / rho_m;
        }
      const bool lsc = laysc[m + (NM + 1) * n];
      std::vector<double> helps((size_t)NM1 * NS), gaux((size_t)NM1 * NS);
      for (int k = 0; k < NSN; ++k) {
        for (int l = m; l <= NM; ++l) {
          for (int o1 = 0; o1 < NS; ++o1) {
            double sps = 0.0;
            for (int j = 0; j < N; ++j) {
              double a5 = halfwts[j], sp = 0.0, sm = 0.0;
              for (int s = 0; s < NS; ++s) {
                sp += PIX(xqp, l, j, o1, s) * a5 * XP(j, s, k, n);
                sm += PIX(xqm_pre, l, j, o1, s) * a5 * XN(j, s, k, n);
              }
              sps = sps + sp + sm;
            }
            helps[l + NM1 * o1] = sps;
          }
          for (int o1 = 0; o1 < NS; ++o1) {
            double g = 0.0;
            for (int s = 0; s < NS; ++s) g += OG(l, n, o1, s) * helps[l + NM1 * s];
            gaux[l + NM1 * o1] = g;
          }
        }
        for (int o1 = 0; o1 < NS; ++o1)
          for (int u = 0; u < nvza; ++u) {
            double dn = 0.0, up = 0.0;
            for (int l = m; l <= NM; ++l)
              for (int s = 0; s < NS; ++s) {
                dn += PIX(xum, l, N + u, o1, s) * gaux[l + NM1 * s];
                up += PIX(xup_pre, l, N + u, o1, s) * gaux[l + NM1 * s];
              }
            UDN(u, o1, k, n) = lsc ? dn : 0.0;
            UUP(u, o1, k, n) = lsc ? up : 0.0;
          }
      }
      // QHOM_NORMS :1051-1165
      for (int k = 0; k < NSN; ++k) {
        double s = 0.0;
        for (int j = 0; j < N; ++j) {
          double t1 = 0.0, t2 = 0.0;
          for (int o1 = 0; o1 < NS; ++o1) {
            t1 += XP(j, o1, k, n) * XP(j, o1, k, n);
            t2 += XN(j, o1, k, n) * XN(j, o1, k, n);
          }
          s += strmwts[j] * (t1 - t2);
        }
        norm[k + NSN * n] = s;
      }
      // HMULT (whole layer) :1651
      for (int u = 0; u < nvza; ++u) {
        double udel = t_user[n + L * u], smu = sec_u[u];
        for (int k = 0; k < NSN; ++k) {
          size_t idx = u + nvza * (k + (size_t)NSN * n);
          double zdel = teig[k + NSN * n], zudel = zdel * udel;
          double th2 = 1.0 - zudel, th1 = zdel - udel;
          if (hsingo[idx]) hm1[idx] = taylor1(order, zeta_m[idx], dtau[n], udel, smu);
          else hm1[idx] = smu * th1 * zeta_m[idx];
          hm2[idx] = smu * th2 * zeta_p[idx];
        }
      }
    }
    // ---------------------------------------------- BVP matrix (bvproblem.f90:627-1178) + LU (:1180)
    std::fill(ab.begin(), ab.end(), 0.0);
    auto AB = [&](int i, int j) -> double& { return ab[(KL + KU + i - j) + (size_t)LDAB * j]; };
    const double kmult = incl_surface ? surface_factor * albedo : 0.0;
    {
      for (int i = 0; i < N; ++i)
        for (int s = 0; s < NS; ++s) {
          int r = NS * i + s;
          for (int k = 0; k < NSN; ++k) {
            AB(r, k) = XP(i, s, k, 0);
            AB(r, k + NSN) = XN(i, s, k, 0) * teig[k];
          }
        }
      for (int n = 1; n < L; ++n) {
        int c0 = n * NSN2 - NSN;
        int ce = c0 - NSN;
        for (int i = 0; i < N2; ++i)
          for (int s = 0; s < NS; ++s) {
            int cm = c0 + NS * i + s;
            for (int k = 0; k < NSN; ++k) {
              AB(cm, ce + k) = teig[k + NSN * (n - 1)] * XP(i, s, k, n - 1);
              AB(cm, ce + k + NSN) = XN(i, s, k, n - 1);
              AB(cm, ce + k + NSN2) = -XP(i, s, k, n);
              AB(cm, ce + k + NSN + NSN2) = -teig[k + NSN * n] * XN(i, s, k, n);
            }
          }
      }
      int c0 = NSN2 * L - NSN, ce = NSN2 * (L - 1);
      std::vector<double> r2p(NSN, 0.0), r2m(NSN, 0.0);  // BVP_SURFACE_SETUP_HOM :439 (Lambertian: I only)
      if (incl_surface)
        for (int k = 0; k < NSN; ++k) {
          double sp = 0.0, sm = 0.0;
          for (int j = 0; j < N; ++j) { sp += strmwts[j] * XP(j, 0, k, L - 1); sm += strmwts[j] * XN(j, 0, k, L - 1); }
          r2p[k] = sp * kmult; r2m[k] = sm * kmult;
        }
      for (int i = 0; i < N; ++i)
        for (int s = 0; s < NS; ++s) {
          int r = c0 + NS * i + s;
          for (int k = 0; k < NSN; ++k) {
            double xpnet = XP(i + N, s, k, L - 1) - (s == 0 ? r2p[k] : 0.0);
            double xmnet = XN(i + N, s, k, L - 1) - (s == 0 ? r2m[k] : 0.0);
            AB(r, ce + k) = teig[k + NSN * (L - 1)] * xpnet;
            AB(r, ce + k + NSN) = xmnet;
          }
        }
    }
    if (band_lu(NT, KL, KU, ab.data(), LDAB, ipiv.data()) != 0) return ORC_BVP_SINGULAR;
    // ---------------------------------------------- beam particular solutions (Green's function)
    const double F1 = o->flux_factor / PI4;
    for (int n = 0; n < L; ++n) {
      bool active = (n + 1 <= cutoff) && laysc[m + (NM + 1) * n];
      for (int i = 0; i < N2; ++i)
        for (int s = 0; s < NS; ++s) { WU(i, s, n) = 0.0; WL(i, s, n) = 0.0; }
      for (int u = 0; u < nvza; ++u)
        for (int s = 0; s < NS; ++s) upar1[u + nvza * (s + NS * n)] = 0.0;
      if (!active) continue;
      // GBEAM_SOLUTION :2649-2935
      double secbar = avsec[n], cnst = itrans[n], wdel = t_mubar[n];
      std::vector<double> cfunc(NSN), dfunc(NSN);
      for (int k = 0; k < NSN; ++k) {
        double zdel = teig[k + NSN * n], zwdel = zdel * wdel;
        gam_p[k + NSN * n] = secbar + keig[k + NSN * n];
        gam_m[k + NSN * n] = secbar - keig[k + NSN * n];
        double eps = gam_m[k + NSN * n];
        if (std::fabs(eps) < TAYLOR_SMALL) cfunc[k] = taylor1(order, eps, dtau[n], wdel, cnst);
        else cfunc[k] = cnst * (zdel - wdel) / gam_m[k + NSN * n];
        dfunc[k] = cnst * (1.0 - zwdel) / gam_p[k + NSN * n];
      }
      std::vector<double> hq((size_t)NM1 * NS, 0.0);  // HELP_QFUNC(l, o1), DFLUX = (1, 0, 0)
      for (int o1 = 0; o1 < NS; ++o1)
        for (int l = m; l <= NM; ++l) {
          double gsum = 0.0;
          for (int o2 = 0; o2 < NS; ++o2) gsum += OG(l, n, o1, o2) * (PIX(x0p, l, I0, o2, 0) * 1.0);
          hq[l + NM1 * o1] = gsum;
        }
      std::vector<double> dpi((size_t)N * NS), dmi((size_t)N * NS);
      for (int o1 = 0; o1 < NS; ++o1)
        for (int i = 0; i < N; ++i) {
          double sp = 0.0, sm = 0.0;
          for (int l = m; l <= NM; ++l)
            for (int s = 0; s < NS; ++s) {
              sp += PIX(xqp, l, i, o1, s) * hq[l + NM1 * s];
              sm += PIX(xqm_post, l, i, o1, s) * hq[l + NM1 * s];
            }
          dpi[i + N * o1] = F1 * sp; dmi[i + N * o1] = F1 * sm;
        }
      std::vector<double> gdn(NSN), gup(NSN);
      for (int k = 0; k < NSN; ++k) {
        double s1 = 0.0, s2 = 0.0;
        for (int i = 0; i < N; ++i) {
          double h1 = 0.0, h2 = 0.0, h3 = 0.0, h4 = 0.0;
          for (int s = 0; s < NS; ++s) {
            h1 += dpi[i + N * s] * XP(i, s, k, n); h2 += dmi[i + N * s] * XN(i, s, k, n);
            h3 += dmi[i + N * s] * XP(i, s, k, n); h4 += dpi[i + N * s] * XN(i, s, k, n);
          }
          s1 += qw[i] * (h1 + h2); s2 += qw[i] * (h3 + h4);
        }
        aterm[k + NSN * n] = s1 / norm[k + NSN * n];
        bterm[k + NSN * n] = s2 / norm[k + NSN * n];
        gdn[k] = cfunc[k] * aterm[k + NSN * n];
        gup[k] = dfunc[k] * bterm[k + NSN * n];
      }
      for (int s = 0; s < NS; ++s)
        for (int i = 0; i < N; ++i) {
          double wu1 = 0, wu2 = 0, wl1 = 0, wl2 = 0;
          for (int k = 0; k < NSN; ++k) {
            wu1 += gup[k] * XN(i, s, k, n); wu2 += gup[k] * XP(i, s, k, n);
            wl1 += gdn[k] * XN(i, s, k, n); wl2 += gdn[k] * XP(i, s, k, n);
          }
          WU(i, s, n) = wu1; WU(i + N, s, n) = s >= 2 ? -wu2 : wu2;
          WL(i + N, s, n) = s >= 2 ? -wl1 : wl1; WL(i, s, n) = wl2;
        }
      // GUSER_SOLUTION :2936-3073 (used only without the FO correction)
      for (int o1 = 0; o1 < NS; ++o1)
        for (int u = 0; u < nvza; ++u) {
          double sv = 0.0;
          for (int l = m; l <= NM; ++l)
            for (int s = 0; s < NS; ++s) sv += (F1 * hq[l + NM1 * s]) * PIX(xum, l, N + u, o1, s);
          upar1[u + nvza * (o1 + NS * n)] = sv;
        }
    }
    // BVP column (bvproblem.f90:1743) and back substitution
    std::fill(col.begin(), col.end(), 0.0);
    for (int i = 0; i < N; ++i)
      for (int s = 0; s < NS; ++s) col[NS * i + s] = -WU(i, s, 0);
    for (int n = 1; n < L; ++n) {
      int c0 = n * NSN2 - NSN;
      for (int i = 0; i < N2; ++i)
        for (int s = 0; s < NS; ++s) col[c0 + NS * i + s] = WU(i, s, n) - WL(i, s, n - 1);
    }
    {
      int c0 = (L - 1) * NSN2 + NSN;
      double r2b = 0.0;
      if (incl_surface) {
        for (int j = 0; j < N; ++j) r2b += strmwts[j] * WL(j, 0, L - 1);
        r2b = r2b * kmult;
      }
      for (int i = 0; i < N; ++i)
        for (int s = 0; s < NS; ++s) {
          double v = -WL(i + N, s, L - 1);
          if (s == 0 && incl_surface) v += r2b;
          if (s == 0 && localbeam && incl_surface) v += direct_beam;
          col[c0 + NS * i + s] = v;
        }
    }
    band_solve(NT, KL, KU, ab.data(), LDAB, ipiv.data(), col.data());
    auto LCON = [&](int k, int n) { return col[n * NSN2 + k]; };
    auto MCON = [&](int k, int n) { return col[n * NSN2 + NSN + k]; };
    // ---------------------------------------------- UPUSER_INTENSITY (intensity.f90:145), TOA only
    std::vector<double> stokes_f((size_t)nvza * NS, 0.0);
    {
      const bool incl_directrf = (localbeam && !do_dbcorr) && !msmode;
      double reflec = 0.0;  // GET_BOA_SOURCE :1096 (Lambertian: I only)
      if (incl_surface) {
        double s = 0.0;
        for (int i = 0; i < N; ++i) {
          double shom = 0.0;
          for (int k = 0; k < NSN; ++k) {
            double lxr = LCON(k, L - 1) * XP(i, 0, k, L - 1);
            double mxr = MCON(k, L - 1) * XN(i, 0, k, L - 1);
            shom = shom + lxr * teig[k + NSN * (L - 1)] + mxr;
          }
          s += strmwts[i] * (WL(i, 0, L - 1) + shom);
        }
        reflec = kmult * s;
      }
      for (int u = 0; u < nvza; ++u) {
        double cum[3] = {0.0, 0.0, 0.0};
        if (incl_surface) cum[0] = reflec;
        if (incl_surface && incl_directrf && !do_dbcorr) cum[0] += direct_beam;
        for (int n = L - 1; n >= 0; --n) {
          double src[3] = {0.0, 0.0, 0.0};
          if (laysc[m + (NM + 1) * n]) {  // WHOLELAYER_STERM_UP, PostProcessing.f90:139
            for (int o1 = 0; o1 < NS; ++o1) {
              double h = 0.0;
              for (int k = 0; k < NSN; ++k) {
                size_t idx = u + nvza * (k + (size_t)NSN * n);
                double luxr = LCON(k, n) * UDN(u, o1, k, n);
                double muxr = MCON(k, n) * UUP(u, o1, k, n);
                h = h + luxr * hm2[idx] + muxr * hm1[idx];
              }
              src[o1] = h;
            }
            if (n + 1 <= cutoff) {
              double wdel = t_mubar[n], it = itrans[n], itw = -it * wdel;
              double spar[3] = {0.0, 0.0, 0.0};
              double em = emult_up[n + L * u];
              for (int k = 0; k < NSN; ++k) {
                size_t idx = u + nvza * (k + (size_t)NSN * n);
                double sd;
                if (std::fabs(gam_m[k + NSN * n]) < TAYLOR_SMALL) {
                  double mult = taylor2(order, gam_m[k + NSN * n], sigma_p[n + L * u], dtau[n], 1.0,
                                        wdel * t_user[n + L * u], 1.0);
                  sd = itrans_u[n + L * u] * mult;
                } else {
                  sd = (it * hm2[idx] - em) / gam_m[k + NSN * n];
                }
                double su = (itw * hm1[idx] + em) / gam_p[k + NSN * n];
                for (int o1 = 0; o1 < NS; ++o1)
                  spar[o1] = spar[o1] + UDN(u, o1, k, n) * sd * aterm[k + NSN * n] +
                             UUP(u, o1, k, n) * su * bterm[k + NSN * n];
              }
              for (int o1 = 0; o1 < NS; ++o1) {
                src[o1] += spar[o1];
                if (!msmode) src[o1] += upar1[u + nvza * (o1 + NS * n)] * em;
              }
            }
          }
          for (int o1 = 0; o1 < NS; ++o1) cum[o1] = src[o1] + t_user[n + L * u] * cum[o1];
        }
        for (int o1 = 0; o1 < NS; ++o1) stokes_f[u + nvza * o1] = flux_multiplier * cum[o1];
      }
    }
    // ---------------------------------------------- convergence (converge.f90:128-538, AZMFAC masters :2608)
    if (m == 0) {
      for (int u = 0; u < nvza; ++u)
        for (int a = 0; a < nraa; ++a) {
          int g = a + nraa * u;
          for (int s = 0; s < NS; ++s) {
            double v = stokes_f[u + nvza * s];
            if (o->do_focorr) v += ss[s + NS * g];
            if (o->do_focorr || do_dbcorr) v += db[s + NS * g];
            stokes[s + NS * g] = v;
          }
        }
    } else {
      int count = 0;
      for (int a = 0; a < nraa; ++a)
        for (int u = 0; u < nvza; ++u) {
          int g = a + nraa * u;
          double arg = raa[a] * (double)m * DTR;
          double cz = std::cos(arg), sz = std::sin(arg);
          double tazm0 = 0.0, tnew0 = 0.0;
          for (int s = 0; s < NS; ++s) {
            double azmfac = s < 2 ? cz : sz;
            double told = stokes[s + NS * g], tazm = azmfac * stokes_f[u + nvza * s], tnew = told + tazm;
            if (s == 0) { tazm0 = tazm; tnew0 = tnew; }
            stokes[s + NS * g] = tnew;
          }
          if (tazm0 != 0.0) {
            if (std::fabs(tazm0 / tnew0) < o->accuracy) count++;
          } else {
            count++;
          }
        }
      if (count == NG) {
        testconv++;
        if (o->do_double_convtest) { if (testconv == 2) iterate = false; }
        else iterate = false;
      } else {
        testconv = 0;
      }
    }
  }
  for (int g = 0; g < NG; ++g)
    for (int s = 0; s < NS; ++s) out[s + NS * g] = stokes[s + NS * g];
  if (nfourier_out) *nfourier_out = fourier;
  return ORC_OK;
}

}  // extern "C"

// ------------------------------------------------------------------------------------------
// The AeroApps glue: VLIDORT_Vector_Lambert (geo_vlidort/VLIDORT_LAMBERT.F90:172-342)
// calling VLIDORT_Init (VLIDORT2p8p3/VLIDORT_Mod.F90:65-383) and
// VLIDORT_Run_Vector_SingleGeom (VLIDORT2p8p3/VLIDORT_ScatMod.F90:284-617) per
// (observation, channel), NSTOKES = 3.  Arrays are Fortran column-major exactly
// as the reference declares them; pmom(km,nch,nobs,nMom,6) holds P11, P12,
// P33, P34, P22, P44.  alpha (km,nobs,nch) may be NULL (no gas absorption),
// flux_factor (nch,nobs) may be NULL (1).  A pixel with MISSING angles or
// albedo gets MISSING in all four outputs.  nfourier/status/nlay optional.
extern "C" double oracle_get_asymtx_tol();
extern "C" int oracle_vector_lambert(int km, int nch, int nobs, int nstreams, int plane_parallel, int nMom,
                                     const double* ROT, const double* depol, const double* alpha, const double* tau,
                                     const double* ssa, const double* pmom, const double* he, const double* albedo,
                                     const double* solar_zenith, const double* relat_azymuth,
                                     const double* sensor_zenith, const double* flux_factor, double MISSING,
                                     double* radiance, double* reflectance, double* Q, double* U, int* nfourier,
                                     int* status, const int* nlay) {
  if (km > 72) return 3;
  if (nMom > 1000) return 5;
  auto is_missing = [&](double x) { return std::fabs(x / MISSING - 1.0) < 0.001; };
  std::vector<char> nadir(nobs, 0);  // sticky DO_FOCORR_NADIR (VLIDORT_ScatMod.F90:395-398)
  {
    bool flag = false;
    for (int j = 0; j < nobs; ++j) {
      bool geo_ok = !(is_missing(solar_zenith[j]) || is_missing(sensor_zenith[j]) || is_missing(relat_azymuth[j]));
      if (geo_ok && solar_zenith[j] == 0.0) {
        for (int i = 0; i < nch; ++i)
          if (!is_missing(albedo[j + nobs * i])) { flag = true; break; }
      }
      nadir[j] = flag;
    }
  }
  const double pi_sp = (double)(4.0f * std::atan(1.0f));
  const double height_scale = (double)1.0e-3f;
  const double ssa_cap = (double)0.99999f;
  const size_t nk = (size_t)km * nch * nobs;
#pragma omp parallel for schedule(dynamic, 1)
  for (int p = 0; p < nobs * nch; ++p) {
    int j = p / nch, i = p % nch;
    size_t o = (size_t)j + (size_t)nobs * i;
    if (nfourier) nfourier[o] = -1;
    if (status) status[o] = 0;
    if (is_missing(solar_zenith[j]) || is_missing(sensor_zenith[j]) || is_missing(relat_azymuth[j]) ||
        is_missing(albedo[o])) {
      radiance[o] = MISSING; reflectance[o] = MISSING; Q[o] = MISSING; U[o] = MISSING;
      continue;
    }
    const int L = nlay ? nlay[j] : km;
    const int G1 = nMom + 1;
    std::vector<double> dt(L), om(L), gr((size_t)G1 * L * 16, 0.0), hg(L + 1);
    const double dep = depol[i];
    // Rayleigh Greek moments (VLIDORT_ScatMod.F90:446-480; SQRT(6.) is REAL*4)
    const double gammamom2 = -(double)std::sqrt(6.0f) * (1.0 - dep) / (2.0 + dep);
    const double alphamom2 = 6.0 * (1.0 - dep) / (2.0 + dep);
    const double deltamom1 = 3.0 * (1.0 - 2.0 * dep) / (2.0 + dep);
    const double raysmom2 = (1.0 - dep) / (2.0 + dep);
    double ray[3][16] = {};
    ray[0][0] = 1.0; ray[2][0] = raysmom2; ray[2][1] = gammamom2; ray[2][4] = gammamom2; ray[2][5] = alphamom2;
    ray[1][15] = deltamom1;
    for (int k = 0; k < L; ++k) {
      double ray_l = ROT[k + (size_t)km * (j + (size_t)nobs * i)];
      double alpha_l = alpha ? alpha[k + (size_t)km * (j + (size_t)nobs * i)] : 0.0;
      size_t a = k + (size_t)km * (i + (size_t)nch * j);
      double tau_l = tau[a], ssa_l = ssa[a];
      double tau_ext = alpha_l + ray_l + tau_l;
      double tau_scat = ray_l + ssa_l * tau_l;
      double ssa_tot = tau_scat / tau_ext;
      if (ssa_tot > ssa_cap) ssa_tot = ssa_cap;
      dt[k] = tau_ext; om[k] = ssa_tot;
      double aerswt = ssa_l * tau_l / tau_scat;
      double rayswt = ray_l / tau_scat;
      auto aer = [&](int l, int ent) -> double {  // aervmoms(l, k, ent): entries from pmom(:, :, 1..6)
        if (l >= nMom) return 0.0;
        auto pm = [&](int ip) { return pmom[a + nk * ((size_t)l + (size_t)nMom * ip)]; };
        switch (ent) {
          case 0: return pm(0);
          case 1: case 4: return pm(1);
          case 10: return pm(2);
          case 11: return pm(3);
          case 14: return -pm(3);
          case 5: return pm(4);
          case 15: return pm(5);
        }
        return 0.0;
      };
      for (int ent = 0; ent < 16; ++ent) {
        for (int l = 0; l <= 2 && l <= nMom; ++l)
          gr[l + G1 * (k + (size_t)L * ent)] = ray[l][ent] * rayswt + aer(l, ent) * aerswt;
        for (int l = 3; l <= nMom; ++l) gr[l + G1 * (k + (size_t)L * ent)] = aer(l, ent) * aerswt;
      }
      gr[0 + G1 * (k + (size_t)L * 0)] = 1.0;
    }
    for (int k = 0; k <= L; ++k) hg[k] = he[k + (size_t)(km + 1) * j] * height_scale;
    OracleOpts op;
    op.do_focorr = 1;
    op.do_focorr_nadir = nadir[j] ? 1 : 0;
    op.do_focorr_outgoing = nadir[j] ? 0 : 1;
    op.do_deltam = 1;
    op.do_plane_parallel = plane_parallel;
    op.do_double_convtest = 1;
    op.nfinelayers = 3;
    op.taylor_order = 3;
    op.accuracy = (double)0.0001f;
    op.asymtx_tol = oracle_get_asymtx_tol();
    op.earth_radius = 6371.0;
    op.flux_factor = flux_factor ? flux_factor[i + (size_t)nch * j] : 1.0;
    double sza = solar_zenith[j], vz = sensor_zenith[j], az = relat_azymuth[j], res[3] = {0.0, 0.0, 0.0};
    int nf = -1;
    int rc = oracle_vlidort_vector_solve(&op, 3, L, nstreams, nMom, hg.data(), dt.data(), om.data(), gr.data(),
                                         albedo[o], sza, 1, &vz, 1, &az, res, &nf);
    if (nfourier) nfourier[o] = nf;
    if (status) status[o] = rc;
    if (rc != 0) { radiance[o] = MISSING; reflectance[o] = MISSING; Q[o] = MISSING; U[o] = MISSING; continue; }
    radiance[o] = res[0]; Q[o] = res[1]; U[o] = res[2];
    reflectance[o] = (pi_sp * res[0]) / (std::cos(sza * pi_sp / 180.0) * op.flux_factor);
  }
  return 0;
}
