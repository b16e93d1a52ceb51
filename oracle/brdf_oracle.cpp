// Test infrastructure only: the CPU oracle for the BRDF supplement of VLIDORT
// 2.8.3 (VBRDF, NSTOKES = 1), the surface that AeroApps' land path uses
// (VLIDORT_Scalar_LandMODIS, geo_vlidort/VLIDORT_BRDF_MODIS.F90:34-200, with
// the kernels set by VLIDORT_LANDMODIS_SingleGeom,
// RTSI/VLIDORT2p8p3/VLIDORT_SurfaceMod.F90:1376-1596: Lambertian (fiso),
// Ross-thick (fvol), Li-sparse (fgeo, h/b, b/r), 50 azimuth streams).
//
// Restates, in FP64, the kernel functions and the Fourier decomposition that
// VBRDF_MAINMASTER (vsup/vbrdf/vbrdf_sup_masters.f90:1559-3293) hands to
// VLIDORT: BRDF_F(m, i, j) between quadrature streams, BRDF_F_0(m, i) from
// the solar beam, USER_BRDF_F(m, u, j), USER_BRDF_F_0(m, u), and the exact
// direct-bounce BRDF EXACTDB_BRDFUNC(u, a) of the first-order correction.
// Paths are relative to the reference project root
// (src/Components/rtms/RTSI/VLIDORT2p8p3/...).  No product code links it.
//
// Parity pin: tests/test_oracle_golden_brdf.py compares it with the
// reference's saved gfortran output vlidort_v_test/saved_results/gfortran/
// results_brdf_supcheck_lattice.res (Ross-thin + Li-dense + Cox-Munk with
// shadowing) and, through the RT oracle, results_brdfplus_tester_lattice_I000.all.
//
// Not reproduced: VBRDF_MAINMASTER's white-sky-albedo check (:2976-2990)
// reads a scaling-kernel array that it fills only when WSA scaling is
// requested, so its outcome rests on unset storage; it never changes a
// Fourier component for physical kernel weights.
#include <cmath>
#include <vector>

#include "vlidort_oracle.h"

using namespace orc;

namespace {

// Complementary error function by the Chebyshev fit of Numerical Recipes
// (Press et al., erfcc; fractional error < 1.2e-7), the approximation the
// reference's Cox-Munk shadowing uses (vsup/vbrdf/vbrdf_sup_aux.f90:266-286).
double erfc_nr(double x) {
  const double z = std::fabs(x), t = 1.0 / (1.0 + 0.5 * z);
  const double c[10] = {-1.26551223, 1.00002368, 0.37409196, 0.09678418, -0.18628806,
                        0.27886807, -1.13520398, 1.48851587, -0.82215223, 0.17087277};
  double p = c[9];
  for (int k = 8; k >= 1; --k) p = c[k] + t * p;
  const double r = t * std::exp(-z * z + c[0] + t * p);
  return x < 0.0 ? 2.0 - r : r;
}

// Li kernels' shared geometry (vbrdf_sup_kernels.f90 LISPARSE/LIDENSE_VFUNCTION):
// incident (xi, sxi) and reflected (xj, sxj) directions stretched by the
// crown shape b/r = pars[1]; returns P, R and the overlap Q of the h/b = pars[0] crowns.
void li_geometry(const double* pars, double xi, double sxi, double xj, double sxj, double cphi, double sphi,
                 double* P, double* R, double* Q) {
  const double ckphi = -cphi;
  double t_inc = pars[1] * (sxi / xi);
  const double a_inc = std::atan(t_inc);
  const double x_inc = std::cos(a_inc), sx_inc = std::sin(a_inc);
  double t_ref = pars[1] * (sxj / xj);
  const double a_ref = std::atan(t_ref);
  const double x_ref = std::cos(a_ref), sx_ref = std::sin(a_ref);
  const double cksi = x_inc * x_ref + sx_inc * sx_ref * ckphi;
  *P = (1.0 + cksi) / x_ref / x_inc;
  *R = 1.0 / x_inc + 1.0 / x_ref;
  const double dt1 = t_ref * t_ref + t_inc * t_inc, dt2 = t_inc * t_ref;
  const double delta = std::sqrt(dt1 - 2.0 * dt2 * ckphi);
  const double h = std::sqrt(delta * delta + sphi * sphi * dt2 * dt2);
  const double cost = pars[0] * h / *R;
  if (cost > 1.0) {
    *Q = 1.0;
  } else {
    const double t = std::acos(cost), sint = std::sqrt(1.0 - cost * cost);
    *Q = 1.0 - (t - sint * cost) / PIE;
  }
}

// Ross kernels (ROSSTHIN/ROSSTHICK_VFUNCTION): the phase angle of the
// backward-reversed azimuth, volumetric term over mu_i mu_j (thin) or
// mu_i + mu_j (thick).
double ross(bool thick, double xi, double sxi, double xj, double sxj, double cphi) {
  double cksi = xi * xj + sxi * sxj * (-cphi);
  if (cksi > 1.0) cksi = 1.0;
  const double sksi = std::sqrt(1.0 - cksi * cksi), ksi = std::acos(cksi);
  const double PIO2 = 0.5 * PIE, PIO4 = 0.25 * PIE;
  const double func = ((PIO2 - ksi) * cksi + sksi) / (thick ? (xi + xj) : (xi * xj));
  return func - (thick ? PIO4 : PIO2);
}

// Cox-Munk glitter with optional shadowing (COXMUNK_VFUNCTION,
// vbrdf_sup_kernels.f90:1018-1135): pars = (slope variance, refractive
// index squared, shadow flag).  `cphi` enters as the routine's CKPHI.
double coxmunk(const double* pars, double xi, double sxi, double xj, double sxj, double cphi) {
  double z = xi * xj + sxi * sxj * (-cphi);
  if (z > 1.0) z = 1.0;
  const double z1 = std::acos(z), z2 = std::cos(z1 * 0.5), z2m1 = z2 * z2 - 1.0;
  const double h1 = pars[1] * z2, h2 = std::sqrt(pars[1] + z2m1);
  const double rp = (h1 - h2) / (h1 + h2), rl = (z2 - h2) / (z2 + h2);
  const double xmp = 0.5 * (rp * rp + rl * rl);
  double a = 2.0 * z2;
  double b = (xi + xj) / a;
  if (b > 1.0) b = 1.0;
  a = 0.5 * PIE - std::asin(b);
  const double ta = std::tan(a), arg = ta * ta / pars[0];
  double k = 0.0;
  if (arg < 88.0) {
    const double prob = std::exp(-arg);
    k = xmp * (prob / pars[0]) * (0.25 / xi / (b * b * b * b)) / xj;
  }
  if (pars[2] == 0.0) return k;
  const double s1 = std::sqrt(pars[0] / PIE), s3 = 1.0 / std::sqrt(pars[0]), s2 = s3 * s3;
  auto shadow = [&](double x) {
    const double dcot = x / std::sqrt(1.0 - x * x);
    return 0.5 * (s1 * std::exp(-dcot * dcot * s2) / dcot - erfc_nr(dcot * s3));
  };
  return k * (1.0 / (1.0 + shadow(xi) + shadow(xj)));
}

// GISS Cox-Munk glint, the (1,1) element (GISSCOXMUNK_VFUNCTION,
// vbrdf_sup_kernels.f90:1145-1492): pars = (slope variance parameter sigma2p,
// real refractive index n, shadow flag); Fresnel reflection of the facet
// between the incident vector (SXI, 0, -XI) and the reflected one
// (SXJ cphi, SXJ sphi, XJ), with cphi, sphi the routine's CKPHI_REF,
// SKPHI_REF.  Cosines within 1e-9 of 1 are replaced by 0.999999999999 for
// the call, as the routine does (it writes them back to the caller's
// variable; here the caller's value is kept).
double giss_coxmunk(const double* pars, double xi, double sxi, double xj, double sxj, double cphi, double sphi) {
  const double sigma2 = pars[0];
  if (std::fabs(xi - 1.0) < 1e-9) xi = 0.999999999999;
  if (std::fabs(xj - 1.0) < 1e-9) xj = 0.999999999999;
  const double vi1 = sxi * 1.0, vi2 = sxi * 0.0, vi3 = -xi;
  const double vr1 = sxj * cphi, vr2 = sxj * sphi, vr3 = xj;
  const double u1 = vi1 - vr1, u2 = vi2 - vr2, u3 = vi3 - vr3;
  const double fact1 = u1 * u1 + u2 * u2 + u3 * u3;
  const double factor = std::sqrt(1.0 / fact1);
  const double cn1 = 1.0, cn2 = pars[1];
  const double xi1 = factor * (u1 * vi1 + u2 * vi2 + u3 * vi3);
  double cxi2 = 1.0 - (1.0 - xi1 * xi1) * cn1 * cn1 / (cn2 * cn2);
  cxi2 = std::sqrt(cxi2);
  double c1 = cn1 * xi1, c2 = cn2 * cxi2;
  const double crper = (c1 - c2) / (c1 + c2);
  c1 = cn2 * xi1;
  c2 = cn1 * cxi2;
  const double crpar = (c1 - c2) / (c1 + c2);
  const double ti1 = -xi * 1.0, ti2 = -xi * 0.0, ti3 = -sxi;
  const double tr1 = xj * cphi, tr2 = xj * sphi, tr3 = -sxj;
  const double pi1 = -0.0, pi2 = 1.0, pi3 = 0.0;
  const double pr1 = -sphi, pr2 = cphi, pr3 = 0.0;
  const double pikr = pi1 * vr1 + pi2 * vr2 + pi3 * vr3;
  const double prki = pr1 * vi1 + pr2 * vi2 + pr3 * vi3;
  const double tikr = ti1 * vr1 + ti2 * vr2 + ti3 * vr3;
  const double trki = tr1 * vi1 + tr2 * vi2 + tr3 * vi3;
  const double e1 = pikr * prki, e2 = tikr * trki, e3 = tikr * prki, e4 = pikr * trki;
  double cf11 = e1 * crper + e2 * crpar;
  const double cf12 = -e3 * crper + e4 * crpar;
  const double cf21 = -e4 * crper + e3 * crpar;
  double cf22 = e2 * crper + e1 * crpar;
  const double vp1 = vi2 * vr3 - vi3 * vr2, vp2 = vi3 * vr1 - vi1 * vr3, vp3 = vi1 * vr2 - vi2 * vr1;
  double dmod = vp1 * vp1 + vp2 * vp2 + vp3 * vp3;
  dmod = dmod * dmod;
  if (dmod == 0.0) {
    cf11 = crpar;
    cf22 = crper;
    dmod = 1.0;
  }
  const double rdz2 = u3 * u3, rdz4 = rdz2 * rdz2;
  const double dcoeff0 = 1.0 / (8.0 * xi * xj * dmod * rdz4 * sigma2);
  const double arg = (u1 * u1 + u2 * u2) / (2.0 * sigma2 * rdz2);
  const double dex = arg > 88.0 ? 0.0 : std::exp(-arg);
  const double dcoeff = dcoeff0 * fact1 * fact1 * dex;
  const double af = 0.5 * dcoeff;
  double a11 = std::fabs(cf11), a12 = std::fabs(cf12), a21 = std::fabs(cf21), a22 = std::fabs(cf22);
  a11 *= a11; a12 *= a12; a21 *= a21; a22 *= a22;
  double k = (a11 + a12 + a21 + a22) * af;
  if (pars[2] == 0.0) return k;
  const double s1 = std::sqrt(2.0 * sigma2 / PIE), s3 = 1.0 / std::sqrt(2.0 * sigma2), s2 = s3 * s3;
  auto shadow = [&](double x) {
    if (x == 1.0) return 0.0;
    const double dcot = x / std::sqrt(1.0 - x * x);
    return 0.5 * (s1 * std::exp(-dcot * dcot * s2) / dcot - erfc_nr(dcot * s3));
  };
  return k * (1.0 / (1.0 + shadow(xi) + shadow(xj)));
}

}  // namespace

namespace orc {

// One kernel value, incident (xi, sxi), reflected (xj, sxj), relative
// azimuth phi (cos, sin).  `which` follows vlidort_pars.f90:466-474.
double brdf_kernel(int which, const double* pars, double xi, double sxi, double xj, double sxj, double cphi,
                   double sphi) {
  switch (which) {
    case 1: return 1.0;                                       // Lambertian
    case 2: return ross(false, xi, sxi, xj, sxj, cphi);      // Ross-thin
    case 3: return ross(true, xi, sxi, xj, sxj, cphi);       // Ross-thick
    case 4: {                                                 // Li-sparse
      double P, R, Q;
      li_geometry(pars, xi, sxi, xj, sxj, cphi, sphi, &P, &R, &Q);
      return 0.5 * P - Q * R;
    }
    case 5: {                                                 // Li-dense
      double P, R, Q;
      li_geometry(pars, xi, sxi, xj, sxj, cphi, sphi, &P, &R, &Q);
      return P / Q / R - 2.0;
    }
    case 9: return coxmunk(pars, xi, sxi, xj, sxj, cphi);    // Cox-Munk
    case 10: return giss_coxmunk(pars, xi, sxi, xj, sxj, cphi, sphi);  // GISS Cox-Munk
  }
  return 0.0;
}

}  // namespace orc

// The BRDF inputs of one VLIDORT solve for one solar beam (VBRDF_MAINMASTER
// with solar sources, user streams, NSTOKES = 1, half-range azimuth quadrature).
//   nk kernels: which[k] (vlidort_pars.f90:466-474), factors[k], pars[3 k..3 k+2]
//   (for Cox-Munk pars[3 k + 2] is replaced by the shadow flag, :2280-2291);
//   nstreams_brdf azimuth streams (halved for the half range, :2242-2247);
//   N quadrature streams, Fourier terms m = 0..nmom.
// Outputs (m fastest-last, row-major):
//   f[(m * N + i) * N + j]  BRDF_F(m, i, j): reflected stream i, incident j
//   f0[m * N + i]           BRDF_F_0(m, i)
//   uf[(m * nvza + u) * N + j]  USER_BRDF_F(m, u, j)
//   uf0[m * nvza + u]       USER_BRDF_F_0(m, u)
//   exactdb[u * nraa + a]   EXACTDB_BRDFUNC(u, a) (lattice of the beam)
// Returns 0.
extern "C" int oracle_brdf_supplement(int nk, const int* which, const double* factors, const double* pars_in,
                                      int do_shadow, int nstreams_brdf, int N, int nmom, double sza, int nvza,
                                      const double* vza, int nraa, const double* raa, double* f, double* f0,
                                      double* uf, double* uf0, double* exactdb) {
  const int M1 = nmom + 1;
  std::vector<double> qx(N), qw(N), qs(N);
  getquad2(0.0, 1.0, N, qx.data(), qw.data());
  for (int i = 0; i < N; ++i) qs[i] = std::sqrt(1.0 - qx[i] * qx[i]);
  // BRDF_QUADRATURE_GAUSSIAN, half range (vbrdf_sup_aux.f90:356-461)
  const int nb = nstreams_brdf / 2;
  std::vector<double> xb(nb), ab(nb), cxb(nb), sxb(nb);
  getquad2(0.0, 1.0, nb, xb.data(), ab.data());
  for (int k = 0; k < nb; ++k) {
    xb[k] = PIE * xb[k];
    cxb[k] = std::cos(xb[k]);
    sxb[k] = std::sin(xb[k]);
  }
  const double mu0 = std::cos(sza * DTR), s0 = std::sqrt(1.0 - mu0 * mu0);
  std::vector<double> mu(nvza), su(nvza);
  for (int u = 0; u < nvza; ++u) {
    mu[u] = std::cos(vza[u] * DTR);
    su[u] = std::sqrt(1.0 - mu[u] * mu[u]);
  }
  for (int e = 0; e < M1 * N * N; ++e) f[e] = 0.0;
  for (int e = 0; e < M1 * N; ++e) f0[e] = 0.0;
  for (int e = 0; e < M1 * nvza * N; ++e) uf[e] = 0.0;
  for (int e = 0; e < M1 * nvza; ++e) uf0[e] = 0.0;
  for (int e = 0; e < nvza * nraa; ++e) exactdb[e] = 0.0;
  std::vector<double> kq(N * N * nb), k0(N * nb), ku(nvza * N * nb), ku0(nvza * nb);
  for (int kk = 0; kk < nk; ++kk) {
    double pars[3] = {pars_in[3 * kk], pars_in[3 * kk + 1], pars_in[3 * kk + 2]};
    if (which[kk] == 9 || which[kk] == 10) pars[2] = do_shadow ? 1.0 : 0.0;
    const int w = which[kk];
    const double fac = factors[kk];
    // exact direct bounce (VBRDF_MAKER, vbrdf_sup_routines.f90:244-266)
    for (int u = 0; u < nvza; ++u)
      for (int a = 0; a < nraa; ++a) {
        const double phi = raa[a] * DTR;
        exactdb[u * nraa + a] += fac * brdf_kernel(w, pars, mu0, s0, mu[u], su[u], std::cos(phi), std::sin(phi));
      }
    // kernels on the azimuth quadrature (:449-602)
    for (int i = 0; i < N; ++i)
      for (int k = 0; k < nb; ++k) k0[i * nb + k] = brdf_kernel(w, pars, mu0, s0, qx[i], qs[i], cxb[k], sxb[k]);
    for (int i = 0; i < N; ++i)
      for (int j = 0; j < N; ++j)
        for (int k = 0; k < nb; ++k)
          kq[(i * N + j) * nb + k] = brdf_kernel(w, pars, qx[j], qs[j], qx[i], qs[i], cxb[k], sxb[k]);
    for (int u = 0; u < nvza; ++u) {
      for (int k = 0; k < nb; ++k) ku0[u * nb + k] = brdf_kernel(w, pars, mu0, s0, mu[u], su[u], cxb[k], sxb[k]);
      for (int j = 0; j < N; ++j)
        for (int k = 0; k < nb; ++k)
          ku[(u * N + j) * nb + k] = brdf_kernel(w, pars, qx[j], qs[j], mu[u], su[u], cxb[k], sxb[k]);
    }
    // Fourier components (VBRDF_FOURIER, vbrdf_sup_routines.f90:2073-2491;
    // master loop vbrdf_sup_masters.f90:3025-3120): the Lambertian kernel
    // adds 1 to term 0 only; the others HELP * sum_k A_k cos(m x_k) K_k with
    // HELP = DELFAC (1 for m = 0, else 2) on the half range.
    std::vector<double> cf(nb);
    for (int m = 0; m <= nmom; ++m) {
      if (w == 1) {
        if (m != 0) continue;
        for (int e = 0; e < N * N; ++e) f[e] += fac;
        for (int i = 0; i < N; ++i) f0[i] += fac;
        for (int e = 0; e < nvza * N; ++e) uf[e] += fac;
        for (int u = 0; u < nvza; ++u) uf0[u] += fac;
        continue;
      }
      const double help = (m == 0) ? 1.0 : 2.0;
      for (int k = 0; k < nb; ++k) cf[k] = (m == 0) ? ab[k] : ab[k] * std::cos((double)m * xb[k]);
      auto dot = [&](const double* kv) {
        double s = 0.0;
        for (int k = 0; k < nb; ++k) s += kv[k] * cf[k];
        return help * s;
      };
      for (int i = 0; i < N; ++i) {
        for (int j = 0; j < N; ++j) f[(m * N + i) * N + j] += fac * dot(&kq[(i * N + j) * nb]);
        f0[m * N + i] += fac * dot(&k0[i * nb]);
      }
      for (int u = 0; u < nvza; ++u) {
        for (int j = 0; j < N; ++j) uf[(m * nvza + u) * N + j] += fac * dot(&ku[(u * N + j) * nb]);
        uf0[m * nvza + u] += fac * dot(&ku0[u * nb]);
      }
    }
  }
  return 0;
}
