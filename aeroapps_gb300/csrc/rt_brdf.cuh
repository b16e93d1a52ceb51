// MODIS RTLS BRDF surface of VLIDORT_Scalar_LandMODIS
// (src/Components/rtms/geo_vlidort/VLIDORT_BRDF_MODIS.F90:34-200): the kernel
// set of VLIDORT_LANDMODIS_SingleGeom
// (RTSI/VLIDORT2p8p3/VLIDORT_SurfaceMod.F90:1376-1596) -- Lambertian (fiso),
// Ross-thick (fvol), Li-sparse (fgeo; crown height h/b and shape b/r) -- with
// the Fourier decomposition of the VBRDF supplement
// (vsup/vbrdf/vbrdf_sup_masters.f90:1559-3293, vbrdf_sup_routines.f90:2073-2491):
// 50 azimuth streams on the half range (25 Gauss nodes of (0, pi)), term m
// weighted by 1 (m = 0) or 2 cos(m phi).
//
// Layout on the GPU.  The quadrature-to-quadrature components depend only on
// the stream count and the Li-sparse parameters, so the host computes them
// once per launch (one Ross-thick table, one Li-sparse table per distinct
// parameter pair) and every solve reads them from global memory (L2-resident:
// 2N x N x N doubles each).  The components that involve the solve's own
// angles -- solar beam to quadrature, quadrature to view, beam to view -- and
// the exact direct-bounce BRDF are formed by the set-up thread of each solve
// (solve_setup) into a per-solve block, element-major like the other scratch.
#pragma once
#include "rt_scalar.cuh"

namespace aerort {

constexpr int kBrdfAzimuth = 25;    // LandMODIS: NSTREAMS_BRDF = 50 on the half range (vbrdf_sup_masters.f90:2242-2247)
constexpr int kBrdfAzimuthCX = 50;  // Cox-Munk: NSTREAMS_BRDF = 100 (VLIDORT_SurfaceMod.F90:881)

// Surface kinds of a BRDF launch.
constexpr int kBrdfRTLS = 0;     // VLIDORT_Scalar_LandMODIS: Lambertian + Ross-thick + Li-sparse
constexpr int kBrdfCoxMunk = 1;  // VLIDORT_Scalar_CX: Cox-Munk glint with shadowing
constexpr int kBrdfGissCoxMunk = 2;  // VLIDORT_Scalar_GissCX: GISS Cox-Munk glint with shadowing

// The half-range azimuth quadrature (BRDF_QUADRATURE_GAUSSIAN,
// vbrdf_sup_aux.f90:356-461): phi_k = pi x_k with Gauss-Legendre (x_k, a_k)
// on (0, 1); cos and sin of phi_k; nb nodes.
struct BrdfQuad {
  double phi[kBrdfAzimuthCX], a[kBrdfAzimuthCX], c[kBrdfAzimuthCX], s[kBrdfAzimuthCX];
  int nb;
};

// Ross-thick volumetric kernel (ROSSTHICK_VFUNCTION, vbrdf_sup_kernels.f90):
// incident (xi, sxi), reflected (xj, sxj), relative azimuth cosine cphi.
RT_HD double brdf_ross_thick(double xi, double sxi, double xj, double sxj, double cphi) {
  double cksi = xi * xj + sxi * sxj * (-cphi);
  if (cksi > 1.0) cksi = 1.0;
  const double sksi = sqrt(1.0 - cksi * cksi), ksi = acos(cksi);
  const double func = ((0.5 * kPIE - ksi) * cksi + sksi) / (xi + xj);
  return func - 0.25 * kPIE;
}

// Li-sparse geometric kernel (LISPARSE_VFUNCTION): crown height hb = h/b and
// shape br = b/r stretch the zenith angles; P, R and the crown overlap Q.
RT_HD double brdf_li_sparse(double hb, double br, double xi, double sxi, double xj, double sxj, double cphi,
                                   double sphi) {
  const double ckphi = -cphi;
  const double t_inc = br * (sxi / xi), a_inc = atan(t_inc);
  const double x_inc = cos(a_inc), sx_inc = sin(a_inc);
  const double t_ref = br * (sxj / xj), a_ref = atan(t_ref);
  const double x_ref = cos(a_ref), sx_ref = sin(a_ref);
  const double cksi = x_inc * x_ref + sx_inc * sx_ref * ckphi;
  const double P = (1.0 + cksi) / x_ref / x_inc;
  const double R = 1.0 / x_inc + 1.0 / x_ref;
  const double dt1 = t_ref * t_ref + t_inc * t_inc, dt2 = t_inc * t_ref;
  const double delta = sqrt(dt1 - 2.0 * dt2 * ckphi);
  const double h = sqrt(delta * delta + sphi * sphi * dt2 * dt2);
  const double cost = hb * h / R;
  double Q = 1.0;
  if (!(cost > 1.0)) {
    const double t = acos(cost), sint = sqrt(1.0 - cost * cost);
    Q = 1.0 - (t - sint * cost) / kPIE;
  }
  return 0.5 * P - Q * R;
}

// Complementary error function of the reference's Cox-Munk shadowing: the
// Chebyshev fit of Numerical Recipes (Press et al., erfcc; fractional error
// < 1.2e-7), vbrdf_sup_aux.f90:266-286.  Its values, not CUDA's erfc, enter
// the reference's radiances.
RT_HD double brdf_erfc(double x) {
  const double z = fabs(x), t = 1.0 / (1.0 + 0.5 * z);
  double p = 0.17087277;
  p = -0.82215223 + t * p;
  p = 1.48851587 + t * p;
  p = -1.13520398 + t * p;
  p = 0.27886807 + t * p;
  p = -0.18628806 + t * p;
  p = 0.09678418 + t * p;
  p = 0.37409196 + t * p;
  p = 1.00002368 + t * p;
  const double r = t * exp(-z * z + -1.26551223 + t * p);
  return x < 0.0 ? 2.0 - r : r;
}

// Cox-Munk surface parameters of one (pixel, channel), from the 10 m wind
// W = |(U10m, V10m)| clamped to [0, 50] m/s and sigma2 = 0.003 + 0.00512 W
// (VLIDORT_SurfaceMod.F90:893-898, :680-685).  Cox-Munk (kernel 9): slope
// variance sigma2 and m2 = mr^2 (:900-907); GISS Cox-Munk (kernel 10): slope
// parameter sigma2 / 2 and the index mr itself (:688-697).  s1, s2, s3 are the
// shadowing constants of either kernel.
struct CoxMunkPars {
  bool giss;
  double sigma2, m2;  // the kernel's first and second parameter
  double s1, s2, s3;
};

RT_HD CoxMunkPars brdf_cm_pars(bool giss, double u10, double v10, double mr) {
  double w = sqrt(u10 * u10 + v10 * v10);
  if (w < 0.0) w = 0.0;
  if (w > 50.0) w = 50.0;
  const double sigma2 = 0.003 + 0.00512 * w;
  CoxMunkPars p;
  p.giss = giss;
  if (giss) {
    p.sigma2 = 0.5 * sigma2;
    p.m2 = mr;
    p.s1 = sqrt(2.0 * p.sigma2 / kPIE);
    p.s3 = 1.0 / sqrt(2.0 * p.sigma2);
  } else {
    p.sigma2 = sigma2;
    p.m2 = mr * mr;
    p.s1 = sqrt(p.sigma2 / kPIE);
    p.s3 = 1.0 / sqrt(p.sigma2);
  }
  p.s2 = p.s3 * p.s3;
  return p;
}

// The GISS kernel replaces a cosine within 1e-9 of 1 by 0.999999999999 for
// the call (GISSCOXMUNK_VFUNCTION, vbrdf_sup_kernels.f90:1238-1239).
RT_HD double brdf_giss_cos(double x) { return fabs(x - 1.0) < 1e-9 ? 0.999999999999 : x; }

// Shadowing term of one direction (cosine x) in either kernel.
RT_HD double brdf_cm_shadow(const CoxMunkPars& p, double x) {
  if (p.giss) {
    x = brdf_giss_cos(x);
    if (x == 1.0) return 0.0;
  }
  const double dcot = x / sqrt(1.0 - x * x);
  return 0.5 * (p.s1 * exp(-dcot * dcot * p.s2) / dcot - brdf_erfc(dcot * p.s3));
}

// Cox-Munk glint kernel with shadowing (COXMUNK_VFUNCTION,
// vbrdf_sup_kernels.f90:1018-1135, NSTOKES = 1): incident (xi, sxi),
// reflected (xj, sxj), relative azimuth cosine cphi; shi, shj the shadowing
// terms of the two directions (brdf_cm_shadow).
RT_HD double brdf_cox_munk(const CoxMunkPars& p, double xi, double sxi, double xj, double sxj, double cphi, double shi,
                           double shj) {
  double z = xi * xj + sxi * sxj * (-cphi);
  if (z > 1.0) z = 1.0;
  const double z1 = acos(z), z2 = cos(z1 * 0.5), z2m1 = z2 * z2 - 1.0;
  const double h1 = p.m2 * z2, h2 = sqrt(p.m2 + z2m1);
  const double rp = (h1 - h2) / (h1 + h2), rl = (z2 - h2) / (z2 + h2);
  const double xmp = 0.5 * (rp * rp + rl * rl);
  double a = 2.0 * z2;
  double b = (xi + xj) / a;
  if (b > 1.0) b = 1.0;
  a = 0.5 * kPIE - asin(b);
  const double ta = tan(a), arg = ta * ta / p.sigma2;
  double k = 0.0;
  if (arg < 88.0) {
    const double prob = exp(-arg);
    k = xmp * (prob / p.sigma2) * (0.25 / xi / (b * b * b * b)) / xj;
  }
  return k * (1.0 / (1.0 + shi + shj));
}

// GISS Cox-Munk glint with shadowing, the (1,1) element (GISSCOXMUNK_VFUNCTION,
// vbrdf_sup_kernels.f90:1145-1492): the Fresnel reflection of the facet
// between the incident vector (sxi, 0, -xi) and the reflected one
// (sxj cphi, sxj sphi, xj), cphi and sphi the routine's CKPHI_REF and
// SKPHI_REF; shi, shj the shadowing terms (brdf_cm_shadow).
RT_HD double brdf_giss_cox_munk(const CoxMunkPars& p, double xi, double sxi, double xj, double sxj, double cphi,
                                double sphi, double shi, double shj) {
  xi = brdf_giss_cos(xi);
  xj = brdf_giss_cos(xj);
  const double vi1 = sxi, vi3 = -xi;
  const double vr1 = sxj * cphi, vr2 = sxj * sphi, vr3 = xj;
  const double u1 = vi1 - vr1, u2 = -vr2, u3 = vi3 - vr3;
  const double fact1 = u1 * u1 + u2 * u2 + u3 * u3;
  const double factor = sqrt(1.0 / fact1);
  const double n = p.m2;
  const double xi1 = factor * (u1 * vi1 + u3 * vi3);
  const double cxi2 = sqrt(1.0 - (1.0 - xi1 * xi1) / (n * n));
  const double crper = (xi1 - n * cxi2) / (xi1 + n * cxi2);
  const double crpar = (n * xi1 - cxi2) / (n * xi1 + cxi2);
  const double pikr = vr2;                    // PI . VR, PI = (0, 1, 0)
  const double prki = -sphi * vi1;            // PR . VI, PR = (-sphi, cphi, 0)
  const double tikr = -xi * vr1 - sxi * vr3;  // TI . VR, TI = (-xi, 0, -sxi)
  const double trki = xj * cphi * vi1 - sxj * vi3;  // TR . VI, TR = (xj cphi, xj sphi, -sxj)
  const double e1 = pikr * prki, e2 = tikr * trki, e3 = tikr * prki, e4 = pikr * trki;
  double cf11 = e1 * crper + e2 * crpar;
  const double cf12 = -e3 * crper + e4 * crpar;
  const double cf21 = -e4 * crper + e3 * crpar;
  double cf22 = e2 * crper + e1 * crpar;
  const double vp1 = -vi3 * vr2, vp2 = vi3 * vr1 - vi1 * vr3, vp3 = vi1 * vr2;  // VI x VR
  double dmod = vp1 * vp1 + vp2 * vp2 + vp3 * vp3;
  dmod = dmod * dmod;
  if (dmod == 0.0) {
    cf11 = crpar;
    cf22 = crper;
    dmod = 1.0;
  }
  const double rdz2 = u3 * u3, rdz4 = rdz2 * rdz2;
  const double dcoeff0 = 1.0 / (8.0 * xi * xj * dmod * rdz4 * p.sigma2);
  const double arg = (u1 * u1 + u2 * u2) / (2.0 * p.sigma2 * rdz2);
  const double dex = arg > 88.0 ? 0.0 : exp(-arg);
  const double af = 0.5 * (dcoeff0 * fact1 * fact1 * dex);
  const double k = (cf11 * cf11 + cf12 * cf12 + cf21 * cf21 + cf22 * cf22) * af;
  return k * (1.0 / (1.0 + shi + shj));
}

// Either glint kernel of p at one direction pair and azimuth node.
RT_HD double brdf_glint(const CoxMunkPars& p, double xi, double sxi, double xj, double sxj, double cphi, double sphi,
                        double shi, double shj) {
  return p.giss ? brdf_giss_cox_munk(p, xi, sxi, xj, sxj, cphi, sphi, shi, shj)
                : brdf_cox_munk(p, xi, sxi, xj, sxj, cphi, shi, shj);
}

// BRDF inputs of a launch.
struct BrdfInputs {
  int kind;            // kBrdfRTLS, kBrdfCoxMunk or kBrdfGissCoxMunk
  // glint kernels (kind != kBrdfRTLS): winds (nobs), refractive index (nch), and
  // the azimuth weights cf[m * nb + k] = a_k (m = 0) or a_k cos(m phi_k), m < 2N
  const double* u10;
  const double* v10;
  const double* mr;
  const double* cf;
  const double* kw;    // (3, nch, nobs) kernel amplitudes fiso, fgeo, fvol (the reference's kernel_wt order)
  const int* tab;      // (nch, nobs) Li-sparse parameter table of each solve
  const double* tpar;  // (2, ntab) h/b, b/r of each table
  const double* qq;    // Fourier tables: Ross-thick [m][i][j], then Li-sparse [t][m][i][j], m < 2N
  double* br;          // (nobs, nch) exact direct-bounce BRDF (output BR of the reference)
  double* terms;       // per-solve blocks (element-major, stride = solves per launch slice)
  long stride;         // solves per launch slice
  BrdfQuad q;
  double qx[16];       // the streams' quadrature cosines
};

// Elements of one solve's block for N streams: R0[m][i], UR[m][j], UR0[m]
// (m < 2N), then fiso, fvol, fgeo and the table index (RTLS); a Cox-Munk
// solve adds its own quadrature-to-quadrature components QQ[m][i][j].
template <int NS>
struct BrdfBlock {
  static constexpr int NMX = 2 * NS;
  static constexpr long r0 = 0, ur = (long)NMX * NS, ur0 = 2L * NMX * NS, w = ur0 + NMX, total = w + 4;
  static constexpr long qq = total, total_cx = qq + (long)NMX * NS * NS;
};

// Exact direct-bounce BRDF of the observation geometry (VBRDF_MAKER,
// vbrdf_sup_routines.f90:244-266, summed with the kernel amplitudes as
// vbrdf_sup_masters.f90:2857-2864): mu0, user mu from the truncated DEG_TO_RAD.
RT_HD double brdf_exact(const double* kw, double hb, double br, double sza, double vza, double raa) {
  const double mu0 = cos(sza * kDTR), s0 = sqrt(1.0 - mu0 * mu0);
  const double mu = cos(vza * kDTR), su = sqrt(1.0 - mu * mu);
  const double phi = raa * kDTR, cp = cos(phi), sp = sin(phi);
  double b = kw[0] * 1.0;  // Lambertian (fiso), Ross-thick (fvol), Li-sparse (fgeo), the supplement's order
  b += kw[2] * brdf_ross_thick(mu0, s0, mu, su, cp);
  b += kw[1] * brdf_li_sparse(hb, br, mu0, s0, mu, su, cp, sp);
  return b;
}

// One solve's beam and view Fourier terms into its block (VBRDF_FOURIER with
// the kernel sum of vbrdf_sup_masters.f90:3057-3120): for every m < 2N,
// R0(m, i) = BRDF_F_0, UR(m, j) = USER_BRDF_F, UR0(m) = USER_BRDF_F_0.  The
// kernel values on the 25 azimuth nodes are formed once per direction pair
// and reused by every m.
template <int NS>
RT_HD void brdf_solve_terms(const BrdfQuad& q, const double* qx, const double* kw, double hb, double br, double sza,
                            double vza, const Scratch& B) {
  using BB = BrdfBlock<NS>;
  const double mu0 = cos(sza * kDTR), s0 = sqrt(1.0 - mu0 * mu0);
  const double mu = cos(vza * kDTR), su = sqrt(1.0 - mu * mu);
  double kv[kBrdfAzimuthCX], kg[kBrdfAzimuthCX];
  // direction pairs: (beam -> stream i) i < N, (stream j -> view) N + j, (beam -> view) 2N
  for (int p = 0; p <= 2 * NS; ++p) {
    double xi, sxi, xj, sxj;
    if (p < NS) { xi = mu0; sxi = s0; xj = qx[p]; sxj = sqrt(1.0 - qx[p] * qx[p]); }
    else if (p < 2 * NS) { xi = qx[p - NS]; sxi = sqrt(1.0 - xi * xi); xj = mu; sxj = su; }
    else { xi = mu0; sxi = s0; xj = mu; sxj = su; }
    for (int k = 0; k < q.nb; ++k) {
      kv[k] = brdf_ross_thick(xi, sxi, xj, sxj, q.c[k]);
      kg[k] = brdf_li_sparse(hb, br, xi, sxi, xj, sxj, q.c[k], q.s[k]);
    }
    for (int m = 0; m < BB::NMX; ++m) {
      double sv = 0.0, sg = 0.0;
      for (int k = 0; k < q.nb; ++k) {
        const double cf = (m == 0) ? q.a[k] : q.a[k] * cos((double)m * q.phi[k]);
        sv += kv[k] * cf;
        sg += kg[k] * cf;
      }
      const double help = (m == 0) ? 1.0 : 2.0;
      double v = (m == 0) ? kw[0] : 0.0;
      v += kw[2] * (help * sv);
      v += kw[1] * (help * sg);
      const long e = p < NS ? BB::r0 + (long)m * NS + p : (p < 2 * NS ? BB::ur + (long)m * NS + (p - NS) : BB::ur0 + m);
      B[e] = v;
    }
  }
  B[BB::w] = kw[0];      // fiso
  B[BB::w + 1] = kw[2];  // fvol
  B[BB::w + 2] = kw[1];  // fgeo
}

// Host: the quadrature-to-quadrature Fourier table of one kernel (Ross-thick
// when li = false) for N streams: out[(m N + i) N + j] = HELP sum_k a_k
// cos(m phi_k) K(stream j -> stream i, phi_k), m < 2N (before the amplitude).
inline void brdf_qq_table(int N, const double* qx, const BrdfQuad& q, bool li, double hb, double br, double* out) {
  double kv[kBrdfAzimuthCX];
  for (int i = 0; i < N; ++i)
    for (int j = 0; j < N; ++j) {
      const double xi = qx[j], sxi = sqrt(1.0 - xi * xi), xj = qx[i], sxj = sqrt(1.0 - xj * xj);
      for (int k = 0; k < q.nb; ++k)
        kv[k] = li ? brdf_li_sparse(hb, br, xi, sxi, xj, sxj, q.c[k], q.s[k])
                   : brdf_ross_thick(xi, sxi, xj, sxj, q.c[k]);
      for (int m = 0; m < 2 * N; ++m) {
        double s = 0.0;
        for (int k = 0; k < q.nb; ++k) s += kv[k] * ((m == 0) ? q.a[k] : q.a[k] * cos((double)m * q.phi[k]));
        out[((long)m * N + i) * N + j] = ((m == 0) ? 1.0 : 2.0) * s;
      }
    }
}

// Exact direct-bounce glint BRDF of the observation geometry.
RT_HD double brdf_exact_cx(const CoxMunkPars& p, double sza, double vza, double raa) {
  const double mu0 = cos(sza * kDTR), s0 = sqrt(1.0 - mu0 * mu0);
  const double mu = cos(vza * kDTR), su = sqrt(1.0 - mu * mu);
  const double phi = raa * kDTR;
  return brdf_glint(p, mu0, s0, mu, su, cos(phi), sin(phi), brdf_cm_shadow(p, mu0), brdf_cm_shadow(p, mu));
}

// One glint solve's Fourier terms into its block (VBRDF_FOURIER, one Cox-Munk
// or GISS Cox-Munk kernel of factor 1): R0, UR, UR0 as brdf_solve_terms, and the quadrature-to-
// quadrature QQ(m, i, j) (reflected stream i, incident j), which depend on
// the solve's wind and refractive index.  The shadowing term of each
// direction is formed once; the kernel on the nb azimuth nodes once per
// direction pair and reused by every m; cf holds the azimuth weights.
template <int NS>
RT_HD void brdf_solve_terms_cx(const BrdfQuad& q, const double* cf, const double* qx, const CoxMunkPars& p,
                               double sza, double vza, const Scratch& B) {
  using BB = BrdfBlock<NS>;
  const int nb = q.nb;
  const double mu0 = cos(sza * kDTR), s0 = sqrt(1.0 - mu0 * mu0);
  const double mu = cos(vza * kDTR), su = sqrt(1.0 - mu * mu);
  double sq[NS], shq[NS];
  for (int i = 0; i < NS; ++i) {
    sq[i] = sqrt(1.0 - qx[i] * qx[i]);
    shq[i] = brdf_cm_shadow(p, qx[i]);
  }
  const double sh0 = brdf_cm_shadow(p, mu0), shu = brdf_cm_shadow(p, mu);
  double kv[kBrdfAzimuthCX];
  auto fourier = [&](long e0, long de) {  // B[e0 + m de] = HELP sum_k kv_k cf[m][k]
    for (int m = 0; m < BB::NMX; ++m) {
      double s = 0.0;
      for (int k = 0; k < nb; ++k) s += kv[k] * cf[m * nb + k];
      B[e0 + m * de] = ((m == 0) ? 1.0 : 2.0) * s;
    }
  };
  // beam -> stream i, stream j -> view, beam -> view
  for (int i = 0; i < NS; ++i) {
    for (int k = 0; k < nb; ++k) kv[k] = brdf_glint(p, mu0, s0, qx[i], sq[i], q.c[k], q.s[k], sh0, shq[i]);
    fourier(BB::r0 + i, NS);
  }
  for (int j = 0; j < NS; ++j) {
    for (int k = 0; k < nb; ++k) kv[k] = brdf_glint(p, qx[j], sq[j], mu, su, q.c[k], q.s[k], shq[j], shu);
    fourier(BB::ur + j, NS);
  }
  for (int k = 0; k < nb; ++k) kv[k] = brdf_glint(p, mu0, s0, mu, su, q.c[k], q.s[k], sh0, shu);
  fourier(BB::ur0, 1);
  // stream j -> stream i
  for (int i = 0; i < NS; ++i)
    for (int j = 0; j < NS; ++j) {
      for (int k = 0; k < nb; ++k)
        kv[k] = brdf_glint(p, qx[j], sq[j], qx[i], sq[i], q.c[k], q.s[k], shq[j], shq[i]);
      fourier(BB::qq + (long)i * NS + j, (long)NS * NS);
    }
}

}  // namespace aerort
