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

constexpr int kBrdfAzimuth = 25;  // NSTREAMS_BRDF = 50 on the half range (vbrdf_sup_masters.f90:2242-2247)

// The half-range azimuth quadrature (BRDF_QUADRATURE_GAUSSIAN,
// vbrdf_sup_aux.f90:356-461): phi_k = pi x_k with Gauss-Legendre (x_k, a_k)
// on (0, 1); cos and sin of phi_k.
struct BrdfQuad {
  double phi[kBrdfAzimuth], a[kBrdfAzimuth], c[kBrdfAzimuth], s[kBrdfAzimuth];
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

// BRDF inputs of a launch.
struct BrdfInputs {
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
// (m < 2N), then fiso, fvol, fgeo and the table index.
template <int NS>
struct BrdfBlock {
  static constexpr int NMX = 2 * NS;
  static constexpr long r0 = 0, ur = (long)NMX * NS, ur0 = 2L * NMX * NS, w = ur0 + NMX, total = w + 4;
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
  double kv[kBrdfAzimuth], kg[kBrdfAzimuth];
  // direction pairs: (beam -> stream i) i < N, (stream j -> view) N + j, (beam -> view) 2N
  for (int p = 0; p <= 2 * NS; ++p) {
    double xi, sxi, xj, sxj;
    if (p < NS) { xi = mu0; sxi = s0; xj = qx[p]; sxj = sqrt(1.0 - qx[p] * qx[p]); }
    else if (p < 2 * NS) { xi = qx[p - NS]; sxi = sqrt(1.0 - xi * xi); xj = mu; sxj = su; }
    else { xi = mu0; sxi = s0; xj = mu; sxj = su; }
    for (int k = 0; k < kBrdfAzimuth; ++k) {
      kv[k] = brdf_ross_thick(xi, sxi, xj, sxj, q.c[k]);
      kg[k] = brdf_li_sparse(hb, br, xi, sxi, xj, sxj, q.c[k], q.s[k]);
    }
    for (int m = 0; m < BB::NMX; ++m) {
      double sv = 0.0, sg = 0.0;
      for (int k = 0; k < kBrdfAzimuth; ++k) {
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
  double kv[kBrdfAzimuth];
  for (int i = 0; i < N; ++i)
    for (int j = 0; j < N; ++j) {
      const double xi = qx[j], sxi = sqrt(1.0 - xi * xi), xj = qx[i], sxj = sqrt(1.0 - xj * xj);
      for (int k = 0; k < kBrdfAzimuth; ++k)
        kv[k] = li ? brdf_li_sparse(hb, br, xi, sxi, xj, sxj, q.c[k], q.s[k])
                   : brdf_ross_thick(xi, sxi, xj, sxj, q.c[k]);
      for (int m = 0; m < 2 * N; ++m) {
        double s = 0.0;
        for (int k = 0; k < kBrdfAzimuth; ++k) s += kv[k] * ((m == 0) ? q.a[k] : q.a[k] * cos((double)m * q.phi[k]));
        out[((long)m * N + i) * N + j] = ((m == 0) ? 1.0 : 2.0) * s;
      }
    }
}

}  // namespace aerort
