/* CPU oracle (test infrastructure only) of the Rayleigh optical thickness
 * calculator VLIDORT_ROT_CALC (geo_vlidort/VLIDORT_ROT.F90:19-86), which runs
 * VLIDORT_Rayleigh, A(), coef_depol and F_air
 * (RTSI/VLIDORT2p8p3/VLIDORT_ScatMod.F90:145-283) per pixel and channel.
 *
 * The reference's literals are default (4-byte) REAL: each enters the REAL*8
 * arithmetic as the float nearest to it, and the expressions whose operands
 * are all literals (`360.0*1e-6`, `1.0/1000`, `78.084 + 20.946 + 0.934`,
 * `4.*atan(1.0)`) are evaluated in single precision.  Operation order follows
 * the Fortran left-to-right evaluation; built with -ffp-contract=off.
 * Parity unpinned: the reference has no saved ROT values.
 */
#include <math.h>

#define F(x) ((double)(x##f)) /* a default-REAL literal widened to REAL*8 */

/* F_air (ScatMod.F90:267-283): King factor of the air mixture. */
static double f_air(double xx2, double c) {
  const double depol1 = F(1.034) + F(3.17E-4) * xx2;
  const double depol2 = F(1.096) + F(1.385E-3) * xx2 + F(1.448E-4) * xx2 * xx2;
  const double depol3 = 1.0;
  const double depol4 = F(1.15);
  const float den_lit = (78.084f + 20.946f) + 0.934f; /* all-literal part, REAL*4 */
  return (F(78.084) * depol1 + F(20.946) * depol2 + F(0.934) * depol3 + c * F(100.0) * depol4) /
         ((double)den_lit + c * F(100.0));
}

/* CO2 volume mixing ratio `360.0*1e-6`, a REAL*4 product. */
static double co2(void) { return (double)(360.0f * 1e-6f); }

/* Ns = (Av/22.4141)*(273.15/Ts)*(1.0/1000), molecules/cm^3 (ScatMod.F90:180, 238). */
static double ns_std(void) {
  const double av = F(6.0221367e23), ts = F(288.15);
  return (av / F(22.4141)) * (F(273.15) / ts) * (double)(1.0f / 1000.0f);
}

/* A(X), Rayleigh cross section [cm^2/molecule] at X micron (ScatMod.F90:211-247). */
static double cross_section(double x) {
  const double pi = (double)3.14159274101257324f; /* 4.*atan(1.0) in REAL*4 */
  const double xx = 1.0 / x;
  const double xx2 = xx * xx;
  const double cm = x / F(10000.0);
  const double pi3 = pi * pi * pi;
  double ri = F(8060.51) + F(2480990.0) / (F(132.274) - xx2) + F(17455.7) / (F(39.32957) - xx2);
  ri = ri * F(1e-8) + 1.0;
  const double c = co2();
  ri = (ri - 1.0) * (1.0 + F(0.54) * (c - F(0.0003))) + 1.0;
  const double ri2 = ri * ri;
  const double ns = ns_std();
  return 24.0 * pi3 * f_air(xx2, c) * ((ri2 - 1.0) * (ri2 - 1.0)) /
         (ns * ns * cm * cm * cm * cm * (ri2 + 2.0) * (ri2 + 2.0));
}

/* coef_depol (ScatMod.F90:251-265). */
double oracle_coef_depol(double x) {
  const double xx = 1.0 / x;
  const double xx2 = xx * xx;
  const double c = co2();
  return 6.0 * (f_air(xx2, c) - 1.0) / (7.0 * f_air(xx2, c) + 3.0);
}

/* VLIDORT_ROT_CALC: ROT(km,nobs,nch), depol(nch) from pe, he, te (km+1,nobs)
 * in Pa, m, K and channels in nm.  Returns rc (always 0: VLIDORT_Rayleigh
 * cannot fail). */
int oracle_rot_calc(int km, int nch, int nobs, const double* channels, const double* pe, const double* he,
                    const double* te, double* rot, double* depol) {
  const double ts = F(288.15), ps = F(1013.25);
  const double ns = ns_std();
  for (int j = 0; j < nobs; ++j) {
    const double* p = pe + (long)(km + 1) * j;
    const double* z = he + (long)(km + 1) * j;
    const double* t = te + (long)(km + 1) * j;
    for (int i = 0; i < nch; ++i) {
      const double wmicron = channels[i] * F(1.E-3);
      const double a = cross_section(wmicron);
      double vprev = 0.0;
      for (int k = 0; k <= km; ++k) {
        /* Vol(k) = A * Ns * (p/Ps) * (Ts/T) * 1e5 [km^-1]; p in hPa */
        double vol = a * ns * ((p[k] * F(1.E-2)) / ps) * (ts / t[k]);
        vol = vol * F(1.E5);
        if (k > 0) {
          const double difz = z[k - 1] * F(1.E-3) - z[k] * F(1.E-3);
          rot[(long)(k - 1) + (long)km * (j + (long)nobs * i)] = difz * (vprev + vol) / 2.0;
        }
        vprev = vol;
      }
      depol[i] = oracle_coef_depol(wmicron);
    }
  }
  return 0;
}
