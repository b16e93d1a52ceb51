// Mie table set-up after the netCDF read: Chem_MieTableRead
// (src/Shared/GMAO_Shared/Chem_Base/Chem_MieTableMod.F90:557-627) takes the
// table fields as read from an optics_*.nc file (REAL*8, wavelength fastest)
// and produces the Chem_MieTable object (REAL*4, RH fastest) on the requested
// channels, interpolating every field linearly in wavelength with its internal
// polint (:671-717).  Host code, run once per table at initialisation.
#include <cmath>

#include "aerort.h"

namespace {

// polint (Chem_MieTableMod.F90:671-717) with its precisions: x, y REAL*8;
// xwant, the slope, dx and the result REAL*4.  Below x(1) it extrapolates
// with the first segment's slope, above x(n) it holds y(n); the reference
// warns in both cases (the caller counts those channels).
void polint(const double* x, const double* y, int n, float xwant, float* ywant) {
  const double xw = (double)xwant;
  int i = 0;
  if (xw < x[0]) i = 1;
  if (xw > x[n - 1]) i = n;
  if (i == 0)
    for (int j = 1; j <= n; ++j)
      if (xw >= x[j - 1]) i = j;
  const float slope = (i == n) ? 0.0f : (float)((y[i] - y[i - 1]) / (x[i] - x[i - 1]));
  const float dx = (float)(xw - x[i - 1]);
  const float sdx = slope * dx;  // REAL*4 product
  *ywant = (float)(y[i - 1] + (double)sdx);
}

// in(nlam, nrh, nbin) -> out(nrh, nch, nbin), both Fortran order
void interp_field(int nlam, const double* lam, int nrh, int nbin, const double* in, int nch, const float* ch,
                  float* out) {
  for (int j = 0; j < nbin; ++j)
    for (int i = 0; i < nrh; ++i) {
      const double* y = in + (long)nlam * (i + (long)nrh * j);
      for (int n = 0; n < nch; ++n) {
        float v;
        polint(lam, y, nlam, ch[n], &v);
        out[i + (long)nrh * (n + (long)nch * j)] = v;
      }
    }
}

}  // namespace

extern "C" int aerort_mie_table_interp(int nlam, const double* lambda_table, int nrh, const double* rh_table, int nbin,
                                       int nmom_table, int npol, const double* bext_table, const double* bsca_table,
                                       const double* g_table, const double* pmom_table, int nch, const float* channels_m,
                                       int nmom, float* rh, float* bext, float* bsca, float* g, float* pmom,
                                       int* nout) {
  if (nlam <= 0 || nrh <= 0 || nbin <= 0 || npol <= 0 || nch <= 0 || nmom < 0 || nmom_table < 0 || !lambda_table ||
      !rh_table || !bext_table || !bsca_table || !g_table || !channels_m || !rh || !bext || !bsca || !g)
    return AERORT_RC_ARG;
  if (nmom > nmom_table) return AERORT_RC_CHANNEL;  // Chem_MieTableRead rc = 99 (:327-331)
  if (nmom > 0 && (!pmom_table || !pmom)) return AERORT_RC_ARG;
  for (int n = 0; n < nch; ++n)
    if (!(channels_m[n] == channels_m[n])) return AERORT_RC_ARG;  // NaN: polint finds no segment
  for (int l = 0; l < nlam; ++l)
    if (!(lambda_table[l] == lambda_table[l])) return AERORT_RC_ARG;
  if (nout) {
    *nout = 0;
    for (int n = 0; n < nch; ++n) {
      const double x = (double)channels_m[n];
      *nout += (x < lambda_table[0] || x > lambda_table[nlam - 1]) ? 1 : 0;
    }
  }
  for (int i = 0; i < nrh; ++i) rh[i] = (float)rh_table[i];
  interp_field(nlam, lambda_table, nrh, nbin, bext_table, nch, channels_m, bext);
  interp_field(nlam, lambda_table, nrh, nbin, bsca_table, nch, channels_m, bsca);
  interp_field(nlam, lambda_table, nrh, nbin, g_table, nch, channels_m, g);
  if (nmom > 0) {
    // pmom_table(nlam, nrh, nbin, nmom_table, npol): the first nmom moments of each polarisation
    const long blk = (long)nlam * nrh * nbin;
    const long oblk = (long)nrh * nch * nbin;
    for (int p = 0; p < npol; ++p)
      for (int m = 0; m < nmom; ++m)
        interp_field(nlam, lambda_table, nrh, nbin, pmom_table + blk * (m + (long)nmom_table * p), nch, channels_m,
                     pmom + oblk * (m + (long)nmom * p));
  }
  return AERORT_OK;
}
