/* CPU oracle (test infrastructure only) of getEdgeVars
 * (src/Shared/GMAO_Shared/Chem_Base/MieObs_py.F90:27-83): edge pressure,
 * height and temperature from layer air density and pressure thickness, in
 * default REAL (IEEE single precision) as the reference evaluates it, with
 * the C library's logf and powf for the Fortran LOG and ** of REAL operands.
 * Built with -ffp-contract=off.  Parity unpinned: the reference keeps no
 * saved edge profiles.
 */
#include <math.h>
#include <stdlib.h>

void oracle_get_edge_vars(int km, int nobs, const float* airdens, const float* delp, float ptop, float* pe,
                          float* ze, float* te) {
  const float grav = 9.80616f, rgas = 287.0f, kappa = 2.0f / 7.0f;
  float* pm = (float*)malloc(sizeof(float) * (size_t)km);
  float* tm = (float*)malloc(sizeof(float) * (size_t)km);
  for (int n = 0; n < nobs; ++n) {
    const float* rho = airdens + (long)km * n;
    const float* dp = delp + (long)km * n;
    float* p = pe + (long)(km + 1) * n;
    float* z = ze + (long)(km + 1) * n;
    float* t = te + (long)(km + 1) * n;
    p[0] = ptop;
    for (int k = 1; k <= km; ++k) p[k] = p[k - 1] + dp[k - 1];
    z[km] = 0.0f;
    for (int k = km; k >= 1; --k) {
      const float r = rho[k - 1] * grav;
      z[k - 1] = z[k] + dp[k - 1] / r;
    }
    for (int k = 1; k <= km; ++k) {
      pm[k - 1] = (p[k - 1] + p[k]) / 2.0f;
      const float r = rho[k - 1] * rgas;
      tm[k - 1] = pm[k - 1] / r;
    }
    t[0] = tm[0];
    for (int k = 2; k <= km; ++k) {
      const float alpha = logf(p[k - 1] / pm[k - 2]) / logf(pm[k - 1] / pm[k - 2]);
      const float d = tm[k - 1] - tm[k - 2];
      const float ad = alpha * d;
      t[k - 1] = tm[k - 2] + ad;
    }
    t[km] = tm[km - 1] * powf(p[km] / pm[km - 1], kappa);
  }
  free(pm);
  free(tm);
}
