/* Test infrastructure only: the CPU oracle for the Mie-table lookup and the
 * aerosol-optics mixing, in IEEE single precision exactly as the reference
 * evaluates it (default-kind REAL, no fused multiply-add; build with
 * -ffp-contract=off).  It is the checker for the CUDA AOP kernel and is
 * never linked by product code.
 *
 *   rh map        src/Shared/GMAO_Shared/Chem_Base/Chem_MieTableMod.F90:612-627
 *   lookup        src/Shared/GMAO_Shared/Chem_Base/Chem_MieMod.F90:789-965 (Chem_MieQueryByInt)
 *   mixing        src/Components/rtms/geo_vlidort/VLIDORT_MieMod.F90:124-336 (VLIDORT_getAOPvector)
 *
 * Table layout (Fortran column-major, as Chem_MieTable):
 *   bext,bsca,g : [irh + nrh*(ich + nch*ibin)]
 *   pmom        : [irh + nrh*(ich + nch*(ibin + nbin*(imom + nmom*ipol)))]
 */
#include <math.h>
#include <stdlib.h>

typedef struct {
  int nrh, nch, nbin, nmom, npol;
  const float* rh;
  const float* channels; /* [m] */
  const float* bext;
  const float* bsca;
  const float* g;
  const float* pmom;
  const int* rhi;   /* 991 entries, 1-based table index */
  const float* rha; /* 991 entries */
} OracleMieTable;

/* Chem_MieTableMod.F90:612-627: map RH in steps of 0.001 to the table node
 * below it and the linear weight of the node above. */
void oracle_mie_rhmap(int nrh, const float* rh, int* rhi, float* rha) {
  for (int j = 1; j <= 991; ++j) {
    for (int i = nrh; i >= 1; --i) {
      if ((j - 1) >= (int)(rh[i - 1] * 1000.0f)) {
        int ip1 = i + 1;
        rhi[j - 1] = i;
        if (ip1 > nrh) {
          rha[j - 1] = 0.0f;
        } else {
          float num = (float)(j - 1) / 1000.0f - rh[i - 1];
          float den = rh[ip1 - 1] - rh[i - 1];
          rha[j - 1] = num / den;
        }
        break;
      }
    }
  }
}

/* Chem_MieMod.F90:856-867 + 873-945 (tau, ssa, gasym, pmom). ich, ibin 0-based. */
static void mie_query(const OracleMieTable* t, int ibin, int ich, float q_mass, float rh, float* tau,
                      float* ssa, float* gasym, float* pmom /* nmom*npol, imom fastest */) {
  float rhUse = rh > 0.0f ? rh : 0.0f; /* dead store in the reference: overwritten below */
  rhUse = rh < 0.99f ? rh : 0.99f;
  int isnap = (int)((rhUse + 0.001f) * 1000.0f);
  if (isnap < 1) isnap = 1;
  float arh = t->rha[isnap - 1];
  int irh = t->rhi[isnap - 1];
  int irhp1 = irh + 1;
  if (irhp1 > t->nrh) irhp1 = t->nrh;
  int b0 = (irh - 1) + t->nrh * (ich + t->nch * ibin);
  int b1 = (irhp1 - 1) + t->nrh * (ich + t->nch * ibin);
  float w0 = 1.0f - arh;
  float bextIn = t->bext[b0] * w0 + t->bext[b1] * arh;
  float bscaIn = t->bsca[b0] * w0 + t->bsca[b1] * arh;
  float gIn = t->g[b0] * w0 + t->g[b1] * arh;
  size_t s = (size_t)t->nrh * t->nch * t->nbin;
  for (int ip = 0; ip < t->npol; ++ip)
    for (int im = 0; im < t->nmom; ++im) {
      size_t o = (size_t)(im + t->nmom * ip) * s;
      pmom[im + t->nmom * ip] = t->pmom[o + b0] * w0 + t->pmom[o + b1] * arh;
    }
  *tau = bextIn * q_mass;
  *ssa = bscaIn / bextIn;
  *gasym = gIn;
}

/* VLIDORT_MieMod.F90:124-336.  Tracer iq uses table q_table[iq] (-1: skip,
 * the reference's "cycle" when the tracer has no optics) and size bin
 * q_bin[iq] (0-based).  channels_nm: requested wavelengths [nm] (REAL);
 * matched against 1e9*table channels within 1 nm.  Arrays are Fortran
 * column-major: qm(km,nq,nobs), rh(km,nobs), tau/ssa/g(km,nch,nobs),
 * pmom(km,nch,nobs,nMom,nPol).  Returns rc: 0, 99 (channel not in table),
 * 666 (too few moments), 777 (inconsistent nPol). */
int oracle_get_aop_vector(int ntables, const OracleMieTable* tables, int km, int nobs, int nch, int nq,
                          const float* channels_nm, const int* q_table, const int* q_bin, const float* qm,
                          const float* rh, int nMom, int nPol, float* tau, float* ssa, float* g, float* pmom) {
  if (ntables < 1) return 99;
  const OracleMieTable* t0 = &tables[0];
  int* idxch = (int*)malloc(sizeof(int) * (nch > 0 ? nch : 1));
  for (int n = 0; n < nch; ++n) {
    idxch[n] = -1;
    for (int m = 0; m < t0->nch; ++m) {
      if (fabsf(channels_nm[n] - 1.0e9f * t0->channels[m]) < 1.0f) { idxch[n] = m; break; }
    }
    if (idxch[n] < 0) { free(idxch); return 99; }
  }
  size_t nk = (size_t)km * nch * nobs;
  for (size_t i = 0; i < nk; ++i) { tau[i] = 0.0f; ssa[i] = 0.0f; g[i] = 0.0f; }
  for (size_t i = 0; i < nk * (size_t)nMom * nPol; ++i) pmom[i] = 0.0f;
  float* pm = (float*)malloc(sizeof(float) * (size_t)(t0->nmom > 0 ? t0->nmom : 1) * 6);
  for (int iq = 0; iq < nq; ++iq) {
    if (q_table[iq] < 0) continue;
    const OracleMieTable* t = &tables[q_table[iq]];
    if (nMom > t->nmom) { free(pm); free(idxch); return 666; }
    int npol_ = 0, spherical_ext = 0;
    if (nPol <= t->npol) npol_ = nPol;
    else if (nPol == 6 && t->npol == 4) { npol_ = 4; spherical_ext = 1; }
    else { free(pm); free(idxch); return 777; }
    for (int i = 0; i < nobs; ++i)
      for (int n = 0; n < nch; ++n)
        for (int k = 0; k < km; ++k) {
          float tau_, ssa_, g_;
          mie_query(t, q_bin[iq], idxch[n], qm[k + (size_t)km * (iq + (size_t)nq * i)], rh[k + (size_t)km * i], &tau_,
                    &ssa_, &g_, pm);
          size_t o = k + (size_t)km * (n + (size_t)nch * i);
          tau[o] = tau[o] + tau_;
          ssa[o] = ssa[o] + ssa_ * tau_;
          g[o] = g[o] + g_ * ssa_ * tau_;
          for (int ip = 0; ip < npol_; ++ip)
            for (int im = 0; im < nMom; ++im) {
              size_t po = o + nk * (im + (size_t)nMom * ip);
              pmom[po] = pmom[po] + pm[im + t->nmom * ip] * ssa_ * tau_;
            }
          if (spherical_ext) { /* P22 = P11, P44 = P33 (iP22=5, iP44=6; iP11=1, iP33=3) */
            for (int im = 0; im < nMom; ++im) {
              pmom[o + nk * (im + (size_t)nMom * 4)] = pmom[o + nk * (im + (size_t)nMom * 0)];
              pmom[o + nk * (im + (size_t)nMom * 5)] = pmom[o + nk * (im + (size_t)nMom * 2)];
            }
          }
        }
  }
  for (size_t i = 0; i < nk; ++i)
    if (tau[i] > 0.0f) ssa[i] = ssa[i] / tau[i];
  for (size_t i = 0; i < nk; ++i)
    if (ssa[i] * tau[i] > 0.0f) g[i] = g[i] / (ssa[i] * tau[i]);
  for (size_t i = 0; i < nk; ++i)
    for (int ip = 0; ip < nPol; ++ip)
      for (int im = 0; im < nMom; ++im)
        if ((ssa[i] * tau[i]) > 0.0f) {
          size_t po = i + nk * (im + (size_t)nMom * ip);
          pmom[po] = pmom[po] / (ssa[i] * tau[i]);
        }
  free(pm);
  free(idxch);
  return 0;
}

/* polint of Chem_MieTableRead (Chem_MieTableMod.F90:671-717), as the
 * reference declares it: x(n), y(n) REAL*8; xWant, slope, dx, yWant REAL*4.
 * Returns 1 when the reference would print its out-of-range warning. */
int oracle_mie_polint(const double* x, const double* y, int n, float xwant, float* ywant) {
  int i = 0, warn = 0, j;
  float slope, dx, sdx;
  if ((double)xwant < x[0]) { warn = 1; i = 1; }
  if ((double)xwant > x[n - 1]) { warn = 1; i = n; }
  if (i == 0)
    for (j = 1; j <= n; ++j)
      if ((double)xwant >= x[j - 1]) i = j;
  if (i == n)
    slope = 0.0f;
  else
    slope = (float)((y[i] - y[i - 1]) / (x[i] - x[i - 1]));
  dx = (float)((double)xwant - x[i - 1]);
  sdx = slope * dx;
  *ywant = (float)(y[i - 1] + (double)sdx);
  return warn;
}

/* The interpolation loop of Chem_MieTableRead (Chem_MieTableMod.F90:575-601)
 * for bext, bsca, g and the first nmom moments of pmom, with the table read
 * as REAL*8 in file order (lambda fastest) and the result in Chem_MieTable
 * order (rh fastest).  Returns the number of polint warnings. */
int oracle_mie_table_interp(int nlam, const double* lam, int nrh, const double* rh_table, int nbin, int nmom_table,
                            int npol, const double* bext_t, const double* bsca_t, const double* g_t,
                            const double* pmom_t, int nch, const float* channels, int nmom, float* rh, float* bext,
                            float* bsca, float* g, float* pmom) {
  int warns = 0;
  double* col = (double*)malloc(sizeof(double) * (size_t)nlam);
  for (int i = 0; i < nrh; ++i) rh[i] = (float)rh_table[i];
  for (int j = 0; j < nbin; ++j)
    for (int i = 0; i < nrh; ++i)
      for (int n = 0; n < nch; ++n) {
        const long o = i + (long)nrh * (n + (long)nch * j);
        const long t = (long)nlam * (i + (long)nrh * j);
        warns += oracle_mie_polint(lam, bext_t + t, nlam, channels[n], &bext[o]);
        warns += oracle_mie_polint(lam, bsca_t + t, nlam, channels[n], &bsca[o]);
        warns += oracle_mie_polint(lam, g_t + t, nlam, channels[n], &g[o]);
        for (int m = 0; m < nmom; ++m)
          for (int p = 0; p < npol; ++p) {
            /* gather the wavelength column of pmom_table(:, i, j, m, p) */
            for (int l = 0; l < nlam; ++l)
              col[l] = pmom_t[l + (long)nlam * (i + (long)nrh * (j + (long)nbin * (m + (long)nmom_table * p)))];
            warns += oracle_mie_polint(lam, col, nlam, channels[n],
                                       &pmom[i + (long)nrh * (n + (long)nch * (j + (long)nbin * (m + (long)nmom * p)))]);
          }
      }
  free(col);
  return warns;
}
