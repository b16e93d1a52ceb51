// Synthetic Mie tables: Lorenz-Mie series (Bohren & Huffman 1983, ch. 4 and
// appendix A; term count after Wiscombe 1980) integrated over lognormal size
// distributions, with hygroscopic growth, producing the fields of the
// reference's Chem_MieTable (src/Shared/GMAO_Shared/Chem_Base/Chem_MieTableMod.F90:55-83):
// mass extinction / scattering efficiency per kg of DRY aerosol, asymmetry
// parameter and Legendre expansion coefficients beta_l of the phase function
// normalised so that beta_0 = 1 (beta_1 = 3 g), in the table layout
// (nrh, nlambda, nbin, nmom).  Host code; used only to build input data.
#include <cmath>
#include <complex>
#include <vector>

typedef std::complex<double> cplx;

namespace {

void gauss_legendre(int n, double* x, double* w) {  // nodes on (-1,1)
  for (int i = 0; i < n; ++i) {
    double z = std::cos(M_PI * (i + 0.75) / (n + 0.5)), dp = 0.0;
    for (int it = 0; it < 100; ++it) {
      double p1 = 1.0, p0 = 0.0;
      for (int j = 1; j <= n; ++j) {
        double pm = p0;
        p0 = p1;
        p1 = ((2.0 * j - 1.0) * z * p0 - (j - 1.0) * pm) / j;
      }
      dp = n * (z * p1 - p0) / (z * z - 1.0);
      double z1 = z;
      z = z1 - p1 / dp;
      if (std::fabs(z - z1) < 1e-15) break;
    }
    x[i] = -z;
    w[i] = 2.0 / ((1.0 - z * z) * dp * dp);
  }
}

// Efficiencies and S11 = (|S1|^2 + |S2|^2)/2 at angle cosines mu[0..na) for a
// homogeneous sphere of size parameter x and refractive index m (n + i k).
void mie_sphere(double x, cplx m, int na, const double* mu, double* qext, double* qsca, double* gq, double* s11) {
  int nstop = (int)(x + 4.0 * std::cbrt(x) + 2.0);
  cplx mx = m * x;
  int nmx = std::max((int)std::abs(mx), nstop) + 16;
  std::vector<cplx> D(nmx + 1);
  D[nmx] = cplx(0.0, 0.0);
  for (int n = nmx; n >= 1; --n) {
    cplx rn = (double)n / mx;
    D[n - 1] = rn - 1.0 / (D[n] + rn);
  }
  std::vector<cplx> a(nstop + 1), b(nstop + 1);
  double psi0 = std::cos(x), psi1 = std::sin(x);
  double chi0 = -std::sin(x), chi1 = std::cos(x);
  cplx xi1(psi1, -chi1);
  double ext = 0.0, sca = 0.0, gsum = 0.0;
  for (int n = 1; n <= nstop; ++n) {
    double fn = (double)n;
    double psi = (2.0 * fn - 1.0) * psi1 / x - psi0;
    double chi = (2.0 * fn - 1.0) * chi1 / x - chi0;
    cplx xi(psi, -chi);
    cplx da = D[n] / m + fn / x, db = D[n] * m + fn / x;
    a[n] = (da * psi - psi1) / (da * xi - xi1);
    b[n] = (db * psi - psi1) / (db * xi - xi1);
    ext += (2.0 * fn + 1.0) * (a[n].real() + b[n].real());
    sca += (2.0 * fn + 1.0) * (std::norm(a[n]) + std::norm(b[n]));
    if (n > 1) {
      double fn1 = fn - 1.0;
      gsum += (fn1 * (fn1 + 2.0) / (fn1 + 1.0)) * (a[n - 1] * std::conj(a[n]) + b[n - 1] * std::conj(b[n])).real() +
              ((2.0 * fn1 + 1.0) / (fn1 * (fn1 + 1.0))) * (a[n - 1] * std::conj(b[n - 1])).real();
    }
    psi0 = psi1; psi1 = psi; chi0 = chi1; chi1 = chi; xi1 = cplx(psi1, -chi1);
  }
  {
    double fn = (double)nstop;
    gsum += ((2.0 * fn + 1.0) / (fn * (fn + 1.0))) * (a[nstop] * std::conj(b[nstop])).real();
  }
  *qext = 2.0 / (x * x) * ext;
  *qsca = 2.0 / (x * x) * sca;
  *gq = 4.0 / (x * x) * gsum;  // = Qsca * g
  for (int k = 0; k < na; ++k) {
    double pim1 = 0.0, pin = 1.0;
    cplx S1(0.0, 0.0), S2(0.0, 0.0);
    for (int n = 1; n <= nstop; ++n) {
      double fn = (double)n;
      double tau = fn * mu[k] * pin - (fn + 1.0) * pim1;
      double f = (2.0 * fn + 1.0) / (fn * (fn + 1.0));
      S1 += f * (a[n] * pin + b[n] * tau);
      S2 += f * (a[n] * tau + b[n] * pin);
      double pnext = ((2.0 * fn + 1.0) * mu[k] * pin - (fn + 1.0) * pim1) / fn;
      pim1 = pin;
      pin = pnext;
    }
    s11[k] = 0.5 * (std::norm(S1) + std::norm(S2));
  }
}

}  // namespace

extern "C" {

// One species: lognormal number distributions (dry mode radius rg_um[b],
// geometric std sigma_g[b]) of spheres with dry refractive index nr - i ni and
// dry density rho_dry [kg m-3]; hygroscopic growth factor (1-RH)^-0.2 and
// volume-mixed water (1.33 - 0i) when `hygroscopic`.  Outputs (float, Fortran
// order): bext, bsca, g (nrh, nlam, nbin) [m2 kg-1]; pmom (nrh, nlam, nbin, nmom).
// Returns 0 on success.
int aerort_miegen_lognormal(int nlam, const double* lam_um, int nrh, const double* rh, int nbin,
                            const double* rg_um, const double* sigma_g, double nr, double ni, int hygroscopic,
                            double rho_dry, int nmom, int nradii, float* bext, float* bsca, float* g,
                            float* pmom) {
  if (nlam <= 0 || nrh <= 0 || nbin <= 0 || nmom < 1 || nradii < 8) return 1;
  const int na = 2 * nmom + 32;
  std::vector<double> mu(na), wa(na);
  gauss_legendre(na, mu.data(), wa.data());
  // common dry-radius grid covering +-3 sigma of every bin
  double lnmin = 1e30, lnmax = -1e30;
  for (int b = 0; b < nbin; ++b) {
    double ls = std::log(sigma_g[b]);
    lnmin = std::min(lnmin, std::log(rg_um[b]) - 3.0 * ls);
    lnmax = std::max(lnmax, std::log(rg_um[b]) + 3.0 * ls);
  }
  const double dln = (lnmax - lnmin) / (nradii - 1);
  const cplx mdry(nr, ni), mwater(1.33, 0.0);
  const int ntask = nrh * nlam;
#pragma omp parallel for schedule(dynamic, 1)
  for (int task = 0; task < ntask; ++task) {
    const int ir = task % nrh, il = task / nrh;
    const double gf = hygroscopic ? std::pow(1.0 - std::min(rh[ir], 0.995), -0.2) : 1.0;
    const cplx m = mwater + (mdry - mwater) / (gf * gf * gf);
    std::vector<double> cext(nradii), csca(nradii), cg(nradii), s11((size_t)nradii * na);
    for (int k = 0; k < nradii; ++k) {
      double rdry = std::exp(lnmin + dln * k);  // um
      double rwet = rdry * gf;
      double x = 2.0 * M_PI * rwet / lam_um[il];
      double qe, qs, gq;
      mie_sphere(x, m, na, mu.data(), &qe, &qs, &gq, &s11[(size_t)k * na]);
      double area = M_PI * (rwet * 1e-6) * (rwet * 1e-6);
      cext[k] = qe * area;
      csca[k] = qs * area;
      cg[k] = gq * area;
    }
    for (int b = 0; b < nbin; ++b) {
      const double lrg = std::log(rg_um[b]), ls = std::log(sigma_g[b]);
      double se = 0.0, ss = 0.0, sg = 0.0, smass = 0.0;
      std::vector<double> p11(na, 0.0);
      for (int k = 0; k < nradii; ++k) {
        double lr = lnmin + dln * k;
        double z = (lr - lrg) / ls;
        if (std::fabs(z) > 3.0) continue;
        double wk = std::exp(-0.5 * z * z) * dln;  // dN/dlnr (unnormalised) * dlnr
        double rdry = std::exp(lr) * 1e-6;
        se += wk * cext[k];
        ss += wk * csca[k];
        sg += wk * cg[k];
        smass += wk * rho_dry * (4.0 / 3.0) * M_PI * rdry * rdry * rdry;
        for (int a = 0; a < na; ++a) p11[a] += wk * s11[(size_t)k * na + a];
      }
      size_t o = (size_t)ir + (size_t)nrh * (il + (size_t)nlam * b);
      bext[o] = (float)(se / smass);
      bsca[o] = (float)(ss / smass);
      g[o] = (float)(ss > 0.0 ? sg / ss : 0.0);
      // Legendre moments of the normalised phase function
      double norm = 0.0;
      for (int a = 0; a < na; ++a) norm += 0.5 * wa[a] * p11[a];
      std::vector<double> mom(nmom, 0.0);
      for (int a = 0; a < na; ++a) {
        double p0 = 1.0, p1 = mu[a], f = 0.5 * wa[a] * p11[a] / norm;
        mom[0] += f * p0;
        if (nmom > 1) mom[1] += 3.0 * f * p1;
        for (int l = 2; l < nmom; ++l) {
          double p2 = ((2.0 * l - 1.0) * mu[a] * p1 - (l - 1.0) * p0) / l;
          mom[l] += (2.0 * l + 1.0) * f * p2;
          p0 = p1;
          p1 = p2;
        }
      }
      size_t s3 = (size_t)nrh * nlam * nbin;
      for (int l = 0; l < nmom; ++l) pmom[o + s3 * l] = (float)mom[l];
    }
  }
  return 0;
}

}  // extern "C"
