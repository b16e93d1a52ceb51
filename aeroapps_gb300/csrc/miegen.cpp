// Synthetic Mie tables: Lorenz-Mie series (Bohren & Huffman 1983, ch. 4 and
// appendix A; term count after Wiscombe 1980) integrated over lognormal size
// distributions, with hygroscopic growth, producing the fields of the
// reference's Chem_MieTable (src/Shared/GMAO_Shared/Chem_Base/Chem_MieTableMod.F90:55-83):
// mass extinction / scattering efficiency per kg of DRY aerosol, asymmetry
// parameter and Legendre expansion coefficients beta_l of the phase function
// normalised so that beta_0 = 1 (beta_1 = 3 g), in the table layout
// (nrh, nlambda, nbin, nmom), or the six Greek-coefficient sequences of the
// scattering matrix (nrh, nlambda, nbin, nmom, 6).  Host code; used only to
// build input data.
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

// Efficiencies and the scattering-matrix elements of a homogeneous sphere of
// size parameter x and refractive index m (n + i k) at angle cosines mu[0..na):
// s11 = (|S1|^2 + |S2|^2)/2 and, when s12 is given, s12 = (|S1|^2 - |S2|^2)/2,
// s33 = Re(S1 S2*), s34 = Im(S1 S2*) (Bohren & Huffman 1983, eq. 4.77; the
// signs make the Rayleigh limit match the Greek coefficients the reference
// mixes in for Rayleigh scattering, VLIDORT_ScatMod.F90:446-480).
void mie_sphere(double x, cplx m, int na, const double* mu, double* qext, double* qsca, double* gq, double* s11,
                double* s12 = nullptr, double* s33 = nullptr, double* s34 = nullptr) {
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
    if (s12) {
      s12[k] = 0.5 * (std::norm(S1) - std::norm(S2));
      const cplx c = S1 * std::conj(S2);
      s33[k] = c.real();
      s34[k] = c.imag();
    }
  }
}

// Expansion coefficients of a scattering matrix of spheres (F22 = F11, F44 =
// F33) in generalized spherical functions (de Rooij & van der Stap 1984,
// A&A 131, 237): alpha1 from F11 and P^l_00, beta1 from F12 and P^l_02, alpha2
// + alpha3 from F22 + F33 and P^l_22, alpha2 - alpha3 from F22 - F33 and
// P^l_2-2, alpha4 from F44 and P^l_00, beta2 from F34 and P^l_02; P^l_02 with
// the sign of the reference's single-scatter functions (-sqrt(6)/4 (1 - mu^2)
// at l = 2, FO_VectorSS_Spherfuncs.f90), so that the Rayleigh limit gives its
// gamma2 = -sqrt(6)(1-d)/(2+d).  Normalised by the F11 integral (alpha1_0 = 1).
// out[e * nmom + l], e = 0..5: alpha1, beta1, alpha3, beta2, alpha2, alpha4
// (the P11, P12, P33, P34, P22, P44 order of the reference's tables).
void greek_expand(int na, const double* mu, const double* wa, const double* f11, const double* f12,
                  const double* f33, const double* f34, int nmom, double* out) {
  double norm = 0.0;
  for (int a = 0; a < na; ++a) norm += 0.5 * wa[a] * f11[a];
  for (int i = 0; i < 6 * nmom; ++i) out[i] = 0.0;
  for (int a = 0; a < na; ++a) {
    const double x = mu[a], w = 0.5 * wa[a] / norm;
    double p00m = 0.0, p00 = 1.0;                 // P^l_00 at l-1, l
    double p02m = 0.0, p02 = 0.0, sql41 = 0.0;    // P^l_02
    double ppm = 0.0, pp = 0.0, pmm = 0.0, pm = 0.0;  // P^l_22, P^l_2-2
    for (int l = 0; l < nmom; ++l) {
      if (l == 1) { p00m = p00; p00 = x; }
      else if (l >= 2) {
        const double t = ((2.0 * l - 1.0) * x * p00 - (l - 1.0) * p00m) / l;
        p00m = p00; p00 = t;
      }
      if (l == 2) {
        p02 = -0.25 * std::sqrt(6.0) * (1.0 - x) * (1.0 + x);
        p02m = 0.0;
        pp = 0.25 * (1.0 + x) * (1.0 + x);
        pm = 0.25 * (1.0 - x) * (1.0 - x);
        ppm = pmm = 0.0;
        sql41 = 0.0;
      } else if (l > 2) {
        const double dl = l, sql4 = sql41;
        sql41 = std::sqrt(dl * dl - 4.0);
        const double t02 = ((2.0 * dl - 1.0) / sql41) * x * p02 - (sql4 / sql41) * p02m;
        p02m = p02; p02 = t02;
        const double perll4 = 1.0 / (dl - 1.0) / (dl * dl - 4.0);
        const double g5 = (2.0 * dl - 1.0) * dl * (dl - 1.0) * perll4, g6 = (2.0 * dl - 1.0) * 4.0 * perll4;
        const double g7 = dl * ((dl - 1.0) * (dl - 1.0) - 4.0) * perll4;
        const double tp = (g5 * x - g6) * pp - g7 * ppm;
        const double tm = (g5 * x + g6) * pm - g7 * pmm;
        ppm = pp; pp = tp; pmm = pm; pm = tm;
      }
      const double c = (2.0 * l + 1.0) * w;
      out[0 * nmom + l] += c * f11[a] * p00;
      out[5 * nmom + l] += c * f33[a] * p00;
      if (l >= 2) {
        out[1 * nmom + l] += c * f12[a] * p02;
        out[3 * nmom + l] += c * f34[a] * p02;
        const double sum23 = c * (f11[a] + f33[a]) * pp, dif23 = c * (f11[a] - f33[a]) * pm;
        out[4 * nmom + l] += 0.5 * (sum23 + dif23);  // alpha2
        out[2 * nmom + l] += 0.5 * (sum23 - dif23);  // alpha3
      }
    }
  }
}

}  // namespace

extern "C" {

int aerort_miegen_lognormal_pol(int nlam, const double* lam_um, int nrh, const double* rh, int nbin,
                                const double* rg_um, const double* sigma_g, double nr, double ni, int hygroscopic,
                                double rho_dry, int nmom, int npol, int nradii, float* bext, float* bsca, float* g,
                                float* pmom);

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
  return aerort_miegen_lognormal_pol(nlam, lam_um, nrh, rh, nbin, rg_um, sigma_g, nr, ni, hygroscopic, rho_dry, nmom,
                                     1, nradii, bext, bsca, g, pmom);
}

// As aerort_miegen_lognormal with npol = 1 (P11 Legendre moments) or npol = 6
// (pmom (nrh, nlam, nbin, nmom, 6): the expansion coefficients of P11, P12,
// P33, P34, P22, P44, see greek_expand).
int aerort_miegen_lognormal_pol(int nlam, const double* lam_um, int nrh, const double* rh, int nbin,
                                const double* rg_um, const double* sigma_g, double nr, double ni, int hygroscopic,
                                double rho_dry, int nmom, int npol, int nradii, float* bext, float* bsca, float* g,
                                float* pmom) {
  if (nlam <= 0 || nrh <= 0 || nbin <= 0 || nmom < 1 || nradii < 8 || (npol != 1 && npol != 6)) return 1;
  // angular quadrature of the moment integrals: fixed at 512 nodes (up to
  // 240 moments), so a table's first moments do not depend on how many it
  // holds, and fine enough for the diffraction peak of the largest wet
  // particles (size parameter ~270 at 470 nm)
  const int na = std::max(2 * nmom + 32, 512);
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
    std::vector<double> s12, s33, s34;
    if (npol == 6) { s12.resize((size_t)nradii * na); s33.resize((size_t)nradii * na); s34.resize((size_t)nradii * na); }
    for (int k = 0; k < nradii; ++k) {
      double rdry = std::exp(lnmin + dln * k);  // um
      double rwet = rdry * gf;
      double x = 2.0 * M_PI * rwet / lam_um[il];
      double qe, qs, gq;
      if (npol == 6)
        mie_sphere(x, m, na, mu.data(), &qe, &qs, &gq, &s11[(size_t)k * na], &s12[(size_t)k * na],
                   &s33[(size_t)k * na], &s34[(size_t)k * na]);
      else
        mie_sphere(x, m, na, mu.data(), &qe, &qs, &gq, &s11[(size_t)k * na]);
      double area = M_PI * (rwet * 1e-6) * (rwet * 1e-6);
      cext[k] = qe * area;
      csca[k] = qs * area;
      cg[k] = gq * area;
    }
    for (int b = 0; b < nbin; ++b) {
      const double lrg = std::log(rg_um[b]), ls = std::log(sigma_g[b]);
      double se = 0.0, ss = 0.0, sg = 0.0, smass = 0.0;
      std::vector<double> p11(na, 0.0), p12(na, 0.0), p33(na, 0.0), p34(na, 0.0);
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
        if (npol == 6)
          for (int a = 0; a < na; ++a) {
            p12[a] += wk * s12[(size_t)k * na + a];
            p33[a] += wk * s33[(size_t)k * na + a];
            p34[a] += wk * s34[(size_t)k * na + a];
          }
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
      if (npol == 6) {
        std::vector<double> gk((size_t)6 * nmom);
        greek_expand(na, mu.data(), wa.data(), p11.data(), p12.data(), p33.data(), p34.data(), nmom, gk.data());
        for (int e = 0; e < 6; ++e)
          for (int l = 0; l < nmom; ++l) pmom[o + s3 * (l + (size_t)nmom * e)] = (float)gk[(size_t)e * nmom + l];
      } else {
        for (int l = 0; l < nmom; ++l) pmom[o + s3 * l] = (float)mom[l];
      }
    }
  }
  return 0;
}

}  // extern "C"
