// One scalar solve (column x wavelength) in the AeroApps VLIDORT_Scalar_Lambert
// configuration, executed by a single thread.  See rt_scalar.cuh for the
// mapping rationale.  Reference routines are cited per block.
#pragma once
#include "rt_scalar.cuh"

namespace aerort {

// Device view of the VLIDORT_Scalar_Lambert argument list
// (src/Components/rtms/geo_vlidort/VLIDORT_LAMBERT.F90:34-95), Fortran
// column-major arrays, FP64.
struct LambertInputs {
  int km, nch, nobs, nmom;
  const double* rot;     // (km, nobs, nch)
  const double* depol;   // (nch)
  const double* tau;     // (km, nch, nobs)
  const double* ssa;     // (km, nch, nobs)
  const double* pmom;    // (km, nch, nobs, nMom, nPol); P11 moments are ipol = 1
  const double* he;      // (km+1, nobs) heights [m]
  const double* albedo;  // (nobs, nch)
  const double* sza;     // (nobs)
  const double* raa;     // (nobs)
  const double* vza;     // (nobs)
  // Optional extensions (null = reference behaviour):
  const int* nlay;       // (nobs) layers of each column, <= km; the column uses the first nlay entries
  const float* tau_f;    // FP32 optics straight from VLIDORT_getAOPvector (replaces tau/ssa/pmom;
  const float* ssa_f;    //   the conversion to FP64 is the driver's dble(), geo_vlidort.F90:598-601)
  const float* pmom_f;
  // Sticky nadir-FO flag (VLIDORT_ScatMod.F90:1123-1126): index of the first
  // pixel in loop order that reaches the solver with solar_zenith == 0; every
  // pixel from there on uses the nadir (regular pseudo-spherical) correction.
  const int* nadir_first;  // device scalar, nobs if never triggered; may be null
  double missing;
};

// Scratch element counts per thread for a solve with at most L layers.
template <int NS>
struct ScratchLayout {
  static constexpr int NMX = 2 * NS;  // NMOMENTS + 1 <= 2 NS
  long og, lnz, dtau, avsec, itrans, tmubar, tuser, emult, ext, escat, hgt, F, f, C, c, a, b, s, total;
  RT_HD explicit ScratchLayout(int L) {
    long o = 0;
    og = o; o += (long)NMX * L;
    lnz = o; o += L;
    dtau = o; o += L; avsec = o; o += L; itrans = o; o += L; tmubar = o; o += L;
    tuser = o; o += L; emult = o; o += L; ext = o; o += L; escat = o; o += L; hgt = o; o += L + 1;
    F = o; o += (long)NS * NS * L; f = o; o += (long)NS * L;
    C = o; o += (long)NS * NS * L; c = o; o += (long)NS * L;
    a = o; o += (long)NS * L; b = o; o += (long)NS * L; s = o; o += L;
    total = o;
  }
};

// Per-solve constants kept in registers / local memory.
template <int NS>
struct SolveCtx {
  int L, NM, cutoff;
  bool msmode, refl_directbeam;
  double qx[NS], qw[NS], sqw[NS];
  double mu_u, sec_u, cos_sza, albedo, trans_solar_beam;
  double pimm_q[NS], pimm_u, pimm_0;  // P_m^m recursion state carried across Fourier terms
};

// Homogeneous + particular solution of one layer for one Fourier term.
template <int NS>
struct LayerSol {
  double P[NS * NS];  // eigenvector components, downwelling streams (X+ rows 1..N)
  double Q[NS * NS];  // eigenvector components, upwelling streams   (X+ rows N+1..2N)
  double t[NS];       // exp(-k dtau)
  double wt[2 * NS];  // particular solution at layer top    (down 0..N-1, up N..2N-1)
  double wb[2 * NS];  // particular solution at layer bottom
};

// Associated Legendre functions normalised as the reference's PI matrices
// (vlidort_miscsetups.f90:2273-2932, NSTOKES = 1) for Fourier term m at
// cosine x; out[l] for l = m..NM, zero below m.  pim carries P_m^m between
// successive Fourier terms.
RT_HD void legendre_m(int m, int NM, double x, double* pim, double* out) {
  for (int l = 0; l < m && l <= NM; ++l) out[l] = 0.0;
  if (m > NM) return;
  double umxsq = 1.0 - x * x;
  double rt = (x == 1.0) ? 0.0 : sqrt(umxsq);
  double pm1 = 0.0, p = 0.0;
  if (m == 0) {
    pm1 = 1.0; out[0] = 1.0;
    if (NM >= 1) { p = x; out[1] = x; }
    if (NM >= 2) { pm1 = x; p = 0.5 * (3.0 * x * x - 1.0); out[2] = p; }
    for (int l = 2; l <= NM - 1; ++l) {
      double pn = (x * (double)(2 * l + 1) * p - (double)l * pm1) * (1.0 / (double)(l + 1));
      pm1 = p; p = pn; out[l + 1] = pn;
    }
  } else if (m == 1) {
    p = rt; out[1] = rt;
    if (NM >= 2) { pm1 = rt; p = 3.0 * (rt * x); out[2] = p; }
    for (int l = 2; l <= NM - 1; ++l) {
      double pn = (x * (double)(2 * l + 1) * p - (double)(l + 1) * pm1) * (1.0 / (double)l);
      pm1 = p; p = pn; out[l + 1] = pn;
    }
  } else {
    if (m == 2) *pim = 3.0 * umxsq;
    else *pim = (double)(2 * m - 1) * rt * (*pim);
    p = *pim; out[m] = p;
    if (m < NM) { pm1 = p; p = x * (double)(2 * m + 1) * p; out[m + 1] = p; }
    for (int l = m + 1; l <= NM - 1; ++l) {
      double pn = (x * (double)(2 * l + 1) * p - (double)(l + m) * pm1) * (1.0 / (double)(l + 1 - m));
      pm1 = p; p = pn; out[l + 1] = pn;
    }
  }
  // normalisation sqrt((l-m)!/(l+m)!)
  double fac = 1.0;
  for (int l = 1; l <= 2 * m; ++l) fac *= (double)l;
  double phi = 1.0 / fac;
  out[m] *= sqrt(phi);
  for (int l = m + 1; l <= NM; ++l) {
    phi = phi * ((double)(l - m) / (double)(l + m));
    out[l] *= sqrt(phi);
  }
}

// Layer eigen-solution (vlidort_solutions.f90:150-1047, VLIDORT_QHOM_SOLUTION).
// The reference forms EIGENMAT = DAB*SAB and solves the nonsymmetric problem
// with ASYMTX.  Here the same eigenpairs are found from a symmetric problem:
// with W = diag(w), M = diag(mu), SAB = M^-1 W^-1/2 As W^1/2 and
// DAB = M^-1 W^-1/2 Bs W^1/2 where As, Bs are symmetric, so
// DAB*SAB ~ (M^-1 Bs M^-1) As.  With Bs = Lb Lb^T and R = M^-1 Lb,
// H = R^T As R is symmetric with the same eigenvalues k^2, and an eigenvector
// q of H maps to x = W^-1/2 R q.  Bs (odd-parity part) is well conditioned
// even for conservative scattering, so its Cholesky factor is always safe.
template <int NS>
RT_HD int layer_eigen(const SolveCtx<NS>& c, int m, double dtau, const double* og, const double* piq,
                      LayerSol<NS>& ls, double* kv, double* Sp) {
  const int N = NS, NM = c.NM;
  double Bs[NS * NS], H[NS * NS], V[NS * NS], lam[NS];
  // Sp (even l-m) and Sm (odd l-m) contractions of omega*beta_l P_l(mu_i) P_l(mu_j)
  for (int j = 0; j < N; ++j)
    for (int i = 0; i <= j; ++i) {
      double se = 0.0, so = 0.0;
      for (int l = m; l <= NM; ++l) {
        double t = og[l] * piq[l + 2 * NS * i] * piq[l + 2 * NS * j];
        if (((l - m) & 1) == 0) se += t; else so += t;
      }
      Sp[i + NS * j] = se; Sp[j + NS * i] = se;
      double b = -c.sqw[i] * c.sqw[j] * so;
      if (i == j) b += 1.0;
      Bs[i + NS * j] = b; Bs[j + NS * i] = b;
    }
  if (!cholesky<NS>(N, Bs)) return RT_EIGEN_FAIL;
  // R = M^-1 Lb (lower triangular)
  for (int j = 0; j < N; ++j)
    for (int i = j; i < N; ++i) Bs[i + NS * j] /= c.qx[i];
  // Y = As R with As = I - W^1/2 Sp W^1/2 ; H = R^T Y
  for (int j = 0; j < N; ++j)
    for (int i = 0; i < N; ++i) {
      double y = Bs[i + NS * j] * ((i >= j) ? 1.0 : 0.0);
      double s = 0.0;
      for (int k = j; k < N; ++k) s += c.sqw[i] * Sp[i + NS * k] * c.sqw[k] * Bs[k + NS * j];
      V[i + NS * j] = y - s;  // V used as temporary for Y
    }
  for (int j = 0; j < N; ++j)
    for (int i = 0; i <= j; ++i) {
      double s = 0.0;
      for (int k = i; k < N; ++k) s += Bs[k + NS * i] * V[k + NS * j];
      H[i + NS * j] = s; H[j + NS * i] = s;
    }
  if (!sym_eigen<NS>(N, H, V, lam)) return RT_EIGEN_FAIL;
  // As = La La^T: the eigenvalues are recomputed as Rayleigh quotients
  // lam = q^T R^T As R q = |La^T (R q)|^2, which keeps full relative accuracy
  // for the small eigenvalues of nearly conservative layers (forming H
  // explicitly leaves them an absolute error of order eps*|H|).
  for (int j = 0; j < N; ++j)
    for (int i = j; i < N; ++i) {
      double a = -c.sqw[i] * Sp[i + NS * j] * c.sqw[j];
      if (i == j) a += 1.0;
      H[i + NS * j] = a;
    }
  if (!cholesky<NS>(N, H)) return RT_EIGEN_FAIL;
  for (int a = 0; a < N; ++a) {
    // v = R q ; sum vector x = W^-1/2 v, unit 2-norm
    double x[NS], v[NS], nrm = 0.0;
    for (int i = 0; i < N; ++i) {
      double s = 0.0;
      for (int j = 0; j <= i; ++j) s += Bs[i + NS * j] * V[j + NS * a];
      v[i] = s;
      x[i] = s / c.sqw[i];
      nrm += x[i] * x[i];
    }
    double qq = 0.0, lr = 0.0;
    for (int i = 0; i < N; ++i) {
      qq += V[i + NS * a] * V[i + NS * a];
      double w = 0.0;
      for (int j = i; j < N; ++j) w += H[j + NS * i] * v[j];
      lr += w * w;
    }
    lr /= qq;
    if (!(lr > 0.0)) return RT_EIGEN_FAIL;
    double k = sqrt(lr);
    kv[a] = k;
    nrm = 1.0 / sqrt(nrm);
    for (int i = 0; i < N; ++i) x[i] *= nrm;
    // difference vector SAB x / k ; SAB(i,j) = (delta_ij - w_j Sp(i,j)) / mu_i
    double invk = 1.0 / k;
    for (int i = 0; i < N; ++i) {
      double s = 0.0;
      for (int j = 0; j < N; ++j) s += c.qw[j] * Sp[i + NS * j] * x[j];
      double dif = (x[i] - s) / c.qx[i] * invk;
      ls.P[i + NS * a] = 0.5 * (x[i] + dif);
      ls.Q[i + NS * a] = 0.5 * (x[i] - dif);
    }
    double help = k * dtau;
    ls.t[a] = help > kMaxTau ? 0.0 : exp(-help);
  }
  return RT_OK;
}

// Solution pieces of one layer for Fourier term m: eigen-solution, user-angle
// homogeneous and particular terms (vlidort_solutions.f90:1051-1163, 1167-1505,
// 1651-1790, 2649-3073; PostProcessing.f90:139-451).  Writes the per-layer
// source coefficients a, b, s (TOA radiance = sum_n Tcum_n (L.a + M.b + s)).
template <int NS>
RT_HD int layer_solution(const SolveCtx<NS>& c, const RtOptions& opt, int m, int n, bool laysc,
                         const Scratch& S, const ScratchLayout<NS>& lay, const double* piq, const double* piu,
                         const double* pi0, LayerSol<NS>& ls) {
  const int N = NS, NM = c.NM, L = c.L;
  double og[2 * NS], kv[NS], Sp[NS * NS];
  for (int l = 0; l <= NM; ++l) og[l] = (l >= m) ? S[lay.og + l + 2 * NS * (long)n] : 0.0;
  const double dtau = S[lay.dtau + n];
  int st = layer_eigen<NS>(c, m, dtau, og, piq, ls, kv, Sp);
  if (st != RT_OK) return st;
  const double tuser = S[lay.tuser + n];
  const double smu = c.sec_u;
  double uh_dn[NS], uh_up[NS], hm1[NS], hm2[NS], norm[NS];
  for (int a = 0; a < N; ++a) {
    // user-angle homogeneous solutions
    double dn = 0.0, up = 0.0;
    for (int l = m; l <= NM; ++l) {
      double sgn = ((l - m) & 1) ? -1.0 : 1.0;
      double sps = 0.0;
      for (int j = 0; j < N; ++j) sps += 0.5 * c.qw[j] * piq[l + 2 * NS * j] * (ls.P[j + NS * a] + sgn * ls.Q[j + NS * a]);
      double h = og[l] * sps;
      dn += sgn * piu[l] * h;
      up += piu[l] * h;
    }
    uh_dn[a] = laysc ? dn : 0.0;
    uh_up[a] = laysc ? up : 0.0;
    // homogeneous multipliers
    double zdel = ls.t[a];
    double rho_p = smu + kv[a], rho_m = smu - kv[a];
    hm2[a] = smu * (1.0 - zdel * tuser) * (1.0 / rho_p);
    if (fabs(rho_m) < kTaylorSmall) hm1[a] = taylor1(opt.taylor_order, rho_m, dtau, tuser, smu);
    else hm1[a] = smu * (zdel - tuser) * (1.0 / rho_m);
    double nr = 0.0;
    for (int j = 0; j < N; ++j) nr += c.qx[j] * c.qw[j] * (ls.P[j + NS * a] * ls.P[j + NS * a] - ls.Q[j + NS * a] * ls.Q[j + NS * a]);
    norm[a] = nr;
  }
  for (int a = 0; a < N; ++a) {
    S[lay.a + a + N * (long)n] = uh_dn[a] * hm2[a];
    S[lay.b + a + N * (long)n] = uh_up[a] * hm1[a];
  }
  for (int i = 0; i < 2 * N; ++i) { ls.wt[i] = 0.0; ls.wb[i] = 0.0; }
  double spart = 0.0;
  const bool active = (n < c.cutoff) && laysc;
  if (active) {
    // Green's-function particular integral (VLIDORT_GBEAM_SOLUTION)
    const double F1 = opt.flux_factor / kPI4;
    const double secbar = S[lay.avsec + n], cnst = S[lay.itrans + n], wdel = S[lay.tmubar + n];
    double hq[2 * NS], dpi[NS], dmi[NS];
    for (int l = m; l <= NM; ++l) hq[l] = og[l] * pi0[l];
    double upar = 0.0;
    for (int l = m; l <= NM; ++l) upar += (F1 * hq[l]) * ((((l - m) & 1) ? -1.0 : 1.0) * piu[l]);
    for (int i = 0; i < N; ++i) {
      double sp = 0.0, sm = 0.0;
      for (int l = m; l <= NM; ++l) {
        double t = piq[l + 2 * NS * i] * hq[l];
        sp += t;
        sm += (((l - m) & 1) ? -t : t);
      }
      dpi[i] = F1 * sp; dmi[i] = F1 * sm;
    }
    const double emult = S[lay.emult + n];
    const double itw = -cnst * wdel;
    const double sigp = secbar + smu;
    double gup[NS], gdn[NS];
    for (int a = 0; a < N; ++a) {
      double zdel = ls.t[a];
      double gp = secbar + kv[a], gm = secbar - kv[a];
      double cf = (fabs(gm) < kTaylorSmall) ? taylor1(opt.taylor_order, gm, dtau, wdel, cnst)
                                            : cnst * (zdel - wdel) / gm;
      double df = cnst * (1.0 - zdel * wdel) / gp;
      double s1 = 0.0, s2 = 0.0;
      for (int i = 0; i < N; ++i) {
        s1 += c.qw[i] * (dpi[i] * ls.P[i + NS * a] + dmi[i] * ls.Q[i + NS * a]);
        s2 += c.qw[i] * (dmi[i] * ls.P[i + NS * a] + dpi[i] * ls.Q[i + NS * a]);
      }
      double at = s1 / norm[a], bt = s2 / norm[a];
      gdn[a] = cf * at;
      gup[a] = df * bt;
      // user-angle particular source (WHOLELAYER_STERM_UP, Green's branch)
      double sd;
      if (fabs(gm) < kTaylorSmall) {
        double mult = taylor2(opt.taylor_order, gm, sigp, dtau, 1.0, wdel * tuser, 1.0);
        sd = (cnst * smu) * mult;
      } else {
        sd = (cnst * hm2[a] - emult) / gm;
      }
      double su = (itw * hm1[a] + emult) / gp;
      spart += uh_dn[a] * sd * at + uh_up[a] * su * bt;
    }
    for (int i = 0; i < N; ++i) {
      double wu1 = 0.0, wu2 = 0.0, wl1 = 0.0, wl2 = 0.0;
      for (int a = 0; a < N; ++a) {
        wu1 += gup[a] * ls.Q[i + NS * a]; wu2 += gup[a] * ls.P[i + NS * a];
        wl1 += gdn[a] * ls.P[i + NS * a]; wl2 += gdn[a] * ls.Q[i + NS * a];
      }
      ls.wt[i] = wu1; ls.wt[N + i] = wu2;
      ls.wb[i] = wl1; ls.wb[N + i] = wl2;
    }
    if (!c.msmode) spart += upar * emult;
  }
  S[lay.s + n] = laysc ? spart : 0.0;
  return RT_OK;
}

// One Fourier term of the TOA upwelling radiance (VLIDORT_FOURIER,
// vlidort_masters_V2p8p3.f90:3107).  The boundary-value problem the reference
// assembles as a banded matrix (bvproblem.f90:627-1284) and factorises with
// DGBTRF is solved here by a block sweep that never forms the band:
// top-down, each layer's L-coefficients are kept as an affine function of its
// M-coefficients (L_n = F_n M_n + f_n); each interface's 2N continuity
// conditions then give (M_{n-1}, L_n) in terms of M_n through one 2N x 2N
// pivoted solve; the surface condition closes the system and a bottom-up pass
// recovers all coefficients while accumulating the TOA source recursion
// (vlidort_intensity.f90:145-643).
template <int NS>
RT_HD int fourier_term(SolveCtx<NS>& c, const RtOptions& opt, int m, const Scratch& S, const ScratchLayout<NS>& lay,
                       double* out) {
  const int N = NS, NM = c.NM, L = c.L;
  const bool incl_surface = (m == 0) && (c.albedo != 0.0);
  const double surface_factor = (m == 0) ? 2.0 : 1.0;
  const double delta_factor = (m == 0) ? 1.0 : 2.0;
  const bool localbeam = incl_surface && c.refl_directbeam;
  double direct_beam = 0.0;
  if (localbeam) {
    double x0 = 4.0 * c.cos_sza / delta_factor;
    x0 = opt.flux_factor * x0 / kPI4;
    direct_beam = x0 * c.trans_solar_beam * c.albedo;
  }
  double piq[2 * NS * NS], piu[2 * NS], pi0[2 * NS];
  for (int i = 0; i < N; ++i) legendre_m(m, NM, c.qx[i], &c.pimm_q[i], &piq[2 * NS * i]);
  legendre_m(m, NM, c.mu_u, &c.pimm_u, piu);
  legendre_m(m, NM, c.cos_sza, &c.pimm_0, pi0);

  LayerSol<NS> A, B;
  LayerSol<NS>* prev = &A;
  LayerSol<NS>* cur = &B;
  double F[NS * NS], f[NS];
  double K[4 * NS * NS], R[2 * NS * (NS + 1)];
  for (int n = 0; n < L; ++n) {
    // DO_LAYER_SCATTERING(m, n) (vlidort_inputs.f90:4321-4330): false for m >= 3
    // when every input moment l = m..NMOMENTS of the layer is zero
    const bool lsc = (m < 3) || (m <= (int)S[lay.lnz + n]);
    int st = layer_solution<NS>(c, opt, m, n, lsc, S, lay, piq, piu, pi0, *cur);
    if (st != RT_OK) return st;
    if (n == 0) {
      // TOA: downwelling diffuse intensity vanishes -> L_1 = F_1 M_1 + f_1
      for (int j = 0; j < N; ++j)
        for (int i = 0; i < N; ++i) {
          K[i + 2 * NS * j] = cur->P[i + NS * j];
          R[i + 2 * NS * j] = -cur->Q[i + NS * j] * cur->t[j];
        }
      for (int i = 0; i < N; ++i) R[i + 2 * NS * N] = -cur->wt[i];
      if (!lu_solve<2 * NS>(N, K, R, N + 1)) return RT_BVP_SINGULAR;
      for (int j = 0; j < N; ++j)
        for (int i = 0; i < N; ++i) { F[i + NS * j] = R[i + 2 * NS * j]; S[lay.F + i + NS * j + (long)NS * NS * n] = F[i + NS * j]; }
      for (int i = 0; i < N; ++i) { f[i] = R[i + 2 * NS * N]; S[lay.f + i + NS * (long)n] = f[i]; }
    } else {
      // interface between layer n-1 (prev) and n (cur):
      // G M_{n-1} + g + Wb_{n-1} = X+_n L_n + X-_n T_n M_n + Wt_n
      double TF[NS * NS], tf[NS];
      for (int j = 0; j < N; ++j)
        for (int k = 0; k < N; ++k) TF[k + NS * j] = prev->t[k] * F[k + NS * j];
      for (int k = 0; k < N; ++k) tf[k] = prev->t[k] * f[k];
      for (int j = 0; j < N; ++j)
        for (int i = 0; i < N; ++i) {
          double gt = prev->Q[i + NS * j], gb = prev->P[i + NS * j];
          for (int k = 0; k < N; ++k) {
            gt += prev->P[i + NS * k] * TF[k + NS * j];
            gb += prev->Q[i + NS * k] * TF[k + NS * j];
          }
          K[i + 2 * NS * j] = gt;
          K[N + i + 2 * NS * j] = gb;
          K[i + 2 * NS * (N + j)] = -cur->P[i + NS * j];
          K[N + i + 2 * NS * (N + j)] = -cur->Q[i + NS * j];
          R[i + 2 * NS * j] = cur->Q[i + NS * j] * cur->t[j];
          R[N + i + 2 * NS * j] = cur->P[i + NS * j] * cur->t[j];
        }
      for (int i = 0; i < N; ++i) {
        double gt = 0.0, gb = 0.0;
        for (int k = 0; k < N; ++k) { gt += prev->P[i + NS * k] * tf[k]; gb += prev->Q[i + NS * k] * tf[k]; }
        R[i + 2 * NS * N] = cur->wt[i] - prev->wb[i] - gt;
        R[N + i + 2 * NS * N] = cur->wt[N + i] - prev->wb[N + i] - gb;
      }
      if (!lu_solve<2 * NS>(2 * N, K, R, N + 1)) return RT_BVP_SINGULAR;
      long oC = lay.C + (long)NS * NS * (n - 1), oc = lay.c + (long)NS * (n - 1);
      long oF = lay.F + (long)NS * NS * n, of = lay.f + (long)NS * n;
      for (int j = 0; j < N; ++j)
        for (int i = 0; i < N; ++i) {
          S[oC + i + NS * j] = R[i + 2 * NS * j];
          F[i + NS * j] = R[N + i + 2 * NS * j];
          S[oF + i + NS * j] = F[i + NS * j];
        }
      for (int i = 0; i < N; ++i) {
        S[oc + i] = R[i + 2 * NS * N];
        f[i] = R[N + i + 2 * NS * N];
        S[of + i] = f[i];
      }
    }
    LayerSol<NS>* t = prev; prev = cur; cur = t;
  }
  // surface: upwelling at the bottom = Lambertian reflection of the downwelling
  // diffuse field + reflected direct beam (bvproblem.f90:439-623, 1625-1739)
  const LayerSol<NS>& bl = *prev;
  const double kmult = incl_surface ? surface_factor * c.albedo : 0.0;
  double r2p[NS], r2m[NS], r2b = 0.0;
  for (int k = 0; k < N; ++k) {
    double sp = 0.0, sm = 0.0;
    for (int j = 0; j < N; ++j) { sp += c.qx[j] * c.qw[j] * bl.P[j + NS * k]; sm += c.qx[j] * c.qw[j] * bl.Q[j + NS * k]; }
    r2p[k] = sp * kmult; r2m[k] = sm * kmult;
  }
  for (int j = 0; j < N; ++j) r2b += c.qx[j] * c.qw[j] * bl.wb[j];
  r2b *= kmult;
  {
    for (int j = 0; j < N; ++j)
      for (int i = 0; i < N; ++i) {
        double s = bl.P[i + NS * j] - r2m[j];
        for (int k = 0; k < N; ++k) s += (bl.Q[i + NS * k] - r2p[k]) * bl.t[k] * F[k + NS * j];
        K[i + 2 * NS * j] = s;
      }
    for (int i = 0; i < N; ++i) {
      double s = -bl.wb[N + i] + r2b + (localbeam ? direct_beam : 0.0);
      for (int k = 0; k < N; ++k) s -= (bl.Q[i + NS * k] - r2p[k]) * bl.t[k] * f[k];
      R[i] = s;
    }
    if (!lu_solve<2 * NS>(N, K, R, 1)) return RT_BVP_SINGULAR;
  }
  double Mc[NS], Lc[NS], Mn[NS];
  for (int i = 0; i < N; ++i) Mc[i] = R[i];
  for (int i = 0; i < N; ++i) {
    double s = f[i];
    for (int k = 0; k < N; ++k) s += F[i + NS * k] * Mc[k];
    Lc[i] = s;
  }
  // bottom boundary source at the user angle (GET_BOA_SOURCE)
  double cum = 0.0;
  if (incl_surface) {
    double s = 0.0;
    for (int i = 0; i < N; ++i) {
      double h = bl.wb[i];
      for (int k = 0; k < N; ++k) h += Lc[k] * bl.P[i + NS * k] * bl.t[k] + Mc[k] * bl.Q[i + NS * k];
      s += c.qx[i] * c.qw[i] * h;
    }
    cum = kmult * s;
    const bool incl_directrf = localbeam && !opt.do_focorr && !c.msmode;
    if (incl_directrf) cum += direct_beam;
  }
  for (int n = L - 1; n >= 0; --n) {
    if (n < L - 1) {
      long oC = lay.C + (long)NS * NS * n, oc = lay.c + (long)NS * n;
      long oF = lay.F + (long)NS * NS * n, of = lay.f + (long)NS * n;
      for (int i = 0; i < N; ++i) {
        double s = S[oc + i];
        for (int k = 0; k < N; ++k) s += S[oC + i + NS * k] * Mc[k];
        Mn[i] = s;
      }
      for (int i = 0; i < N; ++i) {
        double s = S[of + i];
        for (int k = 0; k < N; ++k) s += S[oF + i + NS * k] * Mn[k];
        Lc[i] = s;
      }
      for (int i = 0; i < N; ++i) Mc[i] = Mn[i];
    }
    double src = S[lay.s + n];
    for (int k = 0; k < N; ++k) src += Lc[k] * S[lay.a + k + N * (long)n] + Mc[k] * S[lay.b + k + N * (long)n];
    cum = src + S[lay.tuser + n] * cum;
  }
  *out = delta_factor * cum;
  return RT_OK;
}

// Single-precision literals of the reference wrapper, widened exactly as the
// Fortran compiler widens them (VLIDORT_ScatMod.F90:1036,1128,1169; VLIDORT_Mod.F90 ACCURACY).
constexpr double kPiSingle = 3.1415927410125732421875;        // 4.*atan(1.0) in REAL*4
constexpr double kHeightScale = 0.001000000047497451305389404296875;  // 1.E-3
constexpr double kSsaCap = 0.999989986419677734375;            // 0.99999
constexpr double kAccuracySingle = 9.99999974737875163555145263671875e-05;  // 0.0001

// Sun path through layers 1..nn of a straight ray that leaves radius radstart
// with local solar zenith th (sine sth), layers ordered from TOA (index 0 of
// radii) down; returns sum_k ext_k * path_k.  Direct-sun and tangent-ray
// branches follow FO_geometry_Generic.f90:169-329 (FindSunPaths_D / _T).
RT_HD double sun_optical_path(bool zero_sun_boa, bool direct, double radstart, double th, double sth, int nn,
                              double R0, const Scratch& S, long ohgt, long oext, int L) {
  auto radius = [&](int k) { return R0 + S[ohgt + k]; };
  double tau = 0.0;
  if (direct) {
    if (zero_sun_boa) {
      tau += S[oext + nn - 1] * (radius(nn - 1) - radstart);
      for (int k = nn - 1; k >= 1; --k) tau += S[oext + k - 1] * (radius(k - 1) - radius(k));
      return tau;
    }
    double sth0 = sth, th0 = th;
    double sth1 = sth0 * radstart / radius(nn - 1), th1 = asin(sth1);
    tau += S[oext + nn - 1] * (sin(th0 - th1) * radstart / sth1);
    sth0 = sth1; th0 = th1;
    for (int k = nn - 1; k >= 1; --k) {
      sth1 = sth0 * radius(k) / radius(k - 1);
      th1 = asin(sth1);
      tau += S[oext + k - 1] * (sin(th0 - th1) * radius(k) / sth1);
      sth0 = sth1; th0 = th1;
    }
    return tau;
  }
  // tangent ray: passes its lowest point below the start level, then rises to TOA
  double tanr = sth * radstart;
  int k = nn - 1;
  bool trawl = true;
  while (k >= nn - 1 && trawl && k <= L) { trawl = (radius(k) > tanr); k = k + 1; }
  int nt = k - 1;
  double pnn = 0.0;
  if (nt > nn) {
    double th0 = kPIE - th, sth0 = sth;
    double sth1 = sth0 * radstart / radius(nn), th1 = asin(sth1);
    pnn = 2.0 * sin(th0 - th1) * radstart / sth1;
    sth0 = sth1; th0 = th1;
    for (int kk = nn + 1; kk <= nt - 1; ++kk) {
      sth1 = sth0 * radius(kk - 1) / radius(kk);
      th1 = asin(sth1);
      tau += S[oext + kk - 1] * (2.0 * sin(th0 - th1) * radius(kk) / sth0);
      sth0 = sth1; th0 = th1;
    }
    tau += S[oext + nt - 1] * (2.0 * sin(0.5 * kPIE - th0) * radius(nt - 1));
  } else if (nt == nn) {
    pnn = -2.0 * radstart * cos(th);
  }
  double th0 = kPIE - th, sth0 = sth;
  double sth1 = sth0 * radstart / radius(nn - 1), th1 = asin(sth1);
  tau += S[oext + nn - 1] * (pnn + sin(th0 - th1) * radstart / sth1);
  sth0 = sth1; th0 = th1;
  for (int kk = nn - 1; kk >= 1; --kk) {
    sth1 = sth0 * radius(kk) / radius(kk - 1);
    th1 = asin(sth1);
    tau += S[oext + kk - 1] * (sin(th0 - th1) * radius(kk) / sth1);
    sth0 = sth1; th0 = th1;
  }
  return tau;
}

// First-order single scatter (exact phase function) and direct surface bounce
// at TOA for one geometry (vlidort_focode: FO_SSWPgeometry_master.f90:101,
// FO_WPgeometry_Routines.f90:776-994 regular PS, :1511-1974 and :2409-2862
// enhanced PS with NFINE quadrature points per layer along the line of sight,
// FO_VectorSS_RTCalcs_I.f90:116-787).  Layer phase sums (escat) and
// extinctions (ext, per km) are in scratch.  Returns false on a degenerate path.
RT_HD bool fo_single_scatter(const RtOptions& opt, bool enhanced, int L, double sza, double vza, double phi,
                             double albedo, const double* tu, const double* wu, const Scratch& S, long ohgt, long oext,
                             long oescat, long odts, double* ss, double* db) {
  const double R0 = opt.earth_radius;
  auto radius = [&](int k) { return R0 + S[ohgt + k]; };
  const double flux = opt.flux_factor / kPI4;
  const bool overhead = (sza == 0.0);
  const double th_R = sza * kDTR;
  double cth, sthb;
  if (sza == 90.0) { cth = 0.0; sthb = 1.0; } else { sthb = sin(th_R); cth = cos(th_R); }
  double cum = 0.0, trans_above = 1.0, atten_boa = 0.0;
  if (!enhanced) {
    double ca = (vza == 90.0) ? 0.0 : cos(vza * kDTR);
    double tau_prev = 0.0, att_prev = 1.0;
    for (int n = 1; n <= L; ++n) {
      double st;
      if (opt.do_plane_parallel) {
        st = 0.0;
        for (int k = 1; k <= n; ++k) st += S[oext + k - 1] * ((S[ohgt + k - 1] - S[ohgt + k]) / cth);
      } else {
        st = sun_optical_path(overhead, true, radius(n), th_R, sthb, n, R0, S, ohgt, oext, L);
      }
      double att = st < kFoCutoff ? exp(-st) : 0.0;
      double lostrans = 0.0, mult = 0.0;
      if (ca > 0.0) {
        double lostau = S[odts + n - 1] / ca;
        if (lostau < kFoCutoff) lostrans = exp(-lostau);
        mult = (att_prev - att * lostrans) / (1.0 + (st - tau_prev) / lostau);
      }
      cum += trans_above * S[oescat + n - 1] * mult;
      trans_above *= lostrans;
      tau_prev = st; att_prev = att;
      if (n == L) atten_boa = att;
    }
    *ss = flux * cum;
    *db = flux * (4.0 * cth * albedo * atten_boa) * trans_above;
    return true;
  }
  const bool donadir = (vza == 0.0);
  double raycon = 0.0, alphaL = 0.0, caL = 1.0;
  if (!donadir) {
    alphaL = vza * kDTR;
    double sa = (vza == 90.0) ? 1.0 : sin(alphaL);
    caL = (vza == 90.0) ? 0.0 : cos(alphaL);
    raycon = sa * radius(L);
  }
  // solar direction at BOA (the y component does not enter: the line of sight lies in the x-z plane)
  double sdir0 = 0.0, sdir2 = 0.0;
  if (!overhead) { sdir0 = -sthb * cos(phi * kDTR); sdir2 = -cth; }
  auto findsun = [&](double rad, double cumangle, double* th, double* sth, bool* dirsun) {
    if (donadir) { *dirsun = true; *th = th_R; *sth = sin(th_R); return; }
    if (overhead) { *dirsun = true; *sth = sin(cumangle); *th = cumangle; return; }
    double b = (-rad * sin(cumangle)) * sdir0 + (rad * cos(cumangle)) * sdir2;
    double ct = -b / rad;
    *dirsun = (ct >= 0.0);
    *sth = sqrt(1.0 - ct * ct);
    *th = acos(ct);
  };
  // direct-sun attenuation at the surface (used by the direct bounce)
  {
    double st = sun_optical_path(overhead, true, radius(L), th_R, sthb, L, R0, S, ohgt, oext, L);
    atten_boa = st < kFoCutoff ? exp(-st) : 0.0;
  }
  // top-down accumulation of the line-of-sight source: TOA sees layer n through layers 1..n-1
  for (int n = 1; n <= L; ++n) {
    double r_up = radius(n - 1), r_lo = radius(n);
    double losw, cosa_lo;
    if (donadir) {
      losw = r_up - r_lo;
      cosa_lo = 1.0;
    } else {
      double ca_up = cos(asin(raycon / r_up));
      cosa_lo = (n == L) ? caL : cos(asin(raycon / r_lo));
      losw = r_up * ca_up - r_lo * cosa_lo;
    }
    const double kn = S[oext + n - 1];
    const double lostau = kn * losw;
    const double lostrans = lostau < kFoCutoff ? exp(-lostau) : 0.0;
    const bool zero_sun_boa = overhead && (n == L || donadir);
    double sum = 0.0;
    for (int j = 0; j < opt.nfine; ++j) {
      const double tf = losw * tu[j], wf = losw * wu[j];
      double rf, af = 0.0;
      if (donadir) {
        rf = r_lo + tf;
      } else {
        double tanf = raycon / (r_lo * cosa_lo + tf);
        af = atan(tanf);
        rf = raycon / sin(af);
      }
      double thf, sthf; bool dsf;
      findsun(rf, alphaL - af, &thf, &sthf, &dsf);
      double sd = sun_optical_path(zero_sun_boa, dsf, rf, thf, sthf, n, R0, S, ohgt, oext, L);
      double attf = sd < kFoCutoff ? exp(-sd) : 0.0;
      sum += attf * exp(-kn * (losw - tf)) * wf;
    }
    cum += trans_above * S[oescat + n - 1] * (sum * kn);
    trans_above *= lostrans;
  }
  *ss = flux * cum;
  *db = flux * (4.0 * cth * albedo * atten_boa) * trans_above;
  return true;
}

// Full solve of pixel (obs j, channel i) = solve index sidx = j * nch + i in the
// reference loop order (VLIDORT_LAMBERT.F90:106-165).  Writes radiance,
// reflectance, last Fourier index and status.  qx/qw: Gauss-Legendre streams on
// (0,1); tu/wu: unit fine-layer quadrature for the enhanced-PS line of sight.
template <int NS>
RT_HDN void solve_lambert(const RtOptions& opt, const LambertInputs& in, int sidx, const double* qx,
                          const double* qw, const double* tu, const double* wu, const Scratch& S, double* radiance,
                          double* reflectance, int* nfourier, int* status) {
  const int nch = in.nch, j = sidx / nch, i = sidx % nch;
  const long o = (long)j + (long)in.nobs * i;
  const int L = in.nlay ? in.nlay[j] : in.km, ngreek = in.nmom;
  const ScratchLayout<NS> lay(in.km);
  auto is_missing = [&](double x) { return fabs(x / in.missing - 1.0) < 0.001; };
  const double sza = in.sza[j], vza = in.vza[j], raa = in.raa[j], alb = in.albedo[o];
  if (nfourier) nfourier[o] = -1;
  if (status) status[o] = RT_OK;
  if (is_missing(sza) || is_missing(vza) || is_missing(raa) || is_missing(alb)) {
    radiance[o] = in.missing; reflectance[o] = in.missing;
    return;
  }
  SolveCtx<NS> c;
  c.L = L;
  c.NM = (2 * NS - 1 < ngreek) ? 2 * NS - 1 : ngreek;
  c.msmode = opt.do_focorr != 0;
  c.albedo = alb;
  for (int q = 0; q < NS; ++q) { c.qx[q] = qx[q]; c.qw[q] = qw[q]; c.sqw[q] = sqrt(qw[q]); c.pimm_q[q] = 0.0; }
  c.pimm_u = 0.0; c.pimm_0 = 0.0;
  c.mu_u = cos(kDTR * vza);
  c.sec_u = 1.0 / c.mu_u;
  c.cos_sza = cos(sza * kDTR);
  const int NM = c.NM;
  const bool nadir_fo = in.nadir_first ? (j >= *in.nadir_first) : false;
  // scattering angle for the exact single-scatter phase function
  double cosscat;
  {
    const double th_R = sza * kDTR;
    double cth, sthb;
    if (sza == 90.0) { cth = 0.0; sthb = 1.0; } else { sthb = sin(th_R); cth = cos(th_R); }
    double ca, sa;
    if (vza == 90.0) { ca = 0.0; sa = 1.0; } else { ca = cos(vza * kDTR); sa = sin(vza * kDTR); }
    double phi = raa;
    if (phi < 0.0) phi = -phi;
    if (phi > 360.0) phi = 360.0 - phi - 360.0;
    if (sza == 0.0) { cosscat = -ca; if (ca == 0.0) cosscat = ca; }
    else cosscat = -ca * cth + sa * sthb * cos(phi * kDTR);
  }
  // ---------------------------------------------------------------- layer mixing + delta-M
  // VLIDORT_ScatMod.F90:1138-1204 (Rayleigh + aerosol Greek moments, SSA cap),
  // vlidort_miscsetups.f90:370-760 (delta-M, omega / first-moment clamps, SSALBINIT)
  const double dep = in.depol[i];
  const double raysmom2 = (1.0 - dep) / (2.0 + dep);
  const long nk = (long)in.km * in.nch * in.nobs;
  for (int k = 0; k <= L; ++k) S[lay.hgt + k] = in.he[k + (long)(in.km + 1) * j] * kHeightScale;
  for (int k = 0; k < L; ++k) {
    const double ray = in.rot[k + (long)in.km * (j + (long)in.nobs * i)];
    const long a = k + (long)in.km * (i + (long)in.nch * j);
    const double tl = in.tau_f ? (double)in.tau_f[a] : in.tau[a];
    const double sl = in.ssa_f ? (double)in.ssa_f[a] : in.ssa[a];
    const double tau_ext = 0.0 + ray + tl;
    const double tau_scat = ray + sl * tl;
    if (!(tau_ext > 0.0) || !(tau_scat > 0.0)) {
      radiance[o] = in.missing; reflectance[o] = in.missing;
      if (status) status[o] = RT_BAD_INPUT;
      return;
    }
    double om_in = tau_scat / tau_ext;
    if (om_in > kSsaCap) om_in = kSsaCap;
    const double aerswt = sl * tl / tau_scat, rayswt = ray / tau_scat;
    auto beta_in = [&](int l) -> double {  // GREEKMAT_TOTAL_INPUT(l, k, 1)
      if (l == 0) return 1.0;
      double am = 0.0;
      if (l < ngreek) am = in.pmom_f ? (double)in.pmom_f[a + nk * (long)l] : in.pmom[a + nk * (long)l];
      if (l == 2) return raysmom2 * rayswt + am * aerswt;
      return (l <= ngreek) ? am * aerswt : 0.0;
    };
    // delta-M
    double fdel = 0.0, fac1 = 1.0, fac2 = 1.0;
    if (opt.do_deltam) {
      fdel = beta_in(NM + 1) / (double)(2 * (NM + 1) + 1);
      fac2 = 1.0 - fdel;
      fac1 = 1.0 - fdel * om_in;
    }
    double dtau = tau_ext * fac1;
    double om = opt.do_deltam ? om_in * fac2 / fac1 : om_in;
    if (om > 0.999999999) om = 0.999999999;
    else if (om < 1.0e-9) om = 1.0e-9;
    int lnz = 0;
    for (int l = 0; l <= NM; ++l) {
      double bi = beta_in(l);
      if (bi != 0.0) lnz = l;
      double b = opt.do_deltam ? (bi - fdel * (double)(2 * l + 1)) / fac2 : bi;
      if (l == 0 && opt.do_deltam) b = 1.0;
      if (l == 1) {
        double g1 = b / 3.0;
        if (g1 > 0.999999999) g1 = 0.999999999;
        else if (g1 < -0.999999999) g1 = -0.999999999;
        else if (g1 >= 0.0 && g1 < 1.0e-9) g1 = 1.0e-9;
        else if (g1 < 0.0 && g1 > -1.0e-9) g1 = -1.0e-9;
        b = 3.0 * g1;
      }
      S[lay.og + l + 2 * NS * (long)k] = om * b;
    }
    S[lay.lnz + k] = (double)lnz;
    S[lay.dtau + k] = dtau;
    // single-scatter inputs (vlidort_vfo_interface.f90:377-411; FO_VectorSS_RTCalcs_I.f90:340-380)
    const double dz = S[lay.hgt + k] - S[lay.hgt + k + 1];
    const double dts = opt.do_deltam ? dtau : tau_ext;
    S[lay.ext + k] = dts / dz;
    S[lay.emult + k] = dts;  // temporary: FO regular-PS vertical optical depth
    double tms = opt.do_deltam ? om_in / (1.0 - fdel * om_in) : om_in;
    double p0 = 1.0, p1 = cosscat, fm = beta_in(0) * p0 + (ngreek >= 1 ? beta_in(1) * p1 : 0.0);
    for (int l = 2; l <= ngreek; ++l) {
      double p2 = ((double)(2 * l - 1) / (double)l) * p1 * cosscat - ((double)(l - 1) / (double)l) * p0;
      fm += p2 * beta_in(l);
      p0 = p1; p1 = p2;
    }
    S[lay.escat + k] = fm * tms;
  }
  // ---------------------------------------------------------------- single scatter
  double ss = 0.0, db = 0.0;
  if (opt.do_focorr) {
    const bool enhanced = !opt.do_plane_parallel && !nadir_fo;
    double phi = raa;
    if (phi < 0.0) phi = -phi;
    if (phi > 360.0) phi = 360.0 - phi - 360.0;
    fo_single_scatter(opt, enhanced, L, sza, vza, phi, alb, tu, wu, S, lay.hgt, lay.ext, lay.escat, lay.emult, &ss, &db);
  }
  // ---------------------------------------------------------------- beam attenuation
  // Chapman factors (vlidort_geometry.f90:119-317), QSPREP / PREPTRANS / EMULT
  // (vlidort_miscsetups.f90:813-1292, 3187-3421)
  {
    const double mu_toa = c.cos_sza;
    const double sn_toa = sqrt(1.0 - mu_toa * mu_toa);
    const double R0 = opt.earth_radius;
    int cutoff = L;
    double tslant_prev = 0.0, s_t_0 = 1.0, s_t_1 = 0.0;
    for (int n = 1; n <= L; ++n) {
      double ts = 0.0;
      if (opt.do_plane_parallel || sn_toa == 0.0) {
        double cf = opt.do_plane_parallel ? 1.0 / mu_toa : 1.0;
        for (int k = 1; k <= n; ++k) ts += S[lay.dtau + k - 1] * cf;
      } else {
        const double r0 = S[lay.hgt + 0] + R0;
        double sinth1 = sn_toa * (S[lay.hgt + n] + R0) / r0;
        double sth1 = asin(sinth1), re_upper = r0;
        for (int k = 1; k <= n; ++k) {
          double delz = S[lay.hgt + k - 1] - S[lay.hgt + k];
          double re_lower = re_upper - delz;
          double sinth2 = re_upper * sinth1 / re_lower;
          double sth2 = asin(sinth2);
          double dist = re_upper * sin(sth2 - sth1) / sinth2;
          ts += S[lay.dtau + k - 1] * (dist / delz);
          re_upper = re_lower; sinth1 = sinth2; sth1 = sth2;
        }
      }
      const double dtn = S[lay.dtau + n - 1];
      double avsec = 0.0, itr = 0.0;
      if (n <= cutoff) {
        if (ts > kMaxTau) cutoff = n;
        else s_t_1 = exp(-ts);
        avsec = (ts - tslant_prev) / dtn;
        itr = s_t_0;
        s_t_0 = s_t_1;
      }
      S[lay.avsec + n - 1] = avsec;
      S[lay.itrans + n - 1] = itr;
      tslant_prev = ts;
      if (n == L) {
        c.trans_solar_beam = ts < kMaxTau ? exp(-ts) : 0.0;
        c.refl_directbeam = ts < kMaxTau;
      }
    }
    c.cutoff = cutoff;
    for (int n = 0; n < L; ++n) {
      const double dtn = S[lay.dtau + n];
      double tmu = 0.0, em = 0.0;
      double sp = dtn * c.sec_u;
      double tus = sp > kMaxTau ? 0.0 : exp(-sp);
      if (n < cutoff) {
        double spb = dtn * S[lay.avsec + n];
        tmu = spb > kMaxTau ? 0.0 : exp(-spb);
        double su = (1.0 - tmu * tus) / (S[lay.avsec + n] + c.sec_u);
        em = (S[lay.itrans + n] * c.sec_u) * su;
      }
      S[lay.tmubar + n] = tmu;
      S[lay.tuser + n] = tus;
      S[lay.emult + n] = em;
    }
  }
  // ---------------------------------------------------------------- Fourier series
  // vlidort_masters_V2p8p3.f90:2305-2700 with VLIDORT_CONVERGE_OBSGEO (vlidort_converge.f90:825)
  const int n_fouriers = (vza == 0.0 && !opt.do_focorr) ? 0 : (opt.max_fourier >= 0 && opt.max_fourier < NM ? opt.max_fourier : NM);
  double stokes = 0.0;
  int testconv = 0, m = 0;
  for (m = 0; m <= n_fouriers; ++m) {
    double sf = 0.0;
    int st = fourier_term<NS>(c, opt, m, S, lay, &sf);
    if (st != RT_OK) {
      radiance[o] = in.missing; reflectance[o] = in.missing;
      if (status) status[o] = st;
      if (nfourier) nfourier[o] = m;
      return;
    }
    if (m == 0) {
      stokes = sf;
      if (opt.do_focorr) stokes += ss + db;
    } else {
      double tazm = cos(raa * (double)m * kDTR) * sf;
      double tnew = stokes + tazm;
      bool conv = (tazm != 0.0) ? (fabs(tazm / tnew) < opt.accuracy) : true;
      stokes = tnew;
      if (conv) {
        ++testconv;
        if (!opt.do_double_convtest || testconv == 2) break;
      } else {
        testconv = 0;
      }
    }
  }
  if (m > n_fouriers) m = n_fouriers;
  if (nfourier) nfourier[o] = m;
  radiance[o] = stokes;
  reflectance[o] = (kPiSingle * stokes) / (cos(sza * kPiSingle / 180.0) * opt.flux_factor);
}

}  // namespace aerort
