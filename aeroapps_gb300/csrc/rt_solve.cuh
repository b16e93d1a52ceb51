// One scalar solve (column x wavelength) in the AeroApps VLIDORT_Scalar_Lambert
// configuration, executed by a single thread.  See rt_scalar.cuh for the
// mapping rationale.  Reference routines are cited per block.
//
// Precision: the per-column set-up (layer mixing, delta-M, beam attenuation,
// first-order single scatter) is FP64.  The Fourier series -- the O(N^3 L) part
// -- runs in the working precision T: double for the plain method, float for
// the mixed method.  Where a reference formula loses accuracy in FP32 (the
// exp(-a d) - exp(-b d) differences of thin layers), the float instantiation
// uses an algebraically equal form built on expm1; the double instantiation
// keeps the reference's formulas.
#pragma once
#include "rt_brdf.cuh"
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
  // Trace-gas absorption optical depth alpha(km, nobs, nch) of the polarized
  // wrapper (VLIDORT_LAMBERT.F90:192, VLIDORT_ScatMod.F90:488-497); null = 0
  // (the scalar wrapper has none).
  const double* alpha = nullptr;
};

// Scratch element counts per thread for a solve with at most L layers: an
// FP64 region (set-up, geometry, single scatter) and a region in the working
// precision of the Fourier series.
template <int NS>
struct ScratchLayout {
  static constexpr int NMX = 2 * NS;  // NMOMENTS + 1 <= 2 NS
  long hgt, ext, escat, dts, dtau, avsec, itrans, rec, d_total;                         // FP64
  long og, om1, lnz, tdtau, tavsec, titrans, tmubar, tuser, emult, wh, we, wc, F, f, C, c, a, b, s, t_total;  // working precision
  // sweep = false leaves out F, f, C, c, a, b, s (kept elsewhere by the team kernel)
  RT_HD explicit ScratchLayout(int L, bool sweep = true) {
    long o = 0;
    hgt = o; o += L + 1; ext = o; o += L; escat = o; o += L; dts = o; o += L;
    dtau = o; o += L; avsec = o; o += L; itrans = o; o += L;
    rec = o; o += 16;  // SetupRecord
    d_total = o;
    o = 0;
    og = o; o += (long)NMX * L;
    om1 = o; o += L;
    lnz = o; o += L;
    tdtau = o; o += L; tavsec = o; o += L; titrans = o; o += L; tmubar = o; o += L;
    tuser = o; o += L; emult = o; o += L;
    wh = o; o += L + 1; we = o; o += L;  // heights and extinctions for the working-precision geometry
    wc = o; o += L + 1;                  // shell terms of the previous level (working-precision Chapman)
    if (sweep) {
      F = o; o += (long)NS * NS * L; f = o; o += (long)NS * L;
      C = o; o += (long)NS * NS * L; c = o; o += (long)NS * L;
      a = o; o += (long)NS * L; b = o; o += (long)NS * L; s = o; o += L;
    } else {
      F = f = C = c = a = b = s = -1;
    }
    t_total = o;
  }
  // bytes of scratch one thread needs with working precision T
  template <typename T>
  RT_HD long bytes() const { return d_total * (long)sizeof(double) + t_total * (long)sizeof(T); }
};

// The two scratch regions of one thread.  In a buffer shared by nthreads
// threads, the FP64 region comes first (d_total x nthreads doubles, element
// major), then the working-precision region (t_total x nthreads elements).
template <typename T>
struct SolveScratch {
  Scratch D;
  ScratchT<T> W;
};

template <int NS, typename T>
RT_HD SolveScratch<T> make_scratch(void* buffer, long tid, long nthreads, int km, bool sweep = true) {
  const ScratchLayout<NS> lay(km, sweep);
  double* d = (double*)buffer;
  T* w = (T*)(d + lay.d_total * nthreads);
  return SolveScratch<T>{Scratch{d + tid, nthreads}, ScratchT<T>{w + tid, nthreads}};
}

// Per-solve constants of the Fourier series, in its working precision.
template <int NS, typename T>
struct SolveCtx {
  int L, NM, cutoff;
  bool msmode, refl_directbeam;
  T qx[NS], qw[NS], sqw[NS];
  T mu_u, sec_u, cos_sza, albedo, trans_solar_beam;
  T pimm_q[NS], pimm_u, pimm_0;  // normalised P_m^m carried across Fourier terms
  T sin_q[NS], sin_u, sin_0;     // sqrt(1 - x^2) of the cosines, formed in FP64
};

// Homogeneous + particular solution of one layer for one Fourier term.
template <int NS, typename T>
struct LayerSol {
  T P[NS * NS];  // eigenvector components, downwelling streams (X+ rows 1..N)
  T Q[NS * NS];  // eigenvector components, upwelling streams   (X+ rows N+1..2N)
  T t[NS];       // exp(-k dtau)
  T wt[2 * NS];  // particular solution at layer top    (down 0..N-1, up N..2N-1)
  T wb[2 * NS];  // particular solution at layer bottom
};

// Recurrence coefficients of the normalised associated Legendre functions
// P~_l^m = sqrt((l-m)!/(l+m)!) P_l^m for one Fourier term m:
// P~_l^m = ra[l] x P~_{l-1}^m - rb[l] P~_{l-2}^m  (l >= m+2).
template <int NS, typename T>
struct LegendreCoef {
  T ra[2 * NS], rb[2 * NS], r1;
  RT_HD void init(int m, int NM) {
    r1 = sqrt((T)(2 * m + 1));
    for (int l = m + 2; l <= NM; ++l) {
      T d = (T)1 / sqrt((T)(l * l - m * m));
      ra[l] = (T)(2 * l - 1) * d;
      rb[l] = sqrt((T)((l - 1) * (l - 1) - m * m)) * d;
    }
  }
};

// Associated Legendre functions normalised as the reference's PI matrices
// (vlidort_miscsetups.f90:2273-2932, NSTOKES = 1: sqrt((l-m)!/(l+m)!) P_l^m,
// no Condon-Shortley phase) for Fourier term m at cosine x; out[l] for
// l = m..NM, zero below m.  The normalised recursion never forms the
// factorials, so it is safe in FP32.  pim carries P~_m^m from term m-1 to m:
// the calls for one x must come in the order m = 0, 1, 2, ...
// s = sqrt(1 - x^2), formed in FP64 by the caller (in FP32 the difference
// 1 - x^2 loses its digits at near-nadir view or sun).
template <int NS, typename T>
RT_HD void legendre_m(int m, int NM, const LegendreCoef<NS, T>& lc, T x, T s, T* pim, T* out) {
  for (int l = 0; l < m && l <= NM; ++l) out[l] = 0;
  if (m > NM) return;
  T pmm = (m == 0) ? (T)1 : *pim * s * sqrt((T)(2 * m - 1) / (T)(2 * m));
  *pim = pmm;
  out[m] = pmm;
  if (m + 1 <= NM) out[m + 1] = x * lc.r1 * pmm;
  for (int l = m + 2; l <= NM; ++l) out[l] = lc.ra[l] * x * out[l - 1] - lc.rb[l] * out[l - 2];
}

// ---------------------------------------------------------------- FP32 exponential multipliers
// The layer multipliers of the Green's-function method are divided
// differences of f(x) = exp(-x d) over the layer optical thickness d:
//   first  (e^{-a d} - e^{-b d}) / (b - a)           = -f[a, b]
//   second the user-angle particular sources sd, su  =  f[0, a, b]
// The reference evaluates them from the exponentials directly, switching to
// a Taylor series within 1e-4 of a resonance (vlidort_Taylor.f90); in FP32 the
// direct forms cancel (thin layers, nearly equal nodes), so the float
// instantiation evaluates the divided differences themselves:
//   f[a, b]    = -d e^{-min d} E1(|b - a| d),           E1(z) = (1 - e^{-z}) / z
//   f[0, a, b] = d^2 e^{-m0 d} H(u, v)  with the nodes shifted by their
//                minimum m0 to {0, u, v} (in units of d),
//   H(u, v)    = (E1(u) - E1(v)) / (v - u)
//              = J1(w) + (v-u)^2/24 J3(w) + (v-u)^4/1920 J5(w) + ...,  w = (u+v)/2,
//   J_n(w)     = int_0^1 s^n e^{-w s} ds.
// All are exact rewritings; only the evaluation order changes.
RT_HD float em1n(float z) {  // expm1(-z)
#ifdef __CUDA_ARCH__
  return expm1f(-z);
#else
  return std::expm1(-z);
#endif
}
RT_HD float e1_fn(float z) {  // (1 - e^{-z}) / z, z >= 0
  return (z < 1.0e-4f) ? 1.0f - 0.5f * z * (1.0f - z * (1.0f / 3.0f)) : -em1n(z) / z;
}
// J1, J3, J5 at w >= 0
RT_HD void jn135(float w, float* j1, float* j3, float* j5) {
  if (w < 2.0f) {
    // J_n(w) = sum_k (-w)^k / (k! (n + k + 1))
    float t = 1.0f, a1 = 0.0f, a3 = 0.0f, a5 = 0.0f;
    for (int k = 0; k < 18; ++k) {
      a1 += t / (float)(k + 2);
      a3 += t / (float)(k + 4);
      a5 += t / (float)(k + 6);
      t *= -w / (float)(k + 1);
    }
    *j1 = a1; *j3 = a3; *j5 = a5;
  } else {
    // J_n = (n J_{n-1} - e^{-w}) / w, J_0 = E1(w)
    const float e = expf(-w), iw = 1.0f / w;
    float j = e1_fn(w);
    j = (1.0f * j - e) * iw; *j1 = j;
    j = (2.0f * j - e) * iw;
    j = (3.0f * j - e) * iw; *j3 = j;
    j = (4.0f * j - e) * iw;
    j = (5.0f * j - e) * iw; *j5 = j;
  }
}
RT_HD float h_fn(float u, float v) {  // (E1(u) - E1(v)) / (v - u), u, v >= 0
  const float dl = v - u, w = 0.5f * (u + v);
  if (fabsf(dl) > 0.1f * (1.0f + w)) return (e1_fn(u) - e1_fn(v)) / dl;
  float j1, j3, j5;
  jn135(w, &j1, &j3, &j5);
  const float d2 = dl * dl;
  return j1 + d2 * (1.0f / 24.0f) * (j3 + d2 * (1.0f / 80.0f) * j5);
}
// (e^{-a d} - e^{-b d}) / (b - a), a, b >= 0
RT_HD float dd1_neg(float a, float b, float d) {
  const float lo = fminf(a, b);
  return d * expf(-lo * d) * e1_fn(fabsf(b - a) * d);
}
// f[0, a, b] for f(x) = e^{-x d}, a, b >= 0
RT_HD float dd2(float a, float b, float d) {
  // nodes {0, a, b}: minimum is 0
  return d * d * h_fn(a * d, b * d);
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
//
// Besides the eigenpairs (kv, X+ = (P; Q), transmittances t) it returns, per
// eigenvector a, the Green's-function norm sum_j mu_j w_j (P_ja^2 - Q_ja^2)
// and the user-angle homogeneous solutions (vlidort_solutions.f90:1167-1505),
// both formed from the sum and difference vectors x = P + Q, dif = P - Q: that
// is the same algebra without the cancellation of P^2 - Q^2 when P ~ Q (the
// nearly conservative mode).
template <int NS, typename T>
RT_HD int layer_eigen(const SolveCtx<NS, T>& c, int m, T dtau, T om1, const T* og, const T* piq, const T* piu,
                      LayerSol<NS, T>& ls, T* kv, T* Sp, T* norm, T* uh_dn, T* uh_up) {
  const int N = NS, NM = c.NM;
  T Bs[NS * NS], H[NS * NS], V[NS * NS];
  // Sp (even l-m) and Sm (odd l-m) contractions of omega*beta_l P_l(mu_i) P_l(mu_j)
  for (int j = 0; j < N; ++j)
    for (int i = 0; i <= j; ++i) {
      T se = 0, so = 0;
      for (int l = m; l <= NM; ++l) {
        T t = og[l] * piq[l + 2 * NS * i] * piq[l + 2 * NS * j];
        if (((l - m) & 1) == 0) se += t; else so += t;
      }
      Sp[i + NS * j] = se; Sp[j + NS * i] = se;
      T b = -c.sqw[i] * c.sqw[j] * so;
      if (i == j) b += (T)1;
      Bs[i + NS * j] = b; Bs[j + NS * i] = b;
    }
  if (!cholesky<NS>(N, Bs)) return RT_EIGEN_FAIL;
  // R = M^-1 Lb (lower triangular)
  for (int j = 0; j < N; ++j)
    for (int i = j; i < N; ++i) Bs[i + NS * j] /= c.qx[i];
  T kq[NS];  // k of each eigenvector column of V
  T G[NS * NS];
  // H = G^T G with G = La^T R (As = La La^T).  One-sided Jacobi (Hestenes)
  // orthogonalises the columns of G by plane rotations V, so that the
  // singular values k = |G V e_a| and the eigenvectors (columns of V) come with
  // relative accuracy although k^2 spans four to five decades (1/mu^2 of the
  // shallowest stream); a QR eigensolver on H itself leaves the small-k
  // eigenvectors an error of order eps |H| / gap.
  T rv[NS], rbeta = 0;
  if (m == 0) {
    // Fourier term 0: As has the exact eigenvector s = W^1/2 1 with
    // eigenvalue 1 - omega (the half-range Gauss rule integrates every even
    // moment l >= 2 to zero).  The reflector Q (Q s = -e_1 |s|) splits it
    // off exactly; 1 - omega comes from the FP64 set-up, so nearly
    // conservative layers keep their small eigenvalue in either precision,
    // and only the well-conditioned complement B = (Q As Q)[1:, 1:] is
    // factorised.  La = Q diag(sqrt(1-omega), Lb_B).
    T v[NS], vv = 0;
    {
      T ns = 0;
      for (int i = 0; i < N; ++i) { v[i] = c.sqw[i]; ns += v[i] * v[i]; }
      ns = sqrt(ns);
      v[0] += ns;  // s has positive entries
      for (int i = 0; i < N; ++i) vv += v[i] * v[i];
    }
    const T beta = (T)2 / vv;
    rbeta = beta;
    for (int i = 0; i < N; ++i) rv[i] = v[i];
    // As (full) in H, then C = Q As Q
    for (int j = 0; j < N; ++j)
      for (int i = 0; i < N; ++i) {
        T a = -c.sqw[i] * Sp[i + NS * j] * c.sqw[j];
        if (i == j) a += (T)1;
        H[i + NS * j] = a;
      }
    apply_reflector_sym<NS>(N, H, v, beta);
    H[0] = om1;
    for (int i = 1; i < N; ++i) { H[i] = 0; H[NS * i] = 0; }
    if (!(om1 > (T)0) || !cholesky<NS>(N, H)) return RT_EIGEN_FAIL;
    // G = La^T R = diag-block(L~)^T (Q R)
    T QR[NS * NS];
    for (int j = 0; j < N; ++j) {
      T d = 0;
      for (int k = j; k < N; ++k) d += v[k] * Bs[k + NS * j];
      d *= beta;
      for (int i = 0; i < N; ++i) QR[i + NS * j] = ((i >= j) ? Bs[i + NS * j] : (T)0) - d * v[i];
    }
    for (int j = 0; j < N; ++j)
      for (int i = 0; i < N; ++i) {
        T s = 0;
        for (int k = i; k < N; ++k) s += H[k + NS * i] * QR[k + NS * j];
        G[i + NS * j] = s;
      }
  } else {
    for (int j = 0; j < N; ++j)
      for (int i = j; i < N; ++i) {
        T a = -c.sqw[i] * Sp[i + NS * j] * c.sqw[j];
        if (i == j) a += (T)1;
        H[i + NS * j] = a;
      }
    if (!cholesky<NS>(N, H)) return RT_EIGEN_FAIL;
    for (int j = 0; j < N; ++j)
      for (int i = 0; i < N; ++i) {
        T s = 0;
        for (int k = (i > j ? i : j); k < N; ++k) s += H[k + NS * i] * Bs[k + NS * j];
        G[i + NS * j] = s;
      }
  }
  if (!jacobi_svd<NS>(N, G, V, kq)) return RT_EIGEN_FAIL;
  // G now holds G V = U diag(k).  As v_a = La La^T R q_a = La (G V)e_a, so
  // SAB x / k needs La u_a only (u_a = unit left singular vector): no
  // cancellation for the small-k modes.  Overwrite G[:, a] with La u_a.
  for (int a = 0; a < N; ++a) {
    if (!(kq[a] > (T)0)) return RT_EIGEN_FAIL;
    const T inv = (T)1 / kq[a];
    T u[NS], y[NS];
    for (int i = 0; i < N; ++i) u[i] = G[i + NS * a] * inv;
    for (int i = 0; i < N; ++i) {
      T s = 0;
      for (int k = 0; k <= i; ++k) s += H[i + NS * k] * u[k];
      y[i] = s;
    }
    if (m == 0) {
      T d = 0;
      for (int i = 0; i < N; ++i) d += rv[i] * y[i];
      d *= rbeta;
      for (int i = 0; i < N; ++i) y[i] -= d * rv[i];
    }
    for (int i = 0; i < N; ++i) G[i + NS * a] = y[i];
  }
  for (int a = 0; a < N; ++a) {
    // v = R q ; sum vector x = W^-1/2 v, unit 2-norm
    T x[NS], nrm = 0;
    for (int i = 0; i < N; ++i) {
      T s = 0;
      for (int j = 0; j <= i; ++j) s += Bs[i + NS * j] * V[j + NS * a];
      x[i] = s / c.sqw[i];
      nrm += x[i] * x[i];
    }
    const T k = kq[a];
    if (!(k > (T)0)) return RT_EIGEN_FAIL;
    kv[a] = k;
    nrm = (T)1 / sqrt(nrm);
    for (int i = 0; i < N; ++i) x[i] *= nrm;
    // difference vector SAB x / k = M^-1 W^-1/2 As v / (k |W^-1/2 v|)
    //                             = M^-1 W^-1/2 La u_a / |W^-1/2 v|
    T dif[NS], nr = 0;
    for (int i = 0; i < N; ++i) {
      dif[i] = G[i + NS * a] / (c.qx[i] * c.sqw[i]) * nrm;
      ls.P[i + NS * a] = (T)0.5 * (x[i] + dif[i]);
      ls.Q[i + NS * a] = (T)0.5 * (x[i] - dif[i]);
      nr += c.qx[i] * c.qw[i] * x[i] * dif[i];
    }
    norm[a] = nr;
    T help = k * dtau;
    ls.t[a] = help > (T)kMaxTau ? (T)0 : exp(-help);
    // user-angle homogeneous solutions: sum_j w_j P_l(mu_j) (P +- Q)_ja / 2
    T dn = 0, up = 0;
    for (int l = m; l <= NM; ++l) {
      const bool even = ((l - m) & 1) == 0;
      T sps = 0;
      for (int j = 0; j < N; ++j) sps += c.qw[j] * piq[l + 2 * NS * j] * (even ? x[j] : dif[j]);
      T h = (T)0.5 * og[l] * sps;
      dn += (even ? piu[l] : -piu[l]) * h;
      up += piu[l] * h;
    }
    uh_dn[a] = dn;
    uh_up[a] = up;
  }
  return RT_OK;
}

// Solution pieces of one layer for Fourier term m: eigen-solution, user-angle
// homogeneous and particular terms (vlidort_solutions.f90:1051-1163, 1167-1505,
// 1651-1790, 2649-3073; PostProcessing.f90:139-451).  Writes the per-layer
// source coefficients a, b, s (TOA radiance = sum_n Tcum_n (L.a + M.b + s)).
template <int NS, typename T>
RT_HD int layer_solution(const SolveCtx<NS, T>& c, const RtOptions& opt, int m, int n, bool laysc,
                         const ScratchT<T>& W, const ScratchLayout<NS>& lay, const T* piq, const T* piu, const T* pi0,
                         LayerSol<NS, T>& ls) {
  const int N = NS, NM = c.NM;
  T og[2 * NS], kv[NS], Sp[NS * NS];
  for (int l = 0; l <= NM; ++l) og[l] = (l >= m) ? W[lay.og + l + 2 * NS * (long)n] : (T)0;
  const T dtau = W[lay.tdtau + n];
  T uh_dn[NS], uh_up[NS], hm1[NS], hm2[NS], norm[NS];
  int st = layer_eigen<NS, T>(c, m, dtau, W[lay.om1 + n], og, piq, piu, ls, kv, Sp, norm, uh_dn, uh_up);
  if (st != RT_OK) return st;
  const T tuser = W[lay.tuser + n];
  const T smu = c.sec_u;
  for (int a = 0; a < N; ++a) {
    if (!laysc) { uh_dn[a] = 0; uh_up[a] = 0; }
    // homogeneous multipliers
    T zdel = ls.t[a];
    T rho_p = smu + kv[a], rho_m = smu - kv[a];
    if constexpr (sizeof(T) == sizeof(float)) {
      hm2[a] = smu * dtau * e1_fn(rho_p * dtau);
      hm1[a] = smu * dd1_neg(kv[a], smu, dtau);
    } else {
      hm2[a] = smu * (1.0 - zdel * tuser) * (1.0 / rho_p);
      if (fabs(rho_m) < kTaylorSmall) hm1[a] = taylor1<T>(opt.taylor_order, rho_m, dtau, tuser, smu);
      else hm1[a] = smu * (zdel - tuser) * (1.0 / rho_m);
    }
  }
  for (int a = 0; a < N; ++a) {
    W[lay.a + a + N * (long)n] = uh_dn[a] * hm2[a];
    W[lay.b + a + N * (long)n] = uh_up[a] * hm1[a];
  }
  for (int i = 0; i < 2 * N; ++i) { ls.wt[i] = 0; ls.wb[i] = 0; }
  T spart = 0;
  const bool active = (n < c.cutoff) && laysc;
  if (active) {
    // Green's-function particular integral (VLIDORT_GBEAM_SOLUTION)
    const T F1 = (T)(opt.flux_factor / kPI4);
    const T secbar = W[lay.tavsec + n], cnst = W[lay.titrans + n], wdel = W[lay.tmubar + n];
    T hq[2 * NS], dpi[NS], dmi[NS];
    for (int l = m; l <= NM; ++l) hq[l] = og[l] * pi0[l];
    T upar = 0;
    for (int l = m; l <= NM; ++l) upar += (F1 * hq[l]) * ((((l - m) & 1) ? (T)-1 : (T)1) * piu[l]);
    for (int i = 0; i < N; ++i) {
      T sp = 0, sm = 0;
      for (int l = m; l <= NM; ++l) {
        T t = piq[l + 2 * NS * i] * hq[l];
        sp += t;
        sm += (((l - m) & 1) ? -t : t);
      }
      dpi[i] = F1 * sp; dmi[i] = F1 * sm;
    }
    const T emult = W[lay.emult + n];
    const T itw = -cnst * wdel;
    const T sigp = secbar + smu;
    T gup[NS], gdn[NS];
    for (int a = 0; a < N; ++a) {
      T zdel = ls.t[a];
      T gp = secbar + kv[a], gm = secbar - kv[a];
      const bool tay = fabs(gm) < (T)kTaylorSmall;
      T cf, df;
      if constexpr (sizeof(T) == sizeof(float)) {
        cf = cnst * dd1_neg(kv[a], secbar, dtau);
        df = cnst * dtau * e1_fn(gp * dtau);
      } else {
        cf = tay ? taylor1<T>(opt.taylor_order, gm, dtau, wdel, cnst) : cnst * (zdel - wdel) / gm;
        df = cnst * (1.0 - zdel * wdel) / gp;
      }
      T s1 = 0, s2 = 0;
      for (int i = 0; i < N; ++i) {
        s1 += c.qw[i] * (dpi[i] * ls.P[i + NS * a] + dmi[i] * ls.Q[i + NS * a]);
        s2 += c.qw[i] * (dmi[i] * ls.P[i + NS * a] + dpi[i] * ls.Q[i + NS * a]);
      }
      T at = s1 / norm[a], bt = s2 / norm[a];
      gdn[a] = cf * at;
      gup[a] = df * bt;
      // user-angle particular source (WHOLELAYER_STERM_UP, Green's branch)
      T sd, su;
      if constexpr (sizeof(T) == sizeof(float)) {
        sd = cnst * smu * dd2(kv[a] + smu, sigp, dtau);
        su = cnst * smu * dd2(gp, sigp, dtau);
      } else {
        if (tay) {
          T mult = taylor2<T>(opt.taylor_order, gm, sigp, dtau, (T)1, wdel * tuser, (T)1);
          sd = (cnst * smu) * mult;
        } else {
          sd = (cnst * hm2[a] - emult) / gm;
        }
        su = (itw * hm1[a] + emult) / gp;
      }
      spart += uh_dn[a] * sd * at + uh_up[a] * su * bt;
    }
    for (int i = 0; i < N; ++i) {
      T wu1 = 0, wu2 = 0, wl1 = 0, wl2 = 0;
      for (int a = 0; a < N; ++a) {
        wu1 += gup[a] * ls.Q[i + NS * a]; wu2 += gup[a] * ls.P[i + NS * a];
        wl1 += gdn[a] * ls.P[i + NS * a]; wl2 += gdn[a] * ls.Q[i + NS * a];
      }
      ls.wt[i] = wu1; ls.wt[N + i] = wu2;
      ls.wb[i] = wl1; ls.wb[N + i] = wl2;
    }
    if (!c.msmode) spart += upar * emult;
  }
  W[lay.s + n] = laysc ? spart : (T)0;
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
template <int NS, typename T>
RT_HD int fourier_term(SolveCtx<NS, T>& c, const RtOptions& opt, int m, const ScratchT<T>& W,
                       const ScratchLayout<NS>& lay, T* out) {
  const int N = NS, NM = c.NM, L = c.L;
  const bool incl_surface = (m == 0) && (c.albedo != (T)0);
  const T surface_factor = (m == 0) ? (T)2 : (T)1;
  const T delta_factor = (m == 0) ? (T)1 : (T)2;
  const bool localbeam = incl_surface && c.refl_directbeam;
  T direct_beam = 0;
  if (localbeam) {
    T x0 = (T)4 * c.cos_sza / delta_factor;
    x0 = (T)opt.flux_factor * x0 / (T)kPI4;
    direct_beam = x0 * c.trans_solar_beam * c.albedo;
  }
  T piq[2 * NS * NS], piu[2 * NS], pi0[2 * NS];
  {
    LegendreCoef<NS, T> lc;
    lc.init(m, NM);
    for (int i = 0; i < N; ++i) legendre_m<NS, T>(m, NM, lc, c.qx[i], c.sin_q[i], &c.pimm_q[i], &piq[2 * NS * i]);
    legendre_m<NS, T>(m, NM, lc, c.mu_u, c.sin_u, &c.pimm_u, piu);
    legendre_m<NS, T>(m, NM, lc, c.cos_sza, c.sin_0, &c.pimm_0, pi0);
  }

  LayerSol<NS, T> A, B;
  LayerSol<NS, T>* prev = &A;
  LayerSol<NS, T>* cur = &B;
  T F[NS * NS], f[NS];
  T K[4 * NS * NS], R[2 * NS * (NS + 1)];
  for (int n = 0; n < L; ++n) {
    // DO_LAYER_SCATTERING(m, n) (vlidort_inputs.f90:4321-4330): false for m >= 3
    // when every input moment l = m..NMOMENTS of the layer is zero
    const bool lsc = (m < 3) || ((T)m <= W[lay.lnz + n]);
    int st = layer_solution<NS, T>(c, opt, m, n, lsc, W, lay, piq, piu, pi0, *cur);
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
        for (int i = 0; i < N; ++i) { F[i + NS * j] = R[i + 2 * NS * j]; W[lay.F + i + NS * j + (long)NS * NS * n] = F[i + NS * j]; }
      for (int i = 0; i < N; ++i) { f[i] = R[i + 2 * NS * N]; W[lay.f + i + NS * (long)n] = f[i]; }
    } else {
      // interface between layer n-1 (prev) and n (cur):
      // G M_{n-1} + g + Wb_{n-1} = X+_n L_n + X-_n T_n M_n + Wt_n
      T TF[NS * NS], tf[NS];
      for (int j = 0; j < N; ++j)
        for (int k = 0; k < N; ++k) TF[k + NS * j] = prev->t[k] * F[k + NS * j];
      for (int k = 0; k < N; ++k) tf[k] = prev->t[k] * f[k];
      for (int j = 0; j < N; ++j)
        for (int i = 0; i < N; ++i) {
          T gt = prev->Q[i + NS * j], gb = prev->P[i + NS * j];
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
        T gt = 0, gb = 0;
        for (int k = 0; k < N; ++k) { gt += prev->P[i + NS * k] * tf[k]; gb += prev->Q[i + NS * k] * tf[k]; }
        R[i + 2 * NS * N] = cur->wt[i] - prev->wb[i] - gt;
        R[N + i + 2 * NS * N] = cur->wt[N + i] - prev->wb[N + i] - gb;
      }
      if (!lu_solve<2 * NS>(2 * N, K, R, N + 1)) return RT_BVP_SINGULAR;
      long oC = lay.C + (long)NS * NS * (n - 1), oc = lay.c + (long)NS * (n - 1);
      long oF = lay.F + (long)NS * NS * n, of = lay.f + (long)NS * n;
      for (int j = 0; j < N; ++j)
        for (int i = 0; i < N; ++i) {
          W[oC + i + NS * j] = R[i + 2 * NS * j];
          F[i + NS * j] = R[N + i + 2 * NS * j];
          W[oF + i + NS * j] = F[i + NS * j];
        }
      for (int i = 0; i < N; ++i) {
        W[oc + i] = R[i + 2 * NS * N];
        f[i] = R[N + i + 2 * NS * N];
        W[of + i] = f[i];
      }
    }
    LayerSol<NS, T>* t = prev; prev = cur; cur = t;
  }
  // surface: upwelling at the bottom = Lambertian reflection of the downwelling
  // diffuse field + reflected direct beam (bvproblem.f90:439-623, 1625-1739)
  const LayerSol<NS, T>& bl = *prev;
  const T kmult = incl_surface ? surface_factor * c.albedo : (T)0;
  T r2p[NS], r2m[NS], r2b = 0;
  for (int k = 0; k < N; ++k) {
    T sp = 0, sm = 0;
    for (int j = 0; j < N; ++j) { sp += c.qx[j] * c.qw[j] * bl.P[j + NS * k]; sm += c.qx[j] * c.qw[j] * bl.Q[j + NS * k]; }
    r2p[k] = sp * kmult; r2m[k] = sm * kmult;
  }
  for (int j = 0; j < N; ++j) r2b += c.qx[j] * c.qw[j] * bl.wb[j];
  r2b *= kmult;
  {
    for (int j = 0; j < N; ++j)
      for (int i = 0; i < N; ++i) {
        T s = bl.P[i + NS * j] - r2m[j];
        for (int k = 0; k < N; ++k) s += (bl.Q[i + NS * k] - r2p[k]) * bl.t[k] * F[k + NS * j];
        K[i + 2 * NS * j] = s;
      }
    for (int i = 0; i < N; ++i) {
      T s = -bl.wb[N + i] + r2b + (localbeam ? direct_beam : (T)0);
      for (int k = 0; k < N; ++k) s -= (bl.Q[i + NS * k] - r2p[k]) * bl.t[k] * f[k];
      R[i] = s;
    }
    if (!lu_solve<2 * NS>(N, K, R, 1)) return RT_BVP_SINGULAR;
  }
  T Mc[NS], Lc[NS], Mn[NS];
  for (int i = 0; i < N; ++i) Mc[i] = R[i];
  for (int i = 0; i < N; ++i) {
    T s = f[i];
    for (int k = 0; k < N; ++k) s += F[i + NS * k] * Mc[k];
    Lc[i] = s;
  }
  // bottom boundary source at the user angle (GET_BOA_SOURCE)
  T cum = 0;
  if (incl_surface) {
    T s = 0;
    for (int i = 0; i < N; ++i) {
      T h = bl.wb[i];
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
        T s = W[oc + i];
        for (int k = 0; k < N; ++k) s += W[oC + i + NS * k] * Mc[k];
        Mn[i] = s;
      }
      for (int i = 0; i < N; ++i) {
        T s = W[of + i];
        for (int k = 0; k < N; ++k) s += W[oF + i + NS * k] * Mn[k];
        Lc[i] = s;
      }
      for (int i = 0; i < N; ++i) Mc[i] = Mn[i];
    }
    T src = W[lay.s + n];
    for (int k = 0; k < N; ++k) src += Lc[k] * W[lay.a + k + N * (long)n] + Mc[k] * W[lay.b + k + N * (long)n];
    cum = src + W[lay.tuser + n] * cum;
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

// ---------------------------------------------------------------------------------- geometry
// Two forms of the spherical-shell geometry.  The plain FP64 method keeps the
// reference's law-of-sines form (asin of the local zenith sines, sin of their
// differences), whose rounding at small solar zenith angles is part of the
// result the plain method must reproduce to 1e-9.  The mixed method uses the
// chord form below (square roots only).

// Sun path through layers 1..nn of a straight ray that leaves radius radstart
// with local solar zenith th (sine sth), layers ordered from TOA (index 0 of
// radii) down; returns sum_k ext_k * path_k.  Direct-sun and tangent-ray
// branches follow FO_geometry_Generic.f90:169-329 (FindSunPaths_D / _T).
RT_HD double sun_optical_path_ref(bool zero_sun_boa, bool direct, double radstart, double th, double sth, int nn,
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

// First-order single scatter, law-of-sines geometry (plain method); see
// fo_single_scatter_chord for the references.
RT_HD bool fo_single_scatter_ref(const RtOptions& opt, bool enhanced, int L, double sza, double vza, double phi,
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
        st = sun_optical_path_ref(overhead, true, radius(n), th_R, sthb, n, R0, S, ohgt, oext, L);
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
    double st = sun_optical_path_ref(overhead, true, radius(L), th_R, sthb, L, R0, S, ohgt, oext, L);
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
      double sd = sun_optical_path_ref(zero_sun_boa, dsf, rf, thf, sthf, n, R0, S, ohgt, oext, L);
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


// Spherical-shell geometry without inverse trigonometry.  A straight ray with
// impact parameter p (distance of closest approach to the Earth's centre)
// crosses the shell between radii r_lo < r_hi on a chord of length
//   sqrt(r_hi^2 - p^2) - sqrt(r_lo^2 - p^2) = (r_hi - r_lo)(r_hi + r_lo) / (c_hi + c_lo),
// c = sqrt((r - p)(r + p)).  The reference evaluates the same chord by the
// law of sines, r_lo sin(th_lo - th_hi) / sin(th_hi) with th = asin(p / r)
// (FO_geometry_Generic.f90:169-329, vlidort_geometry.f90:119-317); the form
// here needs one square root per level and has no cancellation between
// nearly equal angles.
RT_HD double shell_c(double r, double p) { return sqrt((r - p) * (r + p)); }

// Sun path through layers 1..nn of a straight ray that leaves radius radstart
// (inside layer nn) towards the sun, with local solar zenith cosine ct and
// sine st there; layers ordered from TOA (level 0) down; returns
// sum_k ext_k * path_k.  Direct-sun and tangent-ray branches follow
// FO_geometry_Generic.f90:169-329 (FindSunPaths_D / _T).
RT_HD double sun_optical_path_chord(bool zero_sun_boa, bool direct, double radstart, double ct, double st, int nn,
                              double R0, const Scratch& S, long ohgt, long oext, int L) {
  auto radius = [&](int k) { return R0 + S[ohgt + k]; };
  double tau = 0.0;
  if (direct) {
    if (zero_sun_boa) {
      tau += S[oext + nn - 1] * (radius(nn - 1) - radstart);
      for (int k = nn - 1; k >= 1; --k) tau += S[oext + k - 1] * (radius(k - 1) - radius(k));
      return tau;
    }
    const double p = radstart * st;
    double r_lo = radstart, c_lo = radstart * ct;
    {
      const double r_hi = radius(nn - 1), c_hi = shell_c(r_hi, p);
      tau += S[oext + nn - 1] * ((r_hi - r_lo) * (r_hi + r_lo) / (c_hi + c_lo));
      r_lo = r_hi; c_lo = c_hi;
    }
    for (int k = nn - 1; k >= 1; --k) {
      const double r_hi = radius(k - 1), c_hi = shell_c(r_hi, p);
      const double dz = S[ohgt + k - 1] - S[ohgt + k];
      tau += S[oext + k - 1] * (dz * (r_hi + r_lo) / (c_hi + c_lo));
      r_lo = r_hi; c_lo = c_hi;
    }
    return tau;
  }
  // tangent ray (sun below the local horizon): passes its lowest point below
  // the start level, then rises to TOA.  Rare at the angles AeroApps uses;
  // kept in the reference's angle form.
  const double th = acos(ct), sth = st;
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
    pnn = -2.0 * radstart * ct;
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
RT_HD bool fo_single_scatter_chord(const RtOptions& opt, bool enhanced, int L, double sza, double vza, double phi,
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
        st = sun_optical_path_chord(overhead, true, radius(n), cth, sthb, n, R0, S, ohgt, oext, L);
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
  double raycon = 0.0, caL = 1.0, saL = 0.0;
  if (!donadir) {
    const double alphaL = vza * kDTR;
    saL = (vza == 90.0) ? 1.0 : sin(alphaL);
    caL = (vza == 90.0) ? 0.0 : cos(alphaL);
    raycon = saL * radius(L);
  }
  // solar direction at BOA (the y component does not enter: the line of sight lies in the x-z plane)
  double sdir0 = 0.0, sdir2 = 0.0;
  if (!overhead) { sdir0 = -sthb * cos(phi * kDTR); sdir2 = -cth; }
  // direct-sun attenuation at the surface (used by the direct bounce)
  {
    double st = sun_optical_path_chord(overhead, true, radius(L), cth, sthb, L, R0, S, ohgt, oext, L);
    atten_boa = st < kFoCutoff ? exp(-st) : 0.0;
  }
  // top-down accumulation of the line-of-sight source: TOA sees layer n through layers 1..n-1
  double c_up = donadir ? 0.0 : shell_c(radius(0), raycon);
  for (int n = 1; n <= L; ++n) {
    const double r_up = radius(n - 1), r_lo = radius(n);
    double losw, c_lo;
    if (donadir) {
      losw = r_up - r_lo;
      c_lo = r_lo;
    } else {
      c_lo = (n == L) ? r_lo * caL : shell_c(r_lo, raycon);
      losw = (S[ohgt + n - 1] - S[ohgt + n]) * (r_up + r_lo) / (c_up + c_lo);
    }
    const double kn = S[oext + n - 1];
    const double lostau = kn * losw;
    const double lostrans = lostau < kFoCutoff ? exp(-lostau) : 0.0;
    const bool zero_sun_boa = overhead && (n == L || donadir);
    double sum = 0.0;
    for (int j = 0; j < opt.nfine; ++j) {
      const double tf = losw * tu[j], wf = losw * wu[j];
      // fine point at distance tf above the layer bottom along the line of
      // sight: radius rf, and the angle af it subtends at the centre from the
      // surface point (tan af = raycon / (c_lo + tf))
      double rf, ct, st;
      if (donadir) {
        rf = r_lo + tf;
        ct = cth; st = sthb;
      } else {
        const double X = c_lo + tf;
        rf = sqrt(raycon * raycon + X * X);
        const double caf = X / rf, saf = raycon / rf;
        // cumulative angle alphaL - af
        const double scum = saL * caf - caL * saf, ccum = caL * caf + saL * saf;
        if (overhead) {
          ct = ccum; st = scum;
        } else {
          // FindSun: cosine of the local solar zenith at the fine point
          ct = scum * sdir0 - ccum * sdir2;
          st = sqrt(1.0 - ct * ct);
        }
      }
      const bool dsf = donadir || overhead || (ct >= 0.0);
      double sd = sun_optical_path_chord(zero_sun_boa, dsf, rf, ct, st, n, R0, S, ohgt, oext, L);
      double attf = sd < kFoCutoff ? exp(-sd) : 0.0;
      sum += attf * exp(-kn * (losw - tf)) * wf;
    }
    cum += trans_above * S[oescat + n - 1] * (sum * kn);
    trans_above *= lostrans;
    c_up = c_lo;
  }
  *ss = flux * cum;
  *db = flux * (4.0 * cth * albedo * atten_boa) * trans_above;
  return true;
}

// What the Fourier series of one solve needs from its set-up, besides the
// per-layer arrays left in scratch (stored in the FP64 scratch record so that
// another thread can run the series).
struct SetupRecord {
  double ss, db, raa, sza, mu_u, sec_u, cos_sza, albedo, trans_solar_beam;
  long o;
  int L, NM, cutoff, n_fouriers;
  bool msmode, refl_directbeam;
  RT_HD void store(const Scratch& S, long at) const {
    double v[16] = {ss, db, raa, sza, mu_u, sec_u, cos_sza, albedo, trans_solar_beam, (double)o, (double)L,
                    (double)NM, (double)cutoff, (double)n_fouriers, msmode ? 1.0 : 0.0, refl_directbeam ? 1.0 : 0.0};
    for (int k = 0; k < 16; ++k) S[at + k] = v[k];
  }
  RT_HD void load(const Scratch& S, long at) {
    ss = S[at]; db = S[at + 1]; raa = S[at + 2]; sza = S[at + 3]; mu_u = S[at + 4]; sec_u = S[at + 5];
    cos_sza = S[at + 6]; albedo = S[at + 7]; trans_solar_beam = S[at + 8]; o = (long)S[at + 9];
    L = (int)S[at + 10]; NM = (int)S[at + 11]; cutoff = (int)S[at + 12]; n_fouriers = (int)S[at + 13];
    msmode = S[at + 14] != 0.0; refl_directbeam = S[at + 15] != 0.0;
  }
};

// Fourier-series context in the working precision from a set-up record.
// sqrt(1 - x^2) of a cosine, formed in FP64 (exactly 0 at x = 1).
RT_HD double quad_sine(double x) { return (x == 1.0) ? 0.0 : sqrt(1.0 - x * x); }

template <int NS, typename T>
RT_HD void make_ctx(const SetupRecord& r, const double* qx, const double* qw, SolveCtx<NS, T>& c) {
  c.L = r.L; c.NM = r.NM; c.cutoff = r.cutoff; c.msmode = r.msmode; c.refl_directbeam = r.refl_directbeam;
  auto sine = quad_sine;
  for (int q = 0; q < NS; ++q) {
    c.qx[q] = (T)qx[q]; c.qw[q] = (T)qw[q]; c.sqw[q] = (T)sqrt(qw[q]); c.pimm_q[q] = 0;
    c.sin_q[q] = (T)sine(qx[q]);
  }
  c.pimm_u = 0; c.pimm_0 = 0;
  c.sin_u = (T)sine(r.mu_u);
  c.sin_0 = (T)sine(r.cos_sza);
  c.mu_u = (T)r.mu_u; c.sec_u = (T)r.sec_u; c.cos_sza = (T)r.cos_sza; c.albedo = (T)r.albedo;
  c.trans_solar_beam = (T)r.trans_solar_beam;
}

// Azimuthal Fourier sum with the reference's double convergence test
// (VLIDORT_CONVERGE_OBSGEO, vlidort_converge.f90:825-1236).  Returns true when
// the series has converged after term m.
struct FourierSum {
  double stokes = 0.0;
  double sumabs = 0.0;  // sum of |contributions|: |stokes| / sumabs measures the cancellation
  double edge = 1e300;  // smallest | |term / sum| / accuracy - 1 | over the convergence tests
  int testconv = 0;
  RT_HD bool add(const RtOptions& opt, const SetupRecord& r, int m, double sf) {
    if (m == 0) {
      stokes = sf;
      sumabs = fabs(sf);
      if (opt.do_focorr) {
        stokes += r.ss + r.db;
        sumabs += fabs(r.ss) + fabs(r.db);
      }
      return false;
    }
    double tazm = cos(r.raa * (double)m * kDTR) * sf;
    sumabs += fabs(tazm);
    double tnew = stokes + tazm;
    bool conv = true;
    if (tazm != 0.0) {
      const double q = fabs(tazm / tnew);
      conv = q < opt.accuracy;
      const double d = fabs(q / opt.accuracy - 1.0);
      if (d < edge) edge = d;
    }
    stokes = tnew;
    if (conv) {
      ++testconv;
      if (!opt.do_double_convtest || testconv == 2) return true;
    } else {
      testconv = 0;
    }
    return false;
  }
};

// Relative distance of a convergence test's |term / sum| from the accuracy
// threshold below which a mixed-method solve is re-solved in FP64: the FP32
// terms were measured within 2e-4 (relative) of the FP64 terms on the
// solves whose test decided the other way.
constexpr double kConvEdge = 1.0e-3;

// Which solves a launch runs and which it hands on.  in_list (device, length
// *in_count): run only these solve indices (the FP64 refinement pass);
// out_list: append every solve that the FP64 pass must re-solve: its Fourier
// sum cancels by more than `ratio` (sum |terms| > ratio |radiance|), or one
// of its convergence tests came within kConvEdge (relative) of the accuracy
// threshold.  The mixed method's terms carry ~1e-6 relative FP32 error each:
// a radiance that is a near-cancellation of much larger terms would inherit
// it amplified, and a test that close to the threshold can decide the other
// way than in FP64 -- the series then ends at another term, and the terms
// that one solve keeps and the other drops are of order accuracy x radiance
// each (up to 8e-4 relative in a slowly converging series).
struct Worklist {
  const int* in_list = nullptr;
  const int* in_count = nullptr;
  int* out_list = nullptr;
  int* out_count = nullptr;
  double ratio = 0.0;
  RT_HD int count(int nsolve) const { return in_list ? *in_count : nsolve; }
  RT_HD int solve(int s) const { return in_list ? in_list[s] : s; }
  RT_HD void flag(const FourierSum& sum, int st, int sidx) const {
    if (!out_list || st != RT_OK || !(sum.sumabs > ratio * fabs(sum.stokes) || sum.edge < kConvEdge)) return;
#ifdef __CUDA_ARCH__
    const int pos = atomicAdd(out_count, 1);
#else
    const int pos = (*out_count)++;
#endif
    out_list[pos] = sidx;
  }
};
// Cancellation ratio above which a mixed-method radiance is re-solved in FP64.
constexpr double kRefineRatio = 10.0;

// Outputs of a finished series (status RT_OK) or of a failed term.
RT_HD void solve_finish(const RtOptions& opt, const LambertInputs& in, const SetupRecord& r, int st, int m,
                        double stokes, double* radiance, double* reflectance, int* nfourier, int* status) {
  const long o = r.o;
  if (st != RT_OK) {
    radiance[o] = in.missing; reflectance[o] = in.missing;
    if (status) status[o] = st;
    if (nfourier) nfourier[o] = m;
    return;
  }
  if (m > r.n_fouriers) m = r.n_fouriers;
  if (nfourier) nfourier[o] = m;
  radiance[o] = stokes;
  reflectance[o] = (kPiSingle * stokes) / (cos(r.sza * kPiSingle / 180.0) * opt.flux_factor);
}

// Set-up of pixel (obs j, channel i) = solve index sidx = j * nch + i in the
// reference loop order (VLIDORT_LAMBERT.F90:106-165): layer mixing, delta-M,
// first-order single scatter, beam attenuation.  Leaves the per-layer inputs of
// the Fourier series in scratch and fills r.  Returns false when the pixel is
// finished already (MISSING inputs or a bad layer: outputs written).
// With `brdf` the surface is a BRDF instead of the albedo: the RTLS kernels of
// VLIDORT_Scalar_LandMODIS (VLIDORT_BRDF_MODIS.F90:113-185) or the Cox-Munk
// glint of VLIDORT_Scalar_CX (VLIDORT_BRDF_CX.F90:497-545).  Its exact
// direct-bounce value BR feeds the first-order correction and the BR output
// (RTLS: a negative BR gives -500 in radiance, reflectance and BR and no
// solve), and the solve's Fourier terms (Cox-Munk: also its quadrature-to-
// quadrature terms) go to block `bidx` of brdf->terms.
template <int NS, typename T>
RT_HD bool solve_setup(const RtOptions& opt, const LambertInputs& in, int sidx, const double* tu, const double* wu,
                       const SolveScratch<T>& SS, double* radiance, double* reflectance, int* nfourier,
                       int* status, SetupRecord& r, const BrdfInputs* brdf = nullptr, long bidx = 0) {
  const Scratch& S = SS.D;
  const ScratchT<T>& W = SS.W;
  const int nch = in.nch, j = sidx / nch, i = sidx % nch;
  const long o = (long)j + (long)in.nobs * i;
  const int L = in.nlay ? in.nlay[j] : in.km, ngreek = in.nmom;
  const ScratchLayout<NS> lay(in.km);
  auto is_missing = [&](double x) { return fabs(x / in.missing - 1.0) < 0.001; };
  const double sza = in.sza[j], vza = in.vza[j], raa = in.raa[j], alb = brdf ? 0.0 : in.albedo[o];
  if (nfourier) nfourier[o] = -1;
  if (status) status[o] = RT_OK;
  if (is_missing(sza) || is_missing(vza) || is_missing(raa) || (!brdf && is_missing(alb))) {
    radiance[o] = in.missing; reflectance[o] = in.missing;
    if (brdf) brdf->br[o] = in.missing;
    return false;
  }
  double refl_db = alb;  // surface reflectance of the direct bounce
  if (brdf && brdf->kind != kBrdfRTLS) {
    // VLIDORT_Scalar_CX / _GissCX (VLIDORT_BRDF_CX.F90:512-545, :1647-1690):
    // MISSING winds or refractive index give MISSING outputs for this channel
    const double u = brdf->u10[j], v = brdf->v10[j], m = brdf->mr[i];
    if (is_missing(u) || is_missing(v) || is_missing(m)) {
      radiance[o] = in.missing; reflectance[o] = in.missing;
      brdf->br[o] = in.missing;
      return false;
    }
    const CoxMunkPars p = brdf_cm_pars(brdf->kind == kBrdfGissCoxMunk, u, v, m);
    const double b = brdf_exact_cx(p, sza, vza, raa);
    brdf->br[o] = b;
    refl_db = b;
    const Scratch B{brdf->terms + bidx, brdf->stride};
    brdf_solve_terms_cx<NS>(brdf->q, brdf->cf, brdf->qx, p, sza, vza, B);
  } else if (brdf) {
    const long w = (long)i + (long)nch * j;
    const double* kw = brdf->kw + 3 * w;
    const int t = brdf->tab ? brdf->tab[w] : 0;
    const double hb = brdf->tpar[2 * t], br = brdf->tpar[2 * t + 1];
    const double b = brdf_exact(kw, hb, br, sza, vza, raa);
    brdf->br[o] = b < 0.0 ? -500.0 : b;
    if (b < 0.0) {
      radiance[o] = -500.0; reflectance[o] = -500.0;
      return false;
    }
    refl_db = b;
    const Scratch B{brdf->terms + bidx, brdf->stride};
    brdf_solve_terms<NS>(brdf->q, brdf->qx, kw, hb, br, sza, vza, B);
    B[BrdfBlock<NS>::w + 3] = (double)t;
  }
  r.o = o;
  r.L = L;
  r.NM = (2 * NS - 1 < ngreek) ? 2 * NS - 1 : ngreek;
  r.msmode = opt.do_focorr != 0;
  r.albedo = brdf ? 1.0 : alb;  // a BRDF surface reflects in every Fourier term
  r.raa = raa;
  r.sza = sza;
  const double mu_u = cos(kDTR * vza), cos_sza = cos(sza * kDTR);
  const double sec_u = 1.0 / mu_u;
  r.mu_u = mu_u;
  r.sec_u = sec_u;
  r.cos_sza = cos_sza;
  const int NM = r.NM;
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
  // Legendre recursion factors (2l-1)/l and (l-1)/l of the single-scatter phase
  // function (FO_VectorSS_Spherfuncs.f90 DF1/DF2), once per solve
  double df1[2 * NS + 2], df2[2 * NS + 2];
  for (int l = 2; l <= ngreek && l < 2 * NS + 2; ++l) {
    df1[l] = (double)(2 * l - 1) / (double)l;
    df2[l] = (double)(l - 1) / (double)l;
  }
  for (int k = 0; k <= L; ++k) S[lay.hgt + k] = in.he[k + (long)(in.km + 1) * j] * kHeightScale;
  for (int k = 0; k < L; ++k) {
    const double ray = in.rot[k + (long)in.km * (j + (long)in.nobs * i)];
    const long a = k + (long)in.km * (i + (long)in.nch * j);
    const double tl = in.tau_f ? (double)in.tau_f[a] : in.tau[a];
    const double sl = in.ssa_f ? (double)in.ssa_f[a] : in.ssa[a];
    const double alpha_l = in.alpha ? in.alpha[k + (long)in.km * (j + (long)in.nobs * i)] : 0.0;
    const double tau_ext = alpha_l + ray + tl;
    const double tau_scat = ray + sl * tl;
    if (!(tau_ext > 0.0) || !(tau_scat > 0.0)) {
      radiance[o] = in.missing; reflectance[o] = in.missing;
      if (status) status[o] = RT_BAD_INPUT;
      return false;
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
      W[lay.og + l + 2 * NS * (long)k] = (T)(om * b);
    }
    W[lay.lnz + k] = (T)lnz;
    W[lay.om1 + k] = (T)(1.0 - om);
    S[lay.dtau + k] = dtau;
    W[lay.tdtau + k] = (T)dtau;
    // single-scatter inputs (vlidort_vfo_interface.f90:377-411; FO_VectorSS_RTCalcs_I.f90:340-380)
    const double dz = S[lay.hgt + k] - S[lay.hgt + k + 1];
    const double dts = opt.do_deltam ? dtau : tau_ext;
    S[lay.ext + k] = dts / dz;
    S[lay.dts + k] = dts;  // FO regular-PS vertical optical depth
    double tms = opt.do_deltam ? om_in / (1.0 - fdel * om_in) : om_in;
    double p0 = 1.0, p1 = cosscat, fm = beta_in(0) * p0 + (ngreek >= 1 ? beta_in(1) * p1 : 0.0);
    for (int l = 2; l <= ngreek; ++l) {
      const bool tab = l < 2 * NS + 2;  // more input moments than the table holds: divide here
      const double f1 = tab ? df1[l] : (double)(2 * l - 1) / (double)l;
      const double f2 = tab ? df2[l] : (double)(l - 1) / (double)l;
      double p2 = f1 * p1 * cosscat - f2 * p0;
      fm += p2 * beta_in(l);
      p0 = p1; p1 = p2;
    }
    S[lay.escat + k] = fm * tms;
  }
  // ---------------------------------------------------------------- single scatter
  double ss = 0.0, db = 0.0;
  r.ss = 0.0; r.db = 0.0;
  if (opt.do_focorr) {
    const bool enhanced = !opt.do_plane_parallel && !nadir_fo;
    double phi = raa;
    if (phi < 0.0) phi = -phi;
    if (phi > 360.0) phi = 360.0 - phi - 360.0;
    if constexpr (sizeof(T) == sizeof(float)) {
      if (enhanced) {
        for (int k = 0; k <= L; ++k) W[lay.wh + k] = (float)S[lay.hgt + k];
        for (int k = 0; k < L; ++k) W[lay.we + k] = (float)S[lay.ext + k];
        fo_enhanced_f32(opt, L, sza, vza, phi, refl_db, tu, wu, W, lay.wh, lay.we, S, lay.hgt, lay.ext, lay.escat, &ss,
                        &db);
      } else {
        fo_single_scatter_chord(opt, enhanced, L, sza, vza, phi, refl_db, tu, wu, S, lay.hgt, lay.ext, lay.escat,
                                lay.dts, &ss, &db);
      }
    }
    else
      fo_single_scatter_ref(opt, enhanced, L, sza, vza, phi, refl_db, tu, wu, S, lay.hgt, lay.ext, lay.escat, lay.dts,
                            &ss, &db);
  }
  // ---------------------------------------------------------------- beam attenuation
  if constexpr (sizeof(T) == sizeof(double)) {
  // Chapman factors (vlidort_geometry.f90:119-317), QSPREP / PREPTRANS / EMULT
  // (vlidort_miscsetups.f90:813-1292, 3187-3421).  The solar zenith is the
  // input angle at every level n (regular pseudo-spherical): the ray through
  // level n has impact parameter p = sin(sza) r_n, and its slant optical depth
  // to TOA is sum_k dtau_k (r_{k-1} + r_k) / (c_{k-1} + c_k).
  {
    const double mu_toa = cos_sza;
    const double sn_toa = sqrt(1.0 - mu_toa * mu_toa);
    const double R0 = opt.earth_radius;
    int cutoff = L;
    double tslant_prev = 0.0, s_t_0 = 1.0, s_t_1 = 0.0;
    bool refl_directbeam = false;
    double trans_solar_beam = 0.0;
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
        trans_solar_beam = ts < kMaxTau ? exp(-ts) : 0.0;
        refl_directbeam = ts < kMaxTau;
      }
    }
    r.cutoff = cutoff;
    r.trans_solar_beam = trans_solar_beam;
    r.refl_directbeam = refl_directbeam;
    for (int n = 0; n < L; ++n) {
      const double dtn = S[lay.dtau + n];
      double tmu = 0.0, em = 0.0;
      double sp = dtn * sec_u;
      double tus = sp > kMaxTau ? 0.0 : exp(-sp);
      const double avs = S[lay.avsec + n], itr = S[lay.itrans + n];
      if (n < cutoff) {
        double spb = dtn * avs;
        tmu = spb > kMaxTau ? 0.0 : exp(-spb);
        double su = (1.0 - tmu * tus) / (avs + sec_u);
        em = (itr * sec_u) * su;
      }
      W[lay.tavsec + n] = (T)avs;
      W[lay.titrans + n] = (T)itr;
      W[lay.tmubar + n] = (T)tmu;
      W[lay.tuser + n] = (T)tus;
      W[lay.emult + n] = (T)em;
    }
  }
  } else {
    // FP32 beam attenuation of the mixed method: the chord form of the
    // Chapman factors, each level's slant increment ts_n - ts_{n-1} formed
    // from differences of the shell terms (c_j(n-1) - c_j(n) =
    // (p_n^2 - p_{n-1}^2) / (c_j(n-1) + c_j(n)), p_n - p_{n-1} = -sin(sza) dz_n)
    // instead of a difference of cumulative slant depths.
    const float mu = (float)cos_sza, sn = (float)sqrt(1.0 - cos_sza * cos_sza);
    const float R0 = (float)opt.earth_radius, secu = (float)sec_u, maxtau = (float)kMaxTau;
    for (int k = 0; k <= L; ++k) W[lay.wh + k] = (float)S[lay.hgt + k];
    auto rad = [&](int k) { return R0 + W[lay.wh + k]; };
    const bool pp = opt.do_plane_parallel || sn == 0.0f;
    const float cf = opt.do_plane_parallel ? 1.0f / mu : 1.0f;
    int cutoff = L;
    float ts = 0.0f, s_t_0 = 1.0f, s_t_1 = 0.0f;
    for (int n = 1; n <= L; ++n) {
      const float dtn = W[lay.tdtau + n - 1];
      float dts = 0.0f;
      if (pp) {
        dts = dtn * cf;
        ts += dts;
      } else {
        const float rn = rad(n), p = sn * rn, pprev = sn * rad(n - 1);
        const float dp2 = -sn * (W[lay.wh + n - 1] - W[lay.wh + n]) * (p + pprev);  // p^2 - pprev^2
        float r_lo = rn, c_lo = rn * mu, tsn = 0.0f;
        for (int k = n; k >= 1; --k) {
          const float r_hi = rad(k - 1), c_hi = sqrtf((r_hi - p) * (r_hi + p));
          const float A = c_hi + c_lo, dt = W[lay.tdtau + k - 1];
          tsn += dt * ((r_hi + r_lo) / A);
          if (k == n) {
            dts += dt * ((r_hi + r_lo) / A);
          } else {
            const float cp_hi = W[lay.wc + k - 1], cp_lo = W[lay.wc + k];
            const float dA = dp2 / (cp_hi + c_hi) + dp2 / (cp_lo + c_lo);
            dts += dt * (r_hi + r_lo) * dA / (A * (cp_hi + cp_lo));
          }
          W[lay.wc + k] = c_lo;
          r_lo = r_hi; c_lo = c_hi;
        }
        W[lay.wc + 0] = c_lo;
        ts = tsn;
      }
      float avsec = 0.0f, itr = 0.0f;
      if (n <= cutoff) {
        if (ts > maxtau) cutoff = n;
        else s_t_1 = expf(-ts);
        avsec = dts / dtn;
        itr = s_t_0;
        s_t_0 = s_t_1;
      }
      W[lay.tavsec + n - 1] = avsec;
      W[lay.titrans + n - 1] = itr;
      if (n == L) {
        r.trans_solar_beam = ts < maxtau ? (double)expf(-ts) : 0.0;
        r.refl_directbeam = ts < maxtau;
      }
    }
    r.cutoff = cutoff;
    for (int n = 0; n < L; ++n) {
      const float dtn = W[lay.tdtau + n];
      const float sp = dtn * secu;
      const float tus = sp > maxtau ? 0.0f : expf(-sp);
      const float avs = W[lay.tavsec + n], itr = W[lay.titrans + n];
      float tmu = 0.0f, em = 0.0f;
      if (n < cutoff) {
        const float spb = dtn * avs;
        tmu = spb > maxtau ? 0.0f : expf(-spb);
        em = (itr * secu) * (-expm1f(-(avs + secu) * dtn) / (avs + secu));
      }
      W[lay.tmubar + n] = tmu;
      W[lay.tuser + n] = tus;
      W[lay.emult + n] = em;
    }
  }
  r.ss = ss;
  r.db = db;
  // vlidort_masters_V2p8p3.f90:2305-2700: Fourier terms 0..NMOMENTS (only m = 0
  // without single-scatter correction at nadir view)
  r.n_fouriers = (vza == 0.0 && !opt.do_focorr) ? 0
                 : (opt.max_fourier >= 0 && opt.max_fourier < NM ? opt.max_fourier : NM);
  return true;
}

// ---------------------------------------------------------------------------------- FP32 geometry
// The enhanced-PS single scatter of the mixed method with its geometry in
// FP32 (fo_single_scatter_chord is the FP64 form).  Radii ~6400 km carry
// 0.4 m of FP32 rounding, so no path is formed as a difference of radii:
// whole-layer chords use the layer thickness, dz (r_hi + r_lo) / (c_hi + c_lo),
// and the partial segment above a fine point uses its offset above the layer
// bottom, rf - r_lo = tf (2 c_lo + tf) / (rf + r_lo).  wh/we: heights above
// the surface [km] and extinctions [1/km] in FP32.
RT_HD float sun_path_f32(int nn, float off, float ct, float st, float R0, const ScratchT<float>& W, long wh, long we) {
  auto rad = [&](int k) { return R0 + W[wh + k]; };
  const float rs = rad(nn) + off;
  const float p = rs * st;
  float r_lo = rs, c_lo = rs * ct;
  float r_hi = rad(nn - 1), c_hi = sqrtf((r_hi - p) * (r_hi + p));
  const float dz0 = (W[wh + nn - 1] - W[wh + nn]) - off;
  float tau = W[we + nn - 1] * (dz0 * (r_hi + r_lo) / (c_hi + c_lo));
  r_lo = r_hi; c_lo = c_hi;
  for (int k = nn - 1; k >= 1; --k) {
    r_hi = rad(k - 1);
    c_hi = sqrtf((r_hi - p) * (r_hi + p));
    tau += W[we + k - 1] * ((W[wh + k - 1] - W[wh + k]) * (r_hi + r_lo) / (c_hi + c_lo));
    r_lo = r_hi; c_lo = c_hi;
  }
  return tau;
}

// Enhanced-PS first-order single scatter and direct bounce (mixed method).
// Tangent rays (sun below the local horizon at a fine point: rare at the
// angles AeroApps uses) fall back to the FP64 path.
RT_HD void fo_enhanced_f32(const RtOptions& opt, int L, double sza, double vza, double phi, double albedo,
                           const double* tu, const double* wu, const ScratchT<float>& W, long wh, long we,
                           const Scratch& S, long ohgt, long oext, long oescat, double* ss, double* db) {
  const float R0 = (float)opt.earth_radius;
  auto rad = [&](int k) { return R0 + W[wh + k]; };
  const double flux = opt.flux_factor / kPI4;
  const bool overhead = (sza == 0.0);
  const double th_R = sza * kDTR;
  double cthd, sthbd;
  if (sza == 90.0) { cthd = 0.0; sthbd = 1.0; } else { sthbd = sin(th_R); cthd = cos(th_R); }
  const float cth = (float)cthd, sthb = (float)sthbd;
  const bool donadir = (vza == 0.0);
  float raycon = 0.0f, caL = 1.0f, saL = 0.0f;
  if (!donadir) {
    const double alphaL = vza * kDTR;
    saL = (vza == 90.0) ? 1.0f : (float)sin(alphaL);
    caL = (vza == 90.0) ? 0.0f : (float)cos(alphaL);
    raycon = saL * rad(L);
  }
  float sdir0 = 0.0f, sdir2 = 0.0f;
  if (!overhead) { sdir0 = (float)(-sthbd * cos(phi * kDTR)); sdir2 = -cth; }
  const float cutoff = (float)kFoCutoff;
  float atten_boa;
  {
    float st;
    if (overhead) {
      st = 0.0f;
      for (int k = L; k >= 1; --k) st += W[we + k - 1] * (W[wh + k - 1] - W[wh + k]);
    } else {
      st = sun_path_f32(L, 0.0f, cth, sthb, R0, W, wh, we);
    }
    atten_boa = st < cutoff ? expf(-st) : 0.0f;
  }
  float cum = 0.0f, trans_above = 1.0f;
  float c_up = donadir ? 0.0f : sqrtf((rad(0) - raycon) * (rad(0) + raycon));
  for (int n = 1; n <= L; ++n) {
    const float r_up = rad(n - 1), r_lo = rad(n);
    const float dzn = W[wh + n - 1] - W[wh + n];
    float losw, c_lo;
    if (donadir) {
      losw = dzn;
      c_lo = r_lo;
    } else {
      c_lo = (n == L) ? r_lo * caL : sqrtf((r_lo - raycon) * (r_lo + raycon));
      losw = dzn * (r_up + r_lo) / (c_up + c_lo);
    }
    const float kn = W[we + n - 1];
    const float lostau = kn * losw;
    const float lostrans = lostau < cutoff ? expf(-lostau) : 0.0f;
    const bool zero_sun_boa = overhead && (n == L || donadir);
    float sum = 0.0f;
    for (int j = 0; j < opt.nfine; ++j) {
      const float tf = losw * (float)tu[j], wf = losw * (float)wu[j];
      float off, ct, st;
      if (donadir) {
        off = tf;
        ct = cth; st = sthb;
      } else {
        const float X = c_lo + tf;
        const float rf = sqrtf(raycon * raycon + X * X);
        off = tf * (2.0f * c_lo + tf) / (rf + r_lo);
        const float caf = X / rf, saf = raycon / rf;
        const float scum = saL * caf - caL * saf, ccum = caL * caf + saL * saf;
        if (overhead) { ct = ccum; st = scum; }
        else { ct = scum * sdir0 - ccum * sdir2; st = sqrtf(fmaxf(0.0f, 1.0f - ct * ct)); }
      }
      const bool dsf = donadir || overhead || (ct >= 0.0f);
      float sd;
      if (zero_sun_boa) {
        sd = W[we + n - 1] * (dzn - off);
        for (int k = n - 1; k >= 1; --k) sd += W[we + k - 1] * (W[wh + k - 1] - W[wh + k]);
      } else if (dsf) {
        sd = sun_path_f32(n, off, ct, st, R0, W, wh, we);
      } else {
        const double rfd = (double)R0 + (double)W[wh + n] + (double)off;
        sd = (float)sun_optical_path_chord(false, false, rfd, (double)ct, (double)st, n, opt.earth_radius, S, ohgt,
                                           oext, L);
      }
      const float attf = sd < cutoff ? expf(-sd) : 0.0f;
      sum += attf * expf(-kn * (losw - tf)) * wf;
    }
    cum += trans_above * (float)S[oescat + n - 1] * (sum * kn);
    trans_above *= lostrans;
    c_up = c_lo;
  }
  *ss = flux * (double)cum;
  *db = flux * (4.0 * cthd * albedo * (double)atten_boa) * (double)trans_above;
}

// Full solve of one pixel by one thread: set-up, then the Fourier series with
// the double convergence test.  qx/qw: Gauss-Legendre streams on (0,1); tu/wu:
// unit fine-layer quadrature for the enhanced-PS line of sight.  T is the
// working precision of the series.
template <int NS, typename T>
RT_HDN void solve_lambert(const RtOptions& opt, const LambertInputs& in, int sidx, const double* qx,
                          const double* qw, const double* tu, const double* wu, const SolveScratch<T>& SS,
                          double* radiance, double* reflectance, int* nfourier, int* status,
                          const Worklist& wl = Worklist()) {
  SetupRecord r;
  if (!solve_setup<NS, T>(opt, in, sidx, tu, wu, SS, radiance, reflectance, nfourier, status, r)) return;
  const ScratchLayout<NS> lay(in.km);
  SolveCtx<NS, T> c;
  make_ctx<NS, T>(r, qx, qw, c);
  FourierSum sum;
  int m = 0, st = RT_OK;
  for (m = 0; m <= r.n_fouriers; ++m) {
    T sf = 0;
    st = fourier_term<NS, T>(c, opt, m, SS.W, lay, &sf);
    if (st != RT_OK || sum.add(opt, r, m, (double)sf)) break;
  }
  solve_finish(opt, in, r, st, m, sum.stokes, radiance, reflectance, nfourier, status);
  wl.flag(sum, st, sidx);
}

}  // namespace aerort
