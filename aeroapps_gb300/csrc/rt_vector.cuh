// Polarized (NSTOKES = 3) VLIDORT-style solve of one (column, wavelength), run
// by the 32 lanes of one warp: VLIDORT_Vector_Lambert's configuration
// (geo_vlidort/VLIDORT_LAMBERT.F90:172-342 -> VLIDORT_ScatMod.F90:284-617 ->
// VLIDORT 2.8.3 regular solar path with NSTOKES = 3).
//
// Layout of the work:
// - set-up: the scalar set-up of rt_solve.cuh (layer mixing of the (1,1)
//   Greek entry, delta-M, Chapman factors, beam transmittances, first-order
//   single scatter of I), run by lane 0, plus the other Greek entries of the
//   16-entry mixing (VLIDORT_ScatMod.F90:446-546) and the Q, U single scatter
//   (FO_VectorSS_Spherfuncs.f90: P02 function and the rotation of the
//   scattering plane), lane per layer;
// - per Fourier term: generalized spherical functions (Siewert 1982 recursion,
//   vlidort_miscsetups.f90:2273-2935), lane per stream; then layer by layer:
//   the 3N x 3N sum and difference matrices (vlidort_solutions.f90:436-476),
//   lane per matrix element; the real eigen-decomposition of DAB.SAB
//   (Householder reduction to Hessenberg form, shifted QR, back substitution
//   on the triangular Schur form: the same algorithm family as the
//   reference's ASYMTX, vlidort_aux.f90:386-958); the solution vectors, user-
//   angle solutions, Green's-function particular integral (vlidort_solutions.f90
//   :1051-1508, 2649-3073), lane per eigen-solution; and one step of a block
//   Riccati sweep of the boundary-value problem, a pivoted 6N x 6N elimination
//   in shared memory with lanes over rows, which replaces the reference's
//   banded LU of the whole 6NL system (vlidort_bvproblem.f90:627-2315);
// - back substitution, then the TOA source recursion (intensity.f90:145,
//   PostProcessing.f90:139) and the Fourier sum with the intensity-only double
//   convergence test (converge.f90:825-1236; cos m phi for I and Q, sin m phi
//   for U, AZMFAC in masters :2608-2625).
// Everything is FP64.  Working arrays of one solve live in a per-warp global
// region (VecLayout); the matrices of the current layer in shared memory
// (VecShared).  The same code runs on the host with one std::thread per lane
// (tests/host_harness/rt_vector_host.cpp).
#pragma once
#include "rt_team.cuh"

namespace aerort {

constexpr int kStokes = 3;

// Device view of the VLIDORT_Vector_Lambert argument list (VLIDORT_LAMBERT.F90
// :172-240), Fortran column-major, FP64 (FP32 optics optional).
struct VectorInputs {
  LambertInputs base;           // rot, depol, tau, ssa, pmom (P11 block first), he, albedo, angles, nlay, alpha ...
  const double* flux_factor;    // (nch, nobs) or null (= 1)
};

// Offsets (in doubles) of one warp's global working region.
template <int N>
struct VecLayout {
  static constexpr int K = kStokes * N, NMX = 2 * N, NA = N + 2;
  long setup, og, escq, escu, pi, pimm, h2s, h2d, xp[2], xn[2], lay0, lstride, total;
  // per-layer block members (offsets inside a layer block)
  static constexpr long kTeig = 0, kUdn = K, kUup = 4 * K, kHm1 = 7 * K, kHm2 = 8 * K, kAt = 9 * K, kBt = 10 * K,
                        kGp = 11 * K, kGm = 12 * K, kWu = 13 * K, kWl = 13 * K + 6 * N, kF = 13 * K + 12 * N,
                        kf = kF + (long)K * K, kG = kf + K, kg = kG + (long)K * K, kLc = kg + K, kMc = kLc + K,
                        kEnd = kMc + K;
  RT_HD explicit VecLayout(int L) {
    const ScratchLayout<N> sl(L, false);
    long o = 0;
    setup = o; o += sl.d_total + sl.t_total;
    og = o; o += (long)NMX * L * 9;
    escq = o; o += L;
    escu = o; o += L;
    pi = o; o += (long)NMX * NA * 9;
    pimm = o; o += 2 * NA;
    h2s = o; o += (long)kStokes * NMX * kStokes * N;
    h2d = o; o += (long)kStokes * NMX * kStokes * N;
    for (int b = 0; b < 2; ++b) {
      xp[b] = o; o += 2L * K * K;
      xn[b] = o; o += 2L * K * K;
    }
    lay0 = o;
    lstride = kEnd;
    o += lstride * L;
    total = o;
  }
};

// Shared-memory working set of one warp.  Eigen phase: SAB, DAB, the
// Hessenberg/Schur matrix H and the accumulated orthogonal Z (column-major,
// leading dimension K + 1).  Boundary-value phase: the augmented interface
// system, 2K rows of [A (2K) | B (K) | rhs] (row-major, stride LR).
template <int N>
struct VecShared {
  static constexpr int K = kStokes * N, LD = K + 1, LR = 3 * K + 1;
  static constexpr int EIG = 4 * K * LD, AUG = 2 * K * LR;
  double m[EIG > AUG ? EIG : AUG];
  double v[K + 2];          // Householder vector
  double red[2 * kTeam];    // reductions
  int ired[2 * kTeam];
  RT_HD double* S() { return m; }
  RT_HD double* D() { return m + K * LD; }
  RT_HD double* H() { return m + 2 * K * LD; }
  RT_HD double* Z() { return m + 3 * K * LD; }
  RT_HD double* aug() { return m; }
};

// Sum of v over the warp (every lane gets it).
RT_HD double warp_sum(const Team& tm, double v, double* red) { return group_sum<kTeam, double>(tm, v, red); }

// Maximum of v over the warp and the lowest lane holding it (v >= 0 on lanes with a candidate).
RT_HD int warp_argmax(const Team& tm, double v, double* red, double* vmax) {
  return team_argmax_lane<double>(tm, v, red, vmax);
}

// ------------------------------------------------------------------------------- dense kernels
// Real eigen-decomposition of the n x n matrix H (column-major, leading
// dimension ld, destroyed): eigenvalues ev[n], right eigenvectors in the
// columns of X (ld).  Householder reduction to upper Hessenberg form with the
// transformations accumulated in Z, shifted QR (Wilkinson shift, Givens
// rotations, deflation at negligible subdiagonals) to the upper-triangular
// Schur form T = Z^T H Z, eigenvectors of T by back substitution, X = Z Y.
// Assumes real eigenvalues (the reference's ASYMTX does too).  Returns false
// if the QR iteration does not converge.  Y uses the storage of X.
RT_HD bool team_eigen(const Team& tm, int n, int ld, double* H, double* Zm, double* X, double* ev, double* v,
                      double* red) {
  auto A = [&](int i, int j) -> double& { return H[i + ld * j]; };
  auto Zz = [&](int i, int j) -> double& { return Zm[i + ld * j]; };
  for (int e = tm.lane; e < n * n; e += kTeam) Zz(e % n, e / n) = (e % n == e / n) ? 1.0 : 0.0;
  tm.sync();
  // ---- Householder reduction to Hessenberg form
  for (int k = 0; k < n - 2; ++k) {
    double ss = 0.0;
    for (int i = k + 1 + tm.lane; i < n; i += kTeam) ss += A(i, k) * A(i, k);
    const double nrm2 = warp_sum(tm, ss, red);
    const double x0 = A(k + 1, k);
    const double tail = nrm2 - x0 * x0;
    tm.sync();
    if (!(tail > 0.0)) continue;  // already reduced in this column
    const double nrm = sqrt(nrm2);
    const double alpha = x0 > 0.0 ? -nrm : nrm;
    // v = x - alpha e1, beta = 2 / v.v = 1 / (nrm2 - alpha x0)
    for (int i = k + 1 + tm.lane; i < n; i += kTeam) v[i] = (i == k + 1) ? x0 - alpha : A(i, k);
    const double beta = 1.0 / (nrm2 - alpha * x0);
    tm.sync();
    // H <- (I - beta v v^T) H, columns k..n-1
    for (int j = k + tm.lane; j < n; j += kTeam) {
      double w = 0.0;
      for (int i = k + 1; i < n; ++i) w += v[i] * A(i, j);
      w *= beta;
      for (int i = k + 1; i < n; ++i) A(i, j) -= w * v[i];
    }
    tm.sync();
    // H <- H (I - beta v v^T), Z <- Z (I - beta v v^T): rows 0..n-1
    for (int i = tm.lane; i < n; i += kTeam) {
      double w = 0.0, wz = 0.0;
      for (int j = k + 1; j < n; ++j) { w += A(i, j) * v[j]; wz += Zz(i, j) * v[j]; }
      w *= beta; wz *= beta;
      for (int j = k + 1; j < n; ++j) { A(i, j) -= w * v[j]; Zz(i, j) -= wz * v[j]; }
    }
    tm.sync();
    for (int i = k + 2 + tm.lane; i < n; i += kTeam) A(i, k) = 0.0;
    if (tm.lane == 0) A(k + 1, k) = alpha;
    tm.sync();
  }
  // ---- shifted QR on the Hessenberg matrix
  const double eps = 2.220446049250313e-16;
  int hi = n - 1, its = 0, total = 0;
  while (hi > 0) {
    // deflation point: largest lo with a negligible subdiagonal H(lo, lo-1)
    int lo = hi;
    while (lo > 0) {
      const double s = fabs(A(lo - 1, lo - 1)) + fabs(A(lo, lo));
      if (fabs(A(lo, lo - 1)) <= eps * (s > 0.0 ? s : 1.0)) break;
      --lo;
    }
    tm.sync();
    if (lo == hi) {  // one eigenvalue converged
      if (tm.lane == 0) A(hi, hi - 1) = 0.0;
      tm.sync();
      --hi;
      its = 0;
      continue;
    }
    if (lo == hi - 1) {
      // an isolated 2 x 2 block: both eigenvalues at once, as ASYMTX's
      // "two eigenvalues found" step (vlidort_aux.f90 ASYMTX): with
      // p = (y - x) / 2, q = p^2 + w, the eigenvalues x + z and x - w / z for
      // z = p + sign(p) sqrt(|q|) -- real even when rounding leaves a nearly
      // degenerate pair complex (q < 0), where a real QR step would never
      // split the block -- and the rotation by the eigenvector (z, c) / r.
      const double xd = A(hi, hi), yd = A(hi - 1, hi - 1), cd = A(hi, hi - 1), wd = cd * A(hi - 1, hi);
      const double pd = 0.5 * (yd - xd), qd = pd * pd + wd;
      const double zd = pd + copysign(sqrt(fabs(qd)), pd);
      const double l1 = xd + zd, l2 = (zd != 0.0) ? xd - wd / zd : l1;
      const double rd = sqrt(cd * cd + zd * zd);
      const double cp = rd > 0.0 ? cd / rd : 0.0, cq = rd > 0.0 ? zd / rd : 1.0;
      tm.sync();
      for (int j = hi - 1 + tm.lane; j < n; j += kTeam) {
        const double a1 = A(hi - 1, j), a2 = A(hi, j);
        A(hi - 1, j) = cq * a1 + cp * a2;
        A(hi, j) = cq * a2 - cp * a1;
      }
      tm.sync();
      for (int i = tm.lane; i < n; i += kTeam) {
        if (i <= hi) {
          const double a1 = A(i, hi - 1), a2 = A(i, hi);
          A(i, hi - 1) = cq * a1 + cp * a2;
          A(i, hi) = cq * a2 - cp * a1;
        }
        const double z1 = Zz(i, hi - 1), z2 = Zz(i, hi);
        Zz(i, hi - 1) = cq * z1 + cp * z2;
        Zz(i, hi) = cq * z2 - cp * z1;
      }
      tm.sync();
      if (tm.lane == 0) {
        A(hi, hi - 1) = 0.0;
        A(hi - 1, hi - 1) = l1;
        A(hi, hi) = l2;
      }
      tm.sync();
      hi -= 2;
      its = 0;
      continue;
    }
    if (++total > 60 * n) return false;
    ++its;
    // Wilkinson shift from the trailing 2x2 block (real part if complex);
    // an exceptional shift every 10 iterations without deflation
    const double a = A(hi - 1, hi - 1), b = A(hi - 1, hi), c = A(hi, hi - 1), d = A(hi, hi);
    double mu;
    if (its % 10 == 0) {
      mu = d + 1.5 * fabs(c);
    } else {
      const double tr = 0.5 * (a + d), df = 0.5 * (a - d);
      const double disc = df * df + b * c;
      if (disc >= 0.0) {
        const double r = sqrt(disc);
        const double l1 = tr + r, l2 = tr - r;
        mu = fabs(l1 - d) < fabs(l2 - d) ? l1 : l2;
      } else {
        mu = tr;
      }
    }
    tm.sync();
    // QR step on rows/columns lo..hi: H - mu I = Q R, H <- R Q + mu I, by Givens
    // rotations; rows are updated over columns lo..n-1 and columns over rows
    // 0..hi (the full Schur form), Z over all rows.
    double x = A(lo, lo) - mu, y = A(lo + 1, lo);
    for (int k = lo; k < hi; ++k) {
      double r = hypot(x, y);
      double cs = r > 0.0 ? x / r : 1.0, sn = r > 0.0 ? y / r : 0.0;
      tm.sync();
      // rotate rows k, k+1 (G^T from the left)
      for (int j = (k > lo ? k - 1 : lo) + tm.lane; j < n; j += kTeam) {
        const double h1 = A(k, j), h2 = A(k + 1, j);
        A(k, j) = cs * h1 + sn * h2;
        A(k + 1, j) = -sn * h1 + cs * h2;
      }
      tm.sync();
      // rotate columns k, k+1 (G from the right) over rows 0..min(k+2, hi), and Z
      const int rmax = (k + 2 < hi ? k + 2 : hi);
      for (int i = tm.lane; i < n; i += kTeam) {
        if (i <= rmax) {
          const double h1 = A(i, k), h2 = A(i, k + 1);
          A(i, k) = cs * h1 + sn * h2;
          A(i, k + 1) = -sn * h1 + cs * h2;
        }
        const double z1 = Zz(i, k), z2 = Zz(i, k + 1);
        Zz(i, k) = cs * z1 + sn * z2;
        Zz(i, k + 1) = -sn * z1 + cs * z2;
      }
      tm.sync();
      if (k + 1 < hi) { x = A(k + 1, k); y = A(k + 2, k); }
    }
    tm.sync();
  }
  // ---- eigenvalues and eigenvectors of the triangular T (lane per eigenvector)
  double tnorm = 0.0;
  for (int e = tm.lane; e < n * n; e += kTeam) {
    const int i = e % n, j = e / n;
    if (i <= j) tnorm = fmax(tnorm, fabs(A(i, j)));
  }
  for (int o = 1; o < kTeam; o <<= 1) {
#ifdef __CUDA_ARCH__
    tnorm = fmax(tnorm, __shfl_xor_sync(0xffffffffu, tnorm, o));
#else
    red[tm.lane] = tnorm;
    tm.sync();
    tnorm = fmax(tnorm, red[tm.lane ^ o]);
    tm.sync();
#endif
  }
  const double small = eps * (tnorm > 0.0 ? tnorm : 1.0);
  for (int k = tm.lane; k < n; k += kTeam) {
    const double lam = A(k, k);
    ev[k] = lam;
    double* y = X + ld * k;
    for (int i = k + 1; i < n; ++i) y[i] = 0.0;
    y[k] = 1.0;
    for (int j = k - 1; j >= 0; --j) {
      double s = 0.0;
      for (int i = j + 1; i <= k; ++i) s += A(j, i) * y[i];
      double den = A(j, j) - lam;
      if (fabs(den) < small) den = den < 0.0 ? -small : small;
      y[j] = -s / den;
    }
  }
  tm.sync();
  // X <- Z Y (Y upper triangular; results to H's storage, then copied back)
  for (int e = tm.lane; e < n * n; e += kTeam) {
    const int i = e % n, k = e / n;
    double s = 0.0;
    for (int j = 0; j <= k; ++j) s += Zz(i, j) * X[j + ld * k];
    A(i, k) = s;
  }
  tm.sync();
  for (int e = tm.lane; e < n * n; e += kTeam) X[(e % n) + ld * (e / n)] = A(e % n, e / n);
  tm.sync();
  return true;
}

// Gaussian elimination with partial pivoting of the n x n system in the first
// n columns of the row-major augmented matrix M (row stride lr), applied to its
// nr right-hand-side columns n..n+nr-1, which receive the solution.  Lanes own
// rows in the elimination and right-hand sides in the back substitution.
// Returns false on a zero pivot.
RT_HD bool team_gauss(const Team& tm, int n, int nr, int lr, double* M, double* red, int* ired) {
  const int nc = n + nr;
  for (int c = 0; c < n; ++c) {
    double best = -1.0;
    int brow = -1;
    for (int r = c + tm.lane; r < n; r += kTeam) {
      const double a = fabs(M[(long)r * lr + c]);
      if (a > best) { best = a; brow = r; }
    }
    double vmax;
    const int src = warp_argmax(tm, best, red, &vmax);
    if (tm.lane == src) ired[0] = brow;
    tm.sync();
    const int p = ired[0];
    tm.sync();
    if (!(vmax > 0.0)) return false;
    if (p != c)
      for (int j = c + tm.lane; j < nc; j += kTeam) {
        const double t = M[(long)p * lr + j];
        M[(long)p * lr + j] = M[(long)c * lr + j];
        M[(long)c * lr + j] = t;
      }
    tm.sync();
    const double* pr = M + (long)c * lr;
    const double inv = 1.0 / pr[c];
    for (int r = c + 1 + tm.lane; r < n; r += kTeam) {
      double* rr = M + (long)r * lr;
      const double f = rr[c] * inv;
      if (f != 0.0)
        for (int j = c + 1; j < nc; ++j) rr[j] -= f * pr[j];
    }
    tm.sync();
  }
  for (int q = tm.lane; q < nr; q += kTeam) {
    for (int r = n - 1; r >= 0; --r) {
      const double* rr = M + (long)r * lr;
      double s = rr[n + q];
      for (int j = r + 1; j < n; ++j) s -= rr[j] * M[(long)j * lr + n + q];
      M[(long)r * lr + n + q] = s / rr[r];
    }
  }
  tm.sync();
  return true;
}

// ------------------------------------------------------------------------------- one solve
// Polarized solve of solve index sidx (= pixel * nch + channel).  ws: this
// warp's working region (VecLayout<N>(in.km).total doubles).  Outputs of
// VLIDORT_Vector_Lambert (radiance, reflectance, Q, U; MISSING for missing
// inputs or failed solves) plus the last Fourier term and the status.
template <int N>
RT_HDN void vec_solve(const Team& tm, VecShared<N>& sh, const RtOptions& opt0, const VectorInputs& vin, int sidx,
                      const double* qx, const double* qw, const double* tu, const double* wu, double* ws,
                      double* radiance, double* reflectance, double* Qo, double* Uo, int* nfourier, int* status) {
  constexpr int K = kStokes * N, K2 = 2 * K, NMX = 2 * N, NA = N + 2, LD = VecShared<N>::LD;
  const LambertInputs& in = vin.base;
  const int nch = in.nch, jp = sidx / nch, ich = sidx % nch;
  const long o = (long)jp + (long)in.nobs * ich;
  const VecLayout<N> lay(in.km);
  const ScratchLayout<N> sl(in.km, false);
  const SolveScratch<double> SS = make_scratch<N, double>(ws + lay.setup, 0, 1, in.km, false);
  const Scratch& S = SS.D;
  const ScratchT<double>& W = SS.W;
  RtOptions opt = opt0;
  opt.flux_factor = vin.flux_factor ? vin.flux_factor[ich + (long)nch * jp] : 1.0;
  // ---------------------------------------------------------------- scalar set-up (lane 0)
  if (tm.lane == 0) {
    SetupRecord r;
    const bool live = solve_setup<N, double>(opt, in, sidx, tu, wu, SS, radiance, reflectance, nfourier, status, r);
    if (live) r.store(S, sl.rec);
    sh.ired[1] = live ? 1 : 0;
    if (!live) { Qo[o] = radiance[o]; Uo[o] = radiance[o]; }
  }
  tm.sync();
  if (!sh.ired[1]) return;
  SetupRecord r;
  r.load(S, sl.rec);
  const int L = r.L, NM = r.NM, NM1 = NM + 1, ngreek = in.nmom;
  // ---------------------------------------------------------------- vector Greek entries and Q, U single scatter
  // VLIDORT_ScatMod.F90:446-546 (entries (1,2) = (2,1), (2,2), (3,3); Rayleigh
  // gamma2, alpha2 with the REAL*4 sqrt(6.)), delta-M of the KTYPE entries
  // (vlidort_miscsetups.f90:484-515), SSALBINIT; FO exactscat Q = -tms F12 C2,
  // U = tms F12 S2 (FO_VectorSS_RTCalcs_I.f90:408-432).
  const double dep = in.depol[ich];
  const double gammamom2 = -(double)sqrtf(6.0f) * (1.0 - dep) / (2.0 + dep);
  const double alphamom2 = 6.0 * (1.0 - dep) / (2.0 + dep);
  const double raysmom2 = (1.0 - dep) / (2.0 + dep);
  const long nk = (long)in.km * in.nch * in.nobs;
  const double sza = r.sza, vza = in.vza[jp], raa = r.raa;
  // scattering cosine and rotation (FO_VectorSS_Spherfuncs.f90:191-293)
  double cosscat, c2 = 0.0, s2 = 0.0;
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
    const double small = 1.0e-12;
    const double salpha = sin(kDTR * vza), calpha = cos(kDTR * vza), ctheta = cos(kDTR * sza);
    const double hs = 1.0 - cosscat * cosscat, sinscat = hs <= 0.0 ? small : sqrt(hs);
    double csig2;
    if (fabs(sinscat) <= small) csig2 = 0.0;
    else if (salpha == 0.0) csig2 = -cos(kDTR * raa);
    else csig2 = (-ctheta - calpha * cosscat) / sinscat / salpha;
    if (csig2 > 1.0) csig2 = 1.0;
    if (csig2 < -1.0) csig2 = -1.0;
    const double ssig2 = fabs(csig2 - 1.0) < small ? 0.0 : sqrt(1.0 - csig2 * csig2);
    c2 = 2.0 * csig2 * csig2 - 1.0;
    s2 = raa <= 180.0 ? 2.0 * csig2 * ssig2 : -2.0 * csig2 * ssig2;
  }
  for (int k = tm.lane; k < L; k += kTeam) {
    const double ray = in.rot[k + (long)in.km * (jp + (long)in.nobs * ich)];
    const long a = k + (long)in.km * (ich + (long)in.nch * jp);
    const double tl = in.tau_f ? (double)in.tau_f[a] : in.tau[a];
    const double sl_ = in.ssa_f ? (double)in.ssa_f[a] : in.ssa[a];
    const double al = in.alpha ? in.alpha[k + (long)in.km * (jp + (long)in.nobs * ich)] : 0.0;
    const double tau_ext = al + ray + tl, tau_scat = ray + sl_ * tl;
    double om_in = tau_scat / tau_ext;
    if (om_in > kSsaCap) om_in = kSsaCap;
    const double aerswt = sl_ * tl / tau_scat, rayswt = ray / tau_scat;
    auto pm = [&](int l, int ip) -> double {  // aerosol moment l of element ip (0-based nPol index)
      if (l >= ngreek) return 0.0;
      const long e = a + nk * ((long)l + (long)ngreek * ip);
      return in.pmom_f ? (double)in.pmom_f[e] : in.pmom[e];
    };
    // GREEKMAT_TOTAL_INPUT(l, k, entry); entries 0 = (1,1), 1 = (1,2) = (2,1), 5 = (2,2), 10 = (3,3)
    auto gin = [&](int l, int ent) -> double {
      if (ent == 0) {  // as beta_in of solve_setup
        if (l == 0) return 1.0;
        const double am = pm(l, 0);
        if (l == 2) return raysmom2 * rayswt + am * aerswt;
        return (l <= ngreek) ? am * aerswt : 0.0;
      }
      if (ent == 1) return l == 2 ? gammamom2 * rayswt + pm(l, 1) * aerswt : pm(l, 1) * aerswt;
      if (ent == 5) return l == 2 ? alphamom2 * rayswt + pm(l, 4) * aerswt : pm(l, 4) * aerswt;
      return l <= 2 ? 0.0 * rayswt + pm(l, 2) * aerswt : pm(l, 2) * aerswt;  // ent 10 (Rayleigh entry 11 is 0)
    };
    double fdel = 0.0, fac1 = 1.0, fac2 = 1.0;
    if (opt.do_deltam) {
      fdel = gin(NM + 1, 0) / (double)(2 * (NM + 1) + 1);
      fac2 = 1.0 - fdel;
      fac1 = 1.0 - fdel * om_in;
    }
    double om = opt.do_deltam ? om_in * fac2 / fac1 : om_in;
    if (om > 0.999999999) om = 0.999999999;
    else if (om < 1.0e-9) om = 1.0e-9;
    for (int l = 0; l <= NM; ++l) {
      const double fd = fdel * (double)(2 * l + 1);
      // (o1, o2) pairs: (0,0) is the scalar entry (W og); (0,1), (1,0) KTYPE2; (1,1), (2,2) KTYPE1
      const double g01 = opt.do_deltam ? gin(l, 1) / fac2 : gin(l, 1);
      const double g11 = opt.do_deltam ? (gin(l, 5) - fd) / fac2 : gin(l, 5);
      const double g22 = opt.do_deltam ? (gin(l, 10) - fd) / fac2 : gin(l, 10);
      double* ogl = ws + lay.og + l + (long)NMX * k;
      const long so = (long)NMX * L;
      for (int e = 0; e < 9; ++e) ogl[so * e] = 0.0;
      ogl[so * 0] = W[sl.og + l + 2 * N * (long)k];  // om * beta(1,1) (busters applied)
      ogl[so * (0 + 3 * 1)] = om * g01;            // (o1=0, o2=1)
      ogl[so * (1 + 3 * 0)] = om * g01;            // (o1=1, o2=0)
      ogl[so * (1 + 3 * 1)] = om * g11;
      ogl[so * (2 + 3 * 2)] = om * g22;
    }
    // single scatter, Q and U
    const double tms = opt.do_deltam ? om_in / (1.0 - fdel * om_in) : om_in;
    double f12 = 0.0;
    {
      const double qroot6 = -0.25 * sqrt(6.0);
      double pm2 = 0.0, pm1 = 0.0, sql41 = 0.0;  // P02 at l-2, l-1 (zero for l < 2)
      for (int l = 2; l <= ngreek; ++l) {
        double p;
        if (l == 2) {
          p = qroot6 * (1.0 - cosscat) * (1.0 + cosscat);
          sql41 = 0.0;
        } else {
          const double sql4 = sql41, dl = (double)l;
          sql41 = sqrt(dl * dl - 4.0);
          p = ((double)(2 * l - 1) / sql41) * cosscat * pm1 - (sql4 / sql41) * pm2;
        }
        f12 += p * gin(l, 1);
        pm2 = pm1; pm1 = p;
      }
    }
    ws[lay.escq + k] = tms * (-f12 * c2);
    ws[lay.escu + k] = tms * (f12 * s2);
  }
  tm.sync();
  double ssq = 0.0, ssu = 0.0;
  if (opt.do_focorr && tm.lane < 2) {
    const bool nadir_fo = in.nadir_first ? (jp >= *in.nadir_first) : false;
    const bool enhanced = !opt.do_plane_parallel && !nadir_fo;
    double phi = raa;
    if (phi < 0.0) phi = -phi;
    if (phi > 360.0) phi = 360.0 - phi - 360.0;
    double ss = 0.0, db = 0.0;
    // the FP64 scratch S starts at ws + lay.setup: the Q/U source arrays sit at
    // S offsets lay.escq - lay.setup and lay.escu - lay.setup
    fo_single_scatter_ref(opt, enhanced, L, sza, vza, phi, r.albedo, tu, wu, S, sl.hgt, sl.ext,
                          (tm.lane == 0 ? lay.escq : lay.escu) - lay.setup, sl.dts, &ss, &db);
    (void)db;
    sh.red[tm.lane] = ss;
  }
  tm.sync();
  if (opt.do_focorr) { ssq = sh.red[0]; ssu = sh.red[1]; }
  tm.sync();
  // ---------------------------------------------------------------- Fourier series
  const double mu_u = r.mu_u, sec_u = r.sec_u, cos_sza = r.cos_sza, albedo = r.albedo;
  const int cutoff = r.cutoff;
  double* PI = ws + lay.pi;
  auto PIX = [&](int l, int i, int s1, int s2) -> double& { return PI[l + NMX * (i + NA * (s1 + 3 * s2))]; };
  auto dm = [](int s) { return s < 2 ? 1.0 : -1.0; };
  // DO_LAYER_SCATTERING(m, n) (vlidort_inputs.f90:4321-4330): some input (1,1)
  // moment l = m..NM of the layer is non-zero (lnz = last non-zero moment)
  auto laysc = [&](int m, int n) -> bool { return m < 3 || (int)W[sl.lnz + n] >= m; };
  double stokes[3] = {0.0, 0.0, 0.0};
  int testconv = 0, st = RT_OK, m = 0;
  for (m = 0; m <= r.n_fouriers; ++m) {
    const bool incl_surface = (m == 0) && (albedo != 0.0);
    const double surface_factor = (m == 0) ? 2.0 : 1.0, delta_factor = (m == 0) ? 1.0 : 2.0;
    const double kmult = incl_surface ? surface_factor * albedo : 0.0;
    double direct_beam = 0.0;
    const bool localbeam = incl_surface && r.refl_directbeam;
    if (localbeam) direct_beam = ((opt.flux_factor * (4.0 * cos_sza / delta_factor) / kPI4) * r.trans_solar_beam) * albedo;
    // ------------------------------------------ generalized spherical functions (lane per stream)
    for (int i = tm.lane; i < NA; i += kTeam) {
      const double x = i < N ? qx[i] : (i == N ? mu_u : cos_sza);
      const double xsq = x * x, umxsq = 1.0 - xsq;
      double rt = 0.0, xrt = 0.0, upx = 0.0, m2x = 0.0;
      if (x != 1.0) { rt = sqrt(umxsq); xrt = rt * x; upx = (1.0 + xsq) / umxsq; m2x = -2.0 * x / umxsq; }
      const double rc20 = 0.25 * sqrt(6.0), rc21 = 2.0 * rc20;
      for (int l = 0; l <= NM; ++l)
        for (int e = 0; e < 9; ++e) PI[l + NMX * (i + NA * e)] = 0.0;
      auto XL = [&](int l, int s) -> double {
        if (m == 0) return s == 0 ? 1.0 / (double)(l + 1) : 1.0 / sqrt((double)((l + 3) * (l - 1)));
        const double d = (double)(l + 1 - m);
        if (s == 0) return 1.0 / d;
        if (l == 1) return 0.0;
        return 1.0 / (sqrt((double)((l + 3) * (l - 1))) * d / (double)(l + 1));
      };
      auto lsq4 = [](int l) { return l >= 3 ? sqrt((double)(l * l - 4)) : 0.0; };
      auto YL = [&](int l, int s) -> double {
        if (m == 0) return s == 0 ? (double)l : lsq4(l);
        if (l == m) return 0.0;
        const double d = (double)(l + m);
        return s == 0 ? d : d * lsq4(l) / (double)l;
      };
      auto ZL = [&](int l, int s1, int s3) -> double {
        if (m == 0 || l < 2) return 0.0;
        if ((s1 == 1 && s3 == 2) || (s1 == 2 && s3 == 1))
          return (double)m * (2.0 * (double)(2 * l + 1) / (double)(l + 1) / (double)l);
        return 0.0;
      };
      auto P = [&](int l, int s1, int s2) -> double& { return PIX(l, i, s1, s2); };
      double* pimm = ws + lay.pimm;
      int lstart;
      if (m == 0) {
        P(0, 0, 0) = 1.0;
        if (NM >= 1) P(1, 0, 0) = x;
        if (NM >= 2) { P(2, 0, 0) = 0.5 * (3.0 * xsq - 1.0); P(2, 1, 1) = rc20 * umxsq; P(2, 2, 2) = P(2, 1, 1); }
        lstart = 2;
      } else if (m == 1) {
        P(1, 0, 0) = rt;
        if (NM >= 2) {
          P(2, 0, 0) = 3.0 * xrt; P(2, 1, 1) = -rc21 * xrt; P(2, 1, 2) = rc21 * rt;
          P(2, 2, 2) = P(2, 1, 1); P(2, 2, 1) = P(2, 1, 2);
        }
        lstart = 2;
      } else {
        double& p11 = pimm[i];
        double& pkm = pimm[NA + i];
        if (m == 2) {
          p11 = 3.0 * umxsq;
          pkm = (x == 1.0) ? rc21 : rc21 * umxsq;
        } else {
          const double h1 = (double)(2 * (m - 1) + 1);
          const double h2 = (double)m * h1 / sqrt((double)((m + 2) * (m - 2)));
          p11 = h1 * rt * p11;
          pkm = (x == 1.0) ? 0.0 : h2 * rt * pkm;
        }
        P(m, 0, 0) = p11;
        if (x == 1.0) { P(m, 1, 1) = pkm * 2.0; P(m, 1, 2) = -pkm * 2.0; }
        else { P(m, 1, 1) = pkm * upx; P(m, 1, 2) = pkm * m2x; }
        P(m, 2, 2) = P(m, 1, 1);
        P(m, 2, 1) = P(m, 1, 2);
        if (m < NM)
          for (int s1 = 0; s1 < 3; ++s1)
            for (int s2 = 0; s2 < 3; ++s2) {
              double hz = 0.0;
              for (int s3 = 0; s3 < 3; ++s3) hz += ZL(m, s1, s3) * P(m, s3, s2);
              P(m + 1, s1, s2) = (x * (double)(2 * m + 1) * P(m, s1, s2) + hz) * XL(m, s1);
            }
        lstart = m + 1;
      }
      for (int l = lstart; l <= NM - 1; ++l)
        for (int s1 = 0; s1 < 3; ++s1)
          for (int s2 = 0; s2 < 3; ++s2) {
            double hz = 0.0;
            for (int s3 = 0; s3 < 3; ++s3) hz += ZL(l, s1, s3) * P(l, s3, s2);
            P(l + 1, s1, s2) = (x * (double)(2 * l + 1) * P(l, s1, s2) - YL(l, s1) * P(l - 1, s1, s2) + hz) * XL(l, s1);
          }
      // normalisation [(l-m)!/(l+m)!]^1/2
      double phi = 1.0;
      for (int q = 1; q <= 2 * m; ++q) phi *= (double)q;
      phi = 1.0 / phi;
      for (int l = m; l <= NM; ++l) {
        if (l > m) phi *= (double)(l - m) / (double)(l + m);
        const double pn = sqrt(phi);
        for (int e = 0; e < 9; ++e) PI[l + NMX * (i + NA * e)] *= pn;
      }
      for (int l = 0; l < m; ++l)
        for (int e = 0; e < 9; ++e) PI[l + NMX * (i + NA * e)] = 0.0;
    }
    tm.sync();
    // xqp = PI(q); xqm_pre = D PI sgn; xqm_post = PI D sgn; xum = D PI D sgn; xup_pre = D PI
    auto sg = [&](int l) { return ((l - m) & 1) ? -1.0 : 1.0; };
    // ------------------------------------------ layers: eigen-solutions, particular integrals, BVP sweep
    for (int n = 0; n < L && st == RT_OK; ++n) {
      const int cb = n & 1, pb = cb ^ 1;
      double* XPc = ws + lay.xp[cb];
      double* XNc = ws + lay.xn[cb];
      double* LB = ws + lay.lay0 + lay.lstride * n;
      const double* OG = ws + lay.og;
      const long so = (long)NMX * L;
      auto og = [&](int l, int o1, int o2) { return OG[l + (long)NMX * n + so * (o1 + 3 * o2)]; };
      const double dtau = S[sl.dtau + n];
      const bool lsc = laysc(m, n);
      // H2S/H2D(o3, l, o2, j) = sum_s og(l, o3, s) PI(l, j, s, o2) (1 +- D_s sgn)
      double* h2s = ws + lay.h2s;
      double* h2d = ws + lay.h2d;
      for (int e = tm.lane; e < 3 * NM1 * 3 * N; e += kTeam) {
        const int o3 = e % 3, l = (e / 3) % NM1, o2 = (e / (3 * NM1)) % 3, j = e / (9 * NM1);
        double hp = 0.0, hm = 0.0;
        if (l >= m)
          for (int s = 0; s < 3; ++s) {
            const double a = og(l, o3, s) * PIX(l, j, s, o2);
            const double b = og(l, o3, s) * (dm(s) * PIX(l, j, s, o2) * sg(l));
            hp += a; hm += b;
          }
        h2s[e] = hp + hm;
        h2d[e] = hp - hm;
      }
      tm.sync();
      double* Sm = sh.S();
      double* Dm = sh.D();
      for (int e = tm.lane; e < K * K; e += kTeam) {
        const int rr = e % K, cc = e / K, i = rr / 3, o1 = rr % 3, j = cc / 3, o2 = cc % 3;
        const double f = (-1.0 / qx[i]) * (0.5 * qw[j]);
        double dp = 0.0, dd = 0.0;
        for (int l = m; l <= NM; ++l)
          for (int s = 0; s < 3; ++s) {
            const double p = PIX(l, i, o1, s);
            const long hi_ = s + 3 * (l + NM1 * (o2 + 3 * j));
            dp += p * h2s[hi_];
            dd += p * h2d[hi_];
          }
        double sv = f * dp, dv = f * dd;
        if (rr == cc) { sv += 1.0 / qx[i]; dv += 1.0 / qx[i]; }
        Sm[rr + LD * cc] = sv;
        Dm[rr + LD * cc] = dv;
      }
      tm.sync();
      double* Hm = sh.H();
      for (int e = tm.lane; e < K * K; e += kTeam) {
        const int rr = e % K, cc = e / K;
        double s = 0.0;
        for (int k = 0; k < K; ++k) s += Dm[rr + LD * k] * Sm[k + LD * cc];
        Hm[rr + LD * cc] = s;
      }
      tm.sync();
      // eigen-decomposition (eigenvectors into D's storage)
      double* evals = LB + VecLayout<N>::kHm1;  // eigenvalues k^2; overwritten by HMULT below
      if (!team_eigen(tm, K, LD, Hm, sh.Z(), Dm, evals, sh.v, sh.red)) { st = RT_EIGEN_FAIL; break; }
      // solution vectors (lane per eigen-solution)
      int bad = 0;
      for (int k = tm.lane; k < K; k += kTeam) {
        const double lam = evals[k];
        if (!(lam > 0.0)) { bad = 1; continue; }
        const double kv = sqrt(lam), sc = 1.0 / kv;
        double nr = 0.0;
        for (int q = 0; q < K; ++q) nr += Dm[q + LD * k] * Dm[q + LD * k];
        nr = sqrt(nr);
        LB[VecLayout<N>::kTeig + k] = (kv * dtau > kMaxTau) ? 0.0 : exp(-kv * dtau);
        LB[VecLayout<N>::kGp + k] = kv;  // keep k until GBEAM below
        for (int i = 0; i < N; ++i)
          for (int s = 0; s < 3; ++s) {
            const int rr = 3 * i + s;
            const double sum = Dm[rr + LD * k] / nr;
            double h = 0.0;
            for (int q = 0; q < K; ++q) h += Sm[rr + LD * q] * (Dm[q + LD * k] / nr);
            const double dif = h * sc;
            const double fpd = 0.5 * (sum + dif), fnd = 0.5 * (sum - dif);
            XPc[rr + K2 * k] = fpd;
            XNc[rr + K2 * k] = fnd;
            XPc[(3 * (i + N) + s) + K2 * k] = s < 2 ? fnd : -fnd;
            XNc[(3 * (i + N) + s) + K2 * k] = s < 2 ? fpd : -fpd;
          }
      }
      if (team_any(tm, bad != 0, sh.ired)) { st = RT_EIGEN_FAIL; break; }
      tm.sync();
      // user-angle solutions, norms, multipliers, Green's function (lane per eigen-solution)
      const double udel = W[sl.tuser + n];
      const double secbar = W[sl.tavsec + n], cnst = W[sl.titrans + n], wdel = W[sl.tmubar + n];
      const bool active = (n < cutoff) && lsc;
      const double F1 = opt.flux_factor / kPI4;
      // hq(l, o1) = F1 sum_o2 og(l, o1, o2) PI0(l, o2, 0) (DFLUX = (1,0,0)), lanes over (l, o1)
      double* hq = ws + lay.h2s;  // h2s is free once SAB/DAB are formed
      for (int e = tm.lane; e < NM1 * 3; e += kTeam) {
        const int l = e % NM1, o1 = e / NM1;
        double g = 0.0;
        if (l >= m)
          for (int o2 = 0; o2 < 3; ++o2) g += og(l, o1, o2) * (PIX(l, N + 1, o2, 0) * 1.0);
        hq[e] = g;
      }
      tm.sync();
      // dpi, dmi (N x 3): lanes over (i, o1)
      double* dpi = ws + lay.h2d;
      double* dmi = dpi + 3 * N;
      for (int e = tm.lane; e < 3 * N; e += kTeam) {
        const int i = e % N, o1 = e / N;
        double sp = 0.0, sm_ = 0.0;
        for (int l = m; l <= NM; ++l)
          for (int s = 0; s < 3; ++s) {
            sp += PIX(l, i, o1, s) * hq[l + NM1 * s];
            sm_ += (PIX(l, i, o1, s) * dm(s) * sg(l)) * hq[l + NM1 * s];
          }
        dpi[e] = F1 * sp;
        dmi[e] = F1 * sm_;
      }
      tm.sync();
      for (int k = tm.lane; k < K; k += kTeam) {
        const double kv = LB[VecLayout<N>::kGp + k];
        const double zdel = LB[VecLayout<N>::kTeig + k];
        // UHOM: helpstokes(l, o1) = sum_j sum_s [PI(l,j,o1,s) a5 X+(j,s) + D_o1 PI sgn a5 X-(j,s)], gaux = og helps
        double uup[3] = {0.0, 0.0, 0.0}, udn[3] = {0.0, 0.0, 0.0};
        if (lsc)
          for (int l = m; l <= NM; ++l) {
            double hs[3];
            for (int o1 = 0; o1 < 3; ++o1) {
              double sps = 0.0;
              for (int j = 0; j < N; ++j) {
                const double a5 = 0.5 * qw[j];
                double sp = 0.0, sm_ = 0.0;
                for (int s = 0; s < 3; ++s) {
                  sp += PIX(l, j, o1, s) * a5 * XPc[(3 * j + s) + K2 * k];
                  sm_ += (dm(o1) * PIX(l, j, o1, s) * sg(l)) * a5 * XNc[(3 * j + s) + K2 * k];
                }
                sps = sps + sp + sm_;
              }
              hs[o1] = sps;
            }
            double ga[3];
            for (int o1 = 0; o1 < 3; ++o1) {
              double g = 0.0;
              for (int s = 0; s < 3; ++s) g += og(l, o1, s) * hs[s];
              ga[o1] = g;
            }
            for (int o1 = 0; o1 < 3; ++o1)
              for (int s = 0; s < 3; ++s) {
                const double pu = PIX(l, N, o1, s);
                udn[o1] += (dm(o1) * (pu * dm(s)) * sg(l)) * ga[s];  // PI_XUM
                uup[o1] += (dm(o1) * pu) * ga[s];                     // PI_XUP_PRE
              }
          }
        for (int o1 = 0; o1 < 3; ++o1) {
          LB[VecLayout<N>::kUdn + o1 * K + k] = udn[o1];
          LB[VecLayout<N>::kUup + o1 * K + k] = uup[o1];
        }
        // HMULT (vlidort_solutions.f90:1651)
        const double rho_p = sec_u + kv, rho_m = sec_u - kv;
        const double zp = 1.0 / rho_p;
        const bool hsing = fabs(rho_m) < kTaylorSmall;
        const double zm = hsing ? rho_m : 1.0 / rho_m;
        const double zudel = zdel * udel;
        const double hm1 = hsing ? taylor1<double>(opt.taylor_order, zm, dtau, udel, sec_u) : sec_u * (zdel - udel) * zm;
        const double hm2 = sec_u * (1.0 - zudel) * zp;
        // norm (QHOM_NORMS) and the Green's-function terms (GBEAM)
        double nrm = 0.0;
        for (int j = 0; j < N; ++j) {
          double t1 = 0.0, t2 = 0.0;
          for (int s = 0; s < 3; ++s) {
            t1 += XPc[(3 * j + s) + K2 * k] * XPc[(3 * j + s) + K2 * k];
            t2 += XNc[(3 * j + s) + K2 * k] * XNc[(3 * j + s) + K2 * k];
          }
          nrm += (qx[j] * qw[j]) * (t1 - t2);
        }
        double aterm = 0.0, bterm = 0.0, gp = 0.0, gm = 0.0, gdn = 0.0, gup = 0.0;
        if (active) {
          gp = secbar + kv;
          gm = secbar - kv;
          const double zwdel = zdel * wdel;
          const double cfunc = fabs(gm) < kTaylorSmall ? taylor1<double>(opt.taylor_order, gm, dtau, wdel, cnst)
                                                       : cnst * (zdel - wdel) / gm;
          const double dfunc = cnst * (1.0 - zwdel) / gp;
          double s1 = 0.0, s2_ = 0.0;
          for (int i = 0; i < N; ++i) {
            double h1 = 0.0, h2 = 0.0, h3 = 0.0, h4 = 0.0;
            for (int s = 0; s < 3; ++s) {
              h1 += dpi[i + N * s] * XPc[(3 * i + s) + K2 * k];
              h2 += dmi[i + N * s] * XNc[(3 * i + s) + K2 * k];
              h3 += dmi[i + N * s] * XPc[(3 * i + s) + K2 * k];
              h4 += dpi[i + N * s] * XNc[(3 * i + s) + K2 * k];
            }
            s1 += qw[i] * (h1 + h2);
            s2_ += qw[i] * (h3 + h4);
          }
          aterm = s1 / nrm;
          bterm = s2_ / nrm;
          gdn = cfunc * aterm;
          gup = dfunc * bterm;
        }
        LB[VecLayout<N>::kHm1 + k] = hm1;
        LB[VecLayout<N>::kHm2 + k] = hm2;
        LB[VecLayout<N>::kAt + k] = aterm;
        LB[VecLayout<N>::kBt + k] = bterm;
        LB[VecLayout<N>::kGp + k] = gp;
        LB[VecLayout<N>::kGm + k] = gm;
        sh.m[k] = gdn;  // staged for the particular solution below (S is free now)
        sh.m[K + k] = gup;
      }
      tm.sync();
      // particular integral at the layer boundaries WU (top), WL (bottom): lanes over (i, s) of 2N x 3
      for (int e = tm.lane; e < 3 * N; e += kTeam) {
        const int i = e / 3, s = e % 3;
        double wu1 = 0.0, wu2 = 0.0, wl1 = 0.0, wl2 = 0.0;
        if (active)
          for (int k = 0; k < K; ++k) {
            const double gdn = sh.m[k], gup = sh.m[K + k];
            wu1 += gup * XNc[(3 * i + s) + K2 * k]; wu2 += gup * XPc[(3 * i + s) + K2 * k];
            wl1 += gdn * XNc[(3 * i + s) + K2 * k]; wl2 += gdn * XPc[(3 * i + s) + K2 * k];
          }
        LB[VecLayout<N>::kWu + 3 * i + s] = wu1;
        LB[VecLayout<N>::kWu + 3 * (i + N) + s] = s >= 2 ? -wu2 : wu2;
        LB[VecLayout<N>::kWl + 3 * (i + N) + s] = s >= 2 ? -wl1 : wl1;
        LB[VecLayout<N>::kWl + 3 * i + s] = wl2;
      }
      tm.sync();
      // ------------------------------------------ Riccati step: top boundary (n = 0) or interface (n-1, n)
      double* M = sh.aug();
      constexpr int LR = VecShared<N>::LR;
      const double* T0 = LB + VecLayout<N>::kTeig;
      if (n == 0) {
        // A0 L0 = -T0 X-(top) M0 - W+(top):  rows (i < N, s), unknown L0 = F0 M0 + f0
        for (int rr = tm.lane; rr < K; rr += kTeam) {
          double* row = M + (long)rr * LR;
          for (int c = 0; c < K; ++c) {
            row[c] = XPc[rr + K2 * c];
            row[K + c] = -T0[c] * XNc[rr + K2 * c];
          }
          row[2 * K] = -LB[VecLayout<N>::kWu + rr];
        }
        tm.sync();
        if (!team_gauss(tm, K, K + 1, LR, M, sh.red, sh.ired)) { st = RT_BVP_SINGULAR; break; }
        for (int e = tm.lane; e < K * (K + 1); e += kTeam) {
          const int rr = e % K, c = e / K;
          if (c < K) LB[VecLayout<N>::kF + rr + (long)K * c] = M[(long)rr * LR + K + c];
          else LB[VecLayout<N>::kf + rr] = M[(long)rr * LR + 2 * K];
        }
        tm.sync();
      } else {
        const double* XPp = ws + lay.xp[pb];
        const double* XNp = ws + lay.xn[pb];
        const double* PB = ws + lay.lay0 + lay.lstride * (n - 1);
        const double* Tp = PB + VecLayout<N>::kTeig;
        const double* Fp = PB + VecLayout<N>::kF;
        const double* fp = PB + VecLayout<N>::kf;
        // [P F + Q | -R] [M_{n-1}; L_n] = [S | rhs - P f] with P = T_{n-1} X+_{n-1}, Q = X-_{n-1},
        // R = X+_n, S = T_n X-_n, rhs = W+_n(top) - W-_{n-1}(bottom)
        for (int rr = tm.lane; rr < K2; rr += kTeam) {
          double* row = M + (long)rr * LR;
          double pf_rhs = 0.0;
          for (int c = 0; c < K; ++c) {
            double s = 0.0;
            for (int k = 0; k < K; ++k) s += (Tp[k] * XPp[rr + K2 * k]) * Fp[k + (long)K * c];
            row[c] = s + XNp[rr + K2 * c];
            row[K + c] = -XPc[rr + K2 * c];
            row[2 * K + c] = T0[c] * XNc[rr + K2 * c];
          }
          for (int k = 0; k < K; ++k) pf_rhs += (Tp[k] * XPp[rr + K2 * k]) * fp[k];
          row[3 * K] = (LB[VecLayout<N>::kWu + rr] - PB[VecLayout<N>::kWl + rr]) - pf_rhs;
        }
        tm.sync();
        if (!team_gauss(tm, K2, K + 1, LR, M, sh.red, sh.ired)) { st = RT_BVP_SINGULAR; break; }
        double* PBw = ws + lay.lay0 + lay.lstride * (n - 1);
        for (int e = tm.lane; e < K2 * (K + 1); e += kTeam) {
          const int rr = e % K2, c = e / K2;
          const double val = M[(long)rr * LR + K2 + c];
          if (rr < K) {
            if (c < K) PBw[VecLayout<N>::kG + rr + (long)K * c] = val;
            else PBw[VecLayout<N>::kg + rr] = val;
          } else {
            if (c < K) LB[VecLayout<N>::kF + (rr - K) + (long)K * c] = val;
            else LB[VecLayout<N>::kf + (rr - K)] = val;
          }
        }
        tm.sync();
      }
    }
    if (st != RT_OK) break;
    // ------------------------------------------ bottom boundary, back substitution
    {
      const int nb = L - 1, cb = nb & 1;
      const double* XPl = ws + lay.xp[cb];
      const double* XNl = ws + lay.xn[cb];
      double* LB = ws + lay.lay0 + lay.lstride * nb;
      const double* Tl = LB + VecLayout<N>::kTeig;
      const double* Fl = LB + VecLayout<N>::kF;
      const double* fl = LB + VecLayout<N>::kf;
      double* M = sh.aug();
      constexpr int LR = VecShared<N>::LR;
      // Lambertian surface terms (BVP_SURFACE_SETUP_HOM / _BEAM): I row only
      double* r2p = M + (long)K * LR;  // rows K.. of the augmented storage are free here
      double* r2m = r2p + K;
      for (int k = tm.lane; k < K; k += kTeam) {
        double sp = 0.0, sm_ = 0.0;
        if (incl_surface)
          for (int j = 0; j < N; ++j) { sp += (qx[j] * qw[j]) * XPl[3 * j + K2 * k]; sm_ += (qx[j] * qw[j]) * XNl[3 * j + K2 * k]; }
        r2p[k] = sp * kmult;
        r2m[k] = sm_ * kmult;
      }
      double r2b = 0.0;
      if (incl_surface) {
        double part = 0.0;
        for (int j = tm.lane; j < N; j += kTeam) part += (qx[j] * qw[j]) * LB[VecLayout<N>::kWl + 3 * j];
        r2b = warp_sum(tm, part, sh.red) * kmult;
      }
      tm.sync();
      for (int rr = tm.lane; rr < K; rr += kTeam) {
        const int i = rr / 3, s = rr % 3, rl = 3 * (i + N) + s;
        double* row = M + (long)rr * LR;
        double pf_rhs = 0.0;
        for (int c = 0; c < K; ++c) {
          double acc = 0.0;
          for (int k = 0; k < K; ++k) {
            const double xpnet = XPl[rl + K2 * k] - (s == 0 ? r2p[k] : 0.0);
            acc += (Tl[k] * xpnet) * Fl[k + (long)K * c];
          }
          const double xmnet = XNl[rl + K2 * c] - (s == 0 ? r2m[c] : 0.0);
          row[c] = acc + xmnet;
        }
        for (int k = 0; k < K; ++k) {
          const double xpnet = XPl[rl + K2 * k] - (s == 0 ? r2p[k] : 0.0);
          pf_rhs += (Tl[k] * xpnet) * fl[k];
        }
        double rhs = -LB[VecLayout<N>::kWl + rl];
        if (s == 0 && incl_surface) rhs += r2b;
        if (s == 0 && localbeam) rhs += direct_beam;
        row[K] = rhs - pf_rhs;
      }
      tm.sync();
      if (!team_gauss(tm, K, 1, LR, M, sh.red, sh.ired)) { st = RT_BVP_SINGULAR; break; }
      for (int k = tm.lane; k < K; k += kTeam) LB[VecLayout<N>::kMc + k] = M[(long)k * LR + K];
      tm.sync();
      for (int nn = nb; nn >= 0; --nn) {
        double* B = ws + lay.lay0 + lay.lstride * nn;
        if (nn < nb) {
          const double* Bn = ws + lay.lay0 + lay.lstride * (nn + 1);
          for (int k = tm.lane; k < K; k += kTeam) {
            double s = B[VecLayout<N>::kg + k];
            for (int c = 0; c < K; ++c) s += B[VecLayout<N>::kG + k + (long)K * c] * Bn[VecLayout<N>::kMc + c];
            B[VecLayout<N>::kMc + k] = s;
          }
          tm.sync();
        }
        for (int k = tm.lane; k < K; k += kTeam) {
          double s = B[VecLayout<N>::kf + k];
          for (int c = 0; c < K; ++c) s += B[VecLayout<N>::kF + k + (long)K * c] * B[VecLayout<N>::kMc + c];
          B[VecLayout<N>::kLc + k] = s;
        }
        tm.sync();
      }
    }
    // ------------------------------------------ TOA upwelling source recursion (lanes over eigen-solutions)
    double sf[3] = {0.0, 0.0, 0.0};
    {
      double cum[3] = {0.0, 0.0, 0.0};
      const int nb = L - 1;
      const double* LB = ws + lay.lay0 + lay.lstride * nb;
      if (incl_surface) {  // GET_BOA_SOURCE (Lambertian: I only)
        const double* XPl = ws + lay.xp[nb & 1];
        const double* XNl = ws + lay.xn[nb & 1];
        double part = 0.0;
        for (int i = tm.lane; i < N; i += kTeam) {
          double shom = 0.0;
          for (int k = 0; k < K; ++k) {
            const double lxr = LB[VecLayout<N>::kLc + k] * XPl[3 * i + K2 * k];
            const double mxr = LB[VecLayout<N>::kMc + k] * XNl[3 * i + K2 * k];
            shom = shom + lxr * LB[VecLayout<N>::kTeig + k] + mxr;
          }
          part += (qx[i] * qw[i]) * (LB[VecLayout<N>::kWl + 3 * i] + shom);
        }
        cum[0] = kmult * warp_sum(tm, part, sh.red);
        if (!opt.do_focorr && localbeam) cum[0] += direct_beam;  // DO_INCLUDE_DIRECTRF without FO
      }
      for (int n = L - 1; n >= 0; --n) {
        const double* B = ws + lay.lay0 + lay.lstride * n;
        double src[3] = {0.0, 0.0, 0.0};
        if (laysc(m, n)) {
          const bool beam = n < cutoff;
          const double it = W[sl.titrans + n], wdel = W[sl.tmubar + n], itw = -it * wdel;
          const double em = W[sl.emult + n], tus = W[sl.tuser + n], avs = W[sl.tavsec + n];
          const double dtau = S[sl.dtau + n];
          double part[3] = {0.0, 0.0, 0.0};
          for (int k = tm.lane; k < K; k += kTeam) {
            const double hm1 = B[VecLayout<N>::kHm1 + k], hm2 = B[VecLayout<N>::kHm2 + k];
            const double lc = B[VecLayout<N>::kLc + k], mc = B[VecLayout<N>::kMc + k];
            double sd = 0.0, su = 0.0;
            if (beam) {
              const double gm = B[VecLayout<N>::kGm + k], gp = B[VecLayout<N>::kGp + k];
              if (fabs(gm) < kTaylorSmall) {
                const double mult = taylor2<double>(opt.taylor_order, gm, avs + sec_u, dtau, 1.0, wdel * tus, 1.0);
                sd = (it * sec_u) * mult;
              } else {
                sd = (it * hm2 - em) / gm;
              }
              su = (itw * hm1 + em) / gp;
            }
            const double at = B[VecLayout<N>::kAt + k], bt = B[VecLayout<N>::kBt + k];
            for (int o1 = 0; o1 < 3; ++o1) {
              const double ud = B[VecLayout<N>::kUdn + o1 * K + k], uu = B[VecLayout<N>::kUup + o1 * K + k];
              double v = lc * ud * hm2 + mc * uu * hm1;
              if (beam) v += ud * sd * at + uu * su * bt;
              part[o1] += v;
            }
          }
          for (int o1 = 0; o1 < 3; ++o1) src[o1] = warp_sum(tm, part[o1], sh.red);
        }
        const double tus = W[sl.tuser + n];
        for (int o1 = 0; o1 < 3; ++o1) cum[o1] = src[o1] + tus * cum[o1];
      }
      for (int o1 = 0; o1 < 3; ++o1) sf[o1] = delta_factor * cum[o1];
    }
    // ------------------------------------------ Fourier sum, intensity convergence test
    bool done = false;
    if (m == 0) {
      stokes[0] = sf[0]; stokes[1] = sf[1]; stokes[2] = sf[2];
      if (opt.do_focorr) { stokes[0] += r.ss + r.db; stokes[1] += ssq; stokes[2] += ssu; }
    } else {
      const double arg = raa * (double)m * kDTR;
      const double cz = cos(arg), sz = sin(arg);
      const double tazm0 = cz * sf[0];
      const double tnew0 = stokes[0] + tazm0;
      stokes[0] = tnew0;
      stokes[1] += cz * sf[1];
      stokes[2] += sz * sf[2];
      const bool conv = (tazm0 != 0.0) ? (fabs(tazm0 / tnew0) < opt.accuracy) : true;
      if (conv) {
        ++testconv;
        if (!opt.do_double_convtest || testconv == 2) done = true;
      } else {
        testconv = 0;
      }
    }
    if (done) break;
  }
  if (tm.lane == 0) {
    if (st != RT_OK) {
      radiance[o] = in.missing; reflectance[o] = in.missing; Qo[o] = in.missing; Uo[o] = in.missing;
      if (status) status[o] = st;
      if (nfourier) nfourier[o] = m;
    } else {
      int mm = m > r.n_fouriers ? r.n_fouriers : m;
      if (nfourier) nfourier[o] = mm;
      radiance[o] = stokes[0];
      Qo[o] = stokes[1];
      Uo[o] = stokes[2];
      reflectance[o] = (kPiSingle * stokes[0]) / (cos(r.sza * kPiSingle / 180.0) * opt.flux_factor);
    }
  }
  tm.sync();
}

}  // namespace aerort
