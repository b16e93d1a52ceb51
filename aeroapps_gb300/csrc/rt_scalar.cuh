// Scalar (NSTOKES=1) discrete-ordinate solar radiative transfer for one
// atmospheric column in one observation geometry, written for one CUDA thread
// per (column, wavelength) solve.
//
// Why one thread per solve: on GB300 the FP64 pipe issues at a small fraction
// of the FP32 rate, so the plain-FP64 solve is bound by FP64 instruction issue.
// Mapping one solve to one thread keeps every lane of every FP64 instruction
// busy (a warp works on 32 independent columns in lock-step) instead of
// leaving most lanes idle on 8x8 matrix work.  Layer-sized state lives in
// per-thread local memory (L1-cached); the per-layer factors that the
// boundary-value sweep needs on the way back up live in a global scratch
// buffer laid out element-major / thread-minor so that a warp's accesses to
// the same element are one coalesced transaction.
//
// The physics is the reference's VLIDORT 2.8.3 regular solar path as driven by
// AeroApps (paths relative to the reference project root):
//   src/Components/rtms/RTSI/VLIDORT2p8p3/VLIDORT_ScatMod.F90:975-1247  (layer mixing, output)
//   .../vlidort_main/regular/vlidort_geometry.f90:119-317              (Chapman factors)
//   .../vlidort_main/regular/vlidort_miscsetups.f90:370-1292,2273,3187 (delta-M, beam, PI functions)
//   .../vlidort_main/regular/vlidort_solutions.f90:150-3073            (homogeneous + Green's solutions)
//   .../vlidort_main/regular/vlidort_bvproblem.f90:147-2311            (boundary-value problem)
//   .../vlidort_main/regular/vlidort_intensity.f90:145, PostProcessing.f90:139 (TOA source recursion)
//   .../vlidort_main/regular/vlidort_converge.f90:825-1236             (Fourier convergence)
//   .../vlidort_focode/*.f90                                           (first-order single scatter)
// The numerical methods differ where GB300 favours another formulation (see
// layer_eigen and the block sweep in fourier_term in rt_solve.cuh); results
// agree with the reference algorithm to round-off.
#pragma once

#ifdef __CUDACC__
#define RT_HD __host__ __device__ __forceinline__
#define RT_HDN __host__ __device__
#else
#include <cmath>
#include <algorithm>
#define RT_HD inline
#define RT_HDN
using std::sqrt; using std::exp; using std::fabs; using std::asin; using std::sin; using std::cos;
using std::atan; using std::acos; using std::copysign; using std::expm1;
#endif

namespace aerort {

// VLIDORT parameters (vlidort_def/vlidort_pars.f90:386-444).  DEG_TO_RAD is the
// reference's truncated constant, kept so that angles map identically.
constexpr double kDTR = 1.7453292519943e-02;
constexpr double kPIE = 180.0 * kDTR;
constexpr double kPI4 = 4.0 * kPIE;
constexpr double kTaylorSmall = 1.0e-4;
constexpr double kMaxTau = 32.0;      // MAX_TAU_SPATH / UPATH / QPATH
constexpr double kFoCutoff = 88.0;    // FO_VectorSS_RTCalcs_I.f90:325
constexpr int kMaxFine = 4;           // MAXFINELAYERS
constexpr int kMaxLayers = 72;        // MAXLAYERS

// Per-solve status codes (0 = radiance valid).
enum RtStatus : int {
  RT_OK = 0,
  RT_EIGEN_FAIL = 1,      // layer eigenproblem: factorisation or QR iteration failed
  RT_BVP_SINGULAR = 2,    // zero pivot in the boundary-value sweep
  RT_BAD_INPUT = 3,       // inputs outside the solver's domain (e.g. tau_ext <= 0)
  RT_FO_FAIL = 4,         // single-scatter geometry failed
};

// Options shared by every solve of a batch (VLIDORT_Init settings).
struct RtOptions {
  int do_focorr;           // first-order single-scatter + direct-bounce correction
  int do_deltam;           // delta-M scaling
  int do_plane_parallel;   // plane-parallel beam attenuation
  int do_double_convtest;  // two consecutive converged Fourier terms end the series
  int nfine;               // fine layers of the enhanced-PS line-of-sight quadrature
  int taylor_order;        // Taylor series order near the exponential singularities
  double accuracy;         // Fourier convergence threshold
  double earth_radius;     // km
  double flux_factor;      // solar flux
  int max_fourier;         // -1: up to NMOMENTS (reference); otherwise cap (testing)
  int moment_contraction = 0;  // FP32 team solve: 0 CUDA-core FMA, 1 tensor cores (3xTF32 mma.sync)
};

// Strided per-thread view of a global scratch buffer (element e of this
// thread at base[e * stride]; stride = number of threads sharing the buffer).
template <typename T>
struct ScratchT {
  T* base;
  long stride;
  RT_HD T& operator[](long e) const { return base[e * stride]; }
};
using Scratch = ScratchT<double>;

// ---------------------------------------------------------------------------------- Taylor
// Series for (exp(-a d) - exp(-b d))/(b - a) near a == b (vlidort_Taylor.f90:101-219).
template <typename T>
RT_HD T taylor1(int order, T eps, T delta, T udel, T sm) {
  T d = 1.0, mult = 0.0, power = 1.0;
  for (int m = 1; m <= order + 1; ++m) {
    d = delta * d / (T)m;
    if (m == 1) mult = d;
    else { power *= eps; mult += power * d; }
  }
  return mult * udel * sm;
}

template <typename T>
RT_HD T taylor2(int order, T eps, T y, T delta, T fac1, T fac2, T sm) {
  T d[10];
  int mterms = order + 1;
  const bool small = fabs(y) < (T)kTaylorSmall;
  if (small) mterms += 1;
  d[0] = 1.0;
  for (int m = 1; m <= mterms; ++m) d[m] = delta * d[m - 1] / (T)m;
  if (small) {
    T power = 1.0, power2 = 1.0, mult = d[2];
    for (int m = 3; m <= mterms; ++m) {
      power = power * (eps - y);
      power2 = power - y * power2;
      mult += d[m] * power2;
    }
    return mult * fac1 * sm;
  }
  T y1 = (T)1.0 / y, ac[10];
  ac[0] = 1.0;
  for (int m = 1; m <= mterms; ++m) ac[m] = y1 * ac[m - 1];
  T mult = 0.0, power = 1.0;
  for (int m = 1; m <= mterms; ++m) {
    T cc = 0.0;
    for (int j = 0; j <= m; ++j) cc += ac[j] * d[m - j];
    T term = fac1 * ac[m] - fac2 * cc;
    if (m == 1) mult = term;
    else { power *= eps; mult += power * term; }
  }
  return mult * sm * y1;
}

// ---------------------------------------------------------------------------------- dense kernels
// Cholesky A = L L^T of an n x n SPD matrix (column-major, lower triangle
// overwritten with L).  Returns false if a pivot is not positive.
template <int NS, typename T>
RT_HD bool cholesky(int n, T* A) {
  for (int j = 0; j < n; ++j) {
    T s = A[j + NS * j];
    for (int k = 0; k < j; ++k) s -= A[j + NS * k] * A[j + NS * k];
    if (!(s > (T)0)) return false;
    T ljj = sqrt(s);
    A[j + NS * j] = ljj;
    T inv = (T)1.0 / ljj;
    for (int i = j + 1; i < n; ++i) {
      T t = A[i + NS * j];
      for (int k = 0; k < j; ++k) t -= A[i + NS * k] * A[j + NS * k];
      A[i + NS * j] = t * inv;
    }
  }
  return true;
}

// Unit roundoff of the working precision.
template <typename T> struct Eps;
template <> struct Eps<double> { static constexpr double v = 2.220446049250313e-16; };
template <> struct Eps<float> { static constexpr float v = 1.1920929e-07f; };

// A <- Q A Q for the reflector Q = I - beta v v^T (A symmetric, full storage,
// column-major with leading dimension NS).
template <int NS, typename T>
RT_HD void apply_reflector_sym(int n, T* A, const T* v, T beta) {
  // p = beta A v ; w = p - (beta/2)(p.v) v ; A -= v w^T + w v^T
  T p[NS], pv = 0;
  for (int i = 0; i < n; ++i) {
    T s = 0;
    for (int j = 0; j < n; ++j) s += A[i + NS * j] * v[j];
    p[i] = beta * s;
    pv += p[i] * v[i];
  }
  const T half = (T)0.5 * beta * pv;
  for (int i = 0; i < n; ++i) p[i] -= half * v[i];
  for (int j = 0; j < n; ++j)
    for (int i = 0; i < n; ++i) A[i + NS * j] -= v[i] * p[j] + p[i] * v[j];
}

// One-sided (Hestenes) Jacobi: orthogonalise the columns of the n x n matrix
// G (column-major, leading dimension NS) by plane rotations accumulated in V,
// until every pair of columns is orthogonal to working precision.  On return
// sigma[a] = |G e_a| (the singular values, with the relative accuracy of a
// column-graded G) and the columns of V are the right singular vectors, i.e.
// the eigenvectors of G^T G.  Returns false if the sweep budget is exhausted.
// 1/sqrt(x), correctly rounded in FP32 on the device (the approximate
// hardware rsqrtf lets cs^2 + sn^2 drift from 1 by a few ulp per rotation,
// which the hundreds of rotations of one eigen-solve accumulate).
template <typename T>
RT_HD T rsqrt_t(T x) {
#ifdef __CUDA_ARCH__
  if constexpr (sizeof(T) == sizeof(float)) return __frsqrt_rn(x);
  else return rsqrt(x);
#else
  return (T)1 / sqrt(x);
#endif
}

// One Hestenes-Jacobi rotation of column pair (p, q) with squared norms al, be
// and inner product ga.  Rotate when ga^2 > tol^2 al be (the pair is not yet
// orthogonal to tol); the return value says whether ga^2 > tol al be (the
// sweep does not count as the converged one).  tan(theta) comes from one
// square root and one division, t = sign(d) 2 ga / (|d| + sqrt(d^2 + 4 ga^2))
// with d = be - al (the smaller root of t^2 + 2 t d / (2 ga) - 1 = 0), and
// cos(theta) from a reciprocal square root.
template <typename T>
struct Rotation {
  T cs, sn;
  bool rotate, unconverged;
  RT_HD Rotation(T al, T be, T ga, T tol) {
    const T ab = al * be, g2 = ga * ga;
    rotate = g2 > tol * tol * ab;
    unconverged = g2 > tol * ab;
    cs = (T)1;
    sn = (T)0;
    if (rotate) {
      const T d = be - al, two_ga = (T)2 * ga;
      const T t = (d < (T)0 ? -two_ga : two_ga) / (fabs(d) + sqrt(d * d + two_ga * two_ga));
      cs = rsqrt_t((T)1 + t * t);
      sn = cs * t;
    }
  }
};

template <int NS, typename T>
RT_HD bool jacobi_svd(int n, T* G, T* V, T* sigma) {
  for (int j = 0; j < n; ++j)
    for (int i = 0; i < n; ++i) V[i + NS * j] = (i == j) ? (T)1 : (T)0;
  const T tol = Eps<T>::v * (T)n;
  bool done = false;
  for (int sweep = 0; sweep < 30 && !done; ++sweep) {
    // converged when no pair rotated, or when every normalised off-diagonal
    // of this sweep, |ga| / sqrt(al be), was below sqrt(tol): Jacobi converges
    // quadratically, so the sweep that follows would not rotate
    bool unconverged = false;
    for (int p = 0; p + 1 < n; ++p)
      for (int q = p + 1; q < n; ++q) {
        T al = 0, be = 0, ga = 0;
        for (int i = 0; i < n; ++i) {
          const T gp = G[i + NS * p], gq = G[i + NS * q];
          al += gp * gp; be += gq * gq; ga += gp * gq;
        }
        const Rotation<T> rot(al, be, ga, tol);
        if (!rot.rotate) continue;
        unconverged = unconverged || rot.unconverged;
        const T cs = rot.cs, sn = rot.sn;
        for (int i = 0; i < n; ++i) {
          const T gp = G[i + NS * p], gq = G[i + NS * q];
          G[i + NS * p] = cs * gp - sn * gq;
          G[i + NS * q] = sn * gp + cs * gq;
          const T vp = V[i + NS * p], vq = V[i + NS * q];
          V[i + NS * p] = cs * vp - sn * vq;
          V[i + NS * q] = sn * vp + cs * vq;
        }
      }
    done = !unconverged;
  }
  for (int a = 0; a < n; ++a) {
    T s = 0;
    for (int i = 0; i < n; ++i) s += G[i + NS * a] * G[i + NS * a];
    sigma[a] = sqrt(s);
  }
  return done;
}

// In-place LU with partial pivoting of an n x n matrix (leading dimension LD)
// and solution of nrhs right-hand sides B (n x nrhs, leading dimension LD).
template <int LD, typename T>
RT_HD bool lu_solve(int n, T* A, T* B, int nrhs) {
  for (int k = 0; k < n; ++k) {
    int piv = k;
    T amax = fabs(A[k + LD * k]);
    for (int i = k + 1; i < n; ++i) {
      T a = fabs(A[i + LD * k]);
      if (a > amax) { amax = a; piv = i; }
    }
    if (amax == (T)0) return false;
    if (piv != k) {
      for (int j = 0; j < n; ++j) { T t = A[k + LD * j]; A[k + LD * j] = A[piv + LD * j]; A[piv + LD * j] = t; }
      for (int j = 0; j < nrhs; ++j) { T t = B[k + LD * j]; B[k + LD * j] = B[piv + LD * j]; B[piv + LD * j] = t; }
    }
    T inv = (T)1.0 / A[k + LD * k];
    for (int i = k + 1; i < n; ++i) {
      T f = A[i + LD * k] * inv;
      A[i + LD * k] = f;
      for (int j = k + 1; j < n; ++j) A[i + LD * j] -= f * A[k + LD * j];
      for (int j = 0; j < nrhs; ++j) B[i + LD * j] -= f * B[k + LD * j];
    }
  }
  for (int j = 0; j < nrhs; ++j)
    for (int i = n - 1; i >= 0; --i) {
      T s = B[i + LD * j];
      for (int k = i + 1; k < n; ++k) s -= A[i + LD * k] * B[k + LD * j];
      B[i + LD * j] = s / A[i + LD * i];
    }
  return true;
}

}  // namespace aerort
