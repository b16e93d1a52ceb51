// Test infrastructure only: the CPU oracle for the scalar VLIDORT 2.8.3 solar path.
//
// This file restates, routine by routine and in FP64, the reference's forward
// model for one atmospheric column seen in one solar geometry (observation
// geometry, or a single-SZA lattice of user zenith/azimuth angles), Lambertian
// surface, pseudo-spherical beam, Green's-function particular integral, TOA
// upwelling output, first-order (FO) single-scatter + direct-bounce correction.
// It is the checker for the CUDA kernels and the CPU baseline of bench.py; no
// product code links it.  Paths are relative to the reference project root
// (src/Components/rtms/RTSI/VLIDORT2p8p3/...).
//
// Parity pin: tests/test_oracle_golden.py compares this oracle with the
// reference's own saved gfortran results (vlidort_s_test/saved_results/
// gfortran/results_solar_tester.all).
#include <cmath>
#include <cstring>
#include <vector>
#include <algorithm>

#include <omp.h>

#include "vlidort_oracle.h"

namespace orc {

typedef std::vector<double> dvec;

// vlidort_aux.f90:960-1042 GETQUAD2 (Gauss-Legendre on [A,B] by Newton on P_N).
// Also vlidort_focode/FO_geometry_Generic.f90:331 (same algorithm).
void getquad2(double a, double b, int n, double* roots, double* wgts) {
  const double QEPS = 1.0e-13;
  int n2 = (n + 1) / 2;
  double nr = (double)n, midpt = 0.5 * (b + a), sfac = 0.5 * (b - a);
  for (int m = 1; m <= n2; ++m) {
    double mr = (double)m;
    double xx = PIE * (mr - 0.25) / (nr + 0.5);
    double x = (1.0 - (nr - 1.0) / (8.0 * nr * nr * nr) -
                1.0 / (384.0 * nr * nr * nr * nr) * (39.0 - 28.0 / (std::sin(xx) * std::sin(xx)))) *
               std::cos(xx);
    double lp = 1.0, lpm1 = 0.0, dlp = 0.0;
    for (int it = 0; it < 100; ++it) {
      lpm1 = 0.0; lp = 1.0;
      for (int i = 1; i <= n; ++i) {
        double ir = (double)i, lpm2 = lpm1;
        lpm1 = lp;
        lp = ((2.0 * ir - 1.0) * x * lpm1 - (ir - 1.0) * lpm2) / ir;
      }
      dlp = nr * (x * lp - lpm1) / (x * x - 1.0);
      double xold = x;
      x = xold - lp / dlp;
      if (std::fabs(x - xold) <= QEPS) break;
    }
    roots[m - 1] = midpt - sfac * x;
    wgts[m - 1] = (2.0 * sfac) / ((1.0 - x * x) * dlp * dlp);
    roots[n - m] = midpt + sfac * x;
    wgts[n - m] = wgts[m - 1];
  }
}

// vlidort_Taylor.f90 Taylor_series_1 / Taylor_Series_2
double taylor1(int order, double eps, double delta, double udel, double sm) {
  double d[16];
  int mterms = order + 1;
  d[0] = 1.0;
  for (int m = 1; m <= mterms; ++m) d[m] = delta * d[m - 1] / (double)m;
  double mult = d[1], power = 1.0;
  for (int m = 2; m <= mterms; ++m) { power *= eps; mult += power * d[m]; }
  return mult * udel * sm;
}

double taylor2(int order, double eps, double y, double delta, double fac1, double fac2, double sm) {
  double d[16], ac[16], cc[16], term1[16];
  int mterms = order + 1;
  if (std::fabs(y) < TAYLOR_SMALL) mterms += 1;
  d[0] = 1.0;
  for (int m = 1; m <= mterms; ++m) d[m] = delta * d[m - 1] / (double)m;
  if (std::fabs(y) < TAYLOR_SMALL) {
    double power = 1.0, power2 = 1.0, mult = d[2];
    for (int m = 3; m <= mterms; ++m) {
      power = power * (eps - y);
      power2 = power - y * power2;
      mult += d[m] * power2;
    }
    return mult * fac1 * sm;
  }
  double y1 = 1.0 / y;
  ac[0] = 1.0;
  for (int m = 1; m <= mterms; ++m) ac[m] = y1 * ac[m - 1];
  cc[0] = 1.0;
  for (int m = 1; m <= mterms; ++m) {
    cc[m] = 0.0;
    for (int j = 0; j <= m; ++j) cc[m] += ac[j] * d[m - j];
  }
  for (int m = 0; m <= mterms; ++m) term1[m] = fac1 * ac[m] - fac2 * cc[m];
  double power = 1.0, mult = term1[1];
  for (int m = 2; m <= mterms; ++m) { power = eps * power; mult += power * term1[m]; }
  return mult * sm * y1;
}

// vlidort_aux.f90:386-956 ASYMTX: eigenvalues/vectors of a real nonsymmetric
// matrix known to have real eigenvalues (balancing, Householder reduction to
// upper Hessenberg, shifted double-step QR, back substitution; EISPACK lineage
// as used in DISORT).  Column-major, 1-based accessors.  Returns ier (0 = ok,
// >0 = eigenvalue ier did not converge in 30 iterations), bad=true on input
// errors.
int asymtx(double tol, double* aad, int m, int ia, double* evecd, double* evald, double* wkd,
           bool* bad) {
#define A(i, j) aad[((i)-1) + ((j)-1) * ia]
#define E(i, j) evecd[((i)-1) + ((j)-1) * ia]
#define W(i) wkd[(i)-1]
#define EV(i) evald[(i)-1]
  const double C1 = 0.4375, C2 = 0.5, C3 = 0.75, C4 = 0.95, C5 = 16.0, C6 = 256.0;
  int ier = 0;
  *bad = false;
  if (m < 1 || ia < m) { *bad = true; return 0; }
  if (m == 1) { EV(1) = A(1, 1); E(1, 1) = 1.0; return 0; }
  if (m == 2) {
    double discri = (A(1, 1) - A(2, 2)) * (A(1, 1) - A(2, 2)) + 4.0 * A(1, 2) * A(2, 1);
    if (discri < 0.0) { *bad = true; return 0; }
    double sgn = 1.0;
    if (A(1, 1) < A(2, 2)) sgn = -1.0;
    EV(1) = 0.5 * (A(1, 1) + A(2, 2) + sgn * std::sqrt(discri));
    EV(2) = 0.5 * (A(1, 1) + A(2, 2) - sgn * std::sqrt(discri));
    E(1, 1) = 1.0; E(2, 2) = 1.0;
    if (A(1, 1) == A(2, 2) && (A(2, 1) == 0.0 || A(1, 2) == 0.0)) {
      double rnorm = std::fabs(A(1, 1)) + std::fabs(A(1, 2)) + std::fabs(A(2, 1)) + std::fabs(A(2, 2));
      double w = tol * rnorm;
      E(2, 1) = A(2, 1) / w;
      E(1, 2) = -A(1, 2) / w;
    } else {
      E(2, 1) = A(2, 1) / (EV(1) - A(2, 2));
      E(1, 2) = A(1, 2) / (EV(2) - A(1, 1));
    }
    return 0;
  }
  for (int i = 1; i <= m; ++i) {
    EV(i) = 0.0;
    for (int j = 1; j <= m; ++j) E(i, j) = 0.0;
    E(i, i) = 1.0;
  }
  double rnorm = 0.0;
  int l = 1, k = m;
  // search for rows isolating an eigenvalue and push them down
L30:
  for (int j = k; j >= 1; --j) {
    double row = 0.0;
    for (int i = 1; i <= k; ++i)
      if (i != j) row += std::fabs(A(j, i));
    if (row == 0.0) {
      W(k) = j;
      if (j != k) {
        for (int i = 1; i <= k; ++i) std::swap(A(i, j), A(i, k));
        for (int i = l; i <= m; ++i) std::swap(A(j, i), A(k, i));
      }
      k = k - 1;
      goto L30;
    }
  }
  // search for columns isolating an eigenvalue and push them left
L80:
  for (int j = l; j <= k; ++j) {
    double col = 0.0;
    for (int i = l; i <= k; ++i)
      if (i != j) col += std::fabs(A(i, j));
    if (col == 0.0) {
      W(l) = j;
      if (j != l) {
        for (int i = 1; i <= k; ++i) std::swap(A(i, j), A(i, l));
        for (int i = l; i <= m; ++i) std::swap(A(j, i), A(l, i));
      }
      l = l + 1;
      goto L80;
    }
  }
  // balance the submatrix in rows l through k
  for (int i = l; i <= k; ++i) W(i) = 1.0;
  {
    bool noconv;
    do {
      noconv = false;
      for (int i = l; i <= k; ++i) {
        double col = 0.0, row = 0.0;
        for (int j = l; j <= k; ++j)
          if (j != i) { col += std::fabs(A(j, i)); row += std::fabs(A(i, j)); }
        double f = 1.0, g = row / C5, h = col + row;
        while (col < g) { f *= C5; col *= C6; }
        g = row * C5;
        while (col >= g) { f /= C5; col /= C6; }
        if ((col + row) / f < C4 * h) {
          W(i) = W(i) * f;
          noconv = true;
          for (int j = l; j <= m; ++j) A(i, j) = A(i, j) / f;
          for (int j = 1; j <= k; ++j) A(j, i) = A(j, i) * f;
        }
      }
    } while (noconv);
  }
  if (k - 1 >= l + 1) {
    // Householder reduction to upper Hessenberg form
    for (int n = l + 1; n <= k - 1; ++n) {
      double h = 0.0, scale = 0.0;
      W(n + m) = 0.0;
      for (int i = n; i <= k; ++i) scale += std::fabs(A(i, n - 1));
      if (scale != 0.0) {
        for (int i = k; i >= n; --i) { W(i + m) = A(i, n - 1) / scale; h += W(i + m) * W(i + m); }
        double g = -std::copysign(std::sqrt(h), W(n + m));
        h = h - W(n + m) * g;
        W(n + m) = W(n + m) - g;
        for (int j = n; j <= m; ++j) {
          double f = 0.0;
          for (int i = k; i >= n; --i) f += W(i + m) * A(i, j);
          for (int i = n; i <= k; ++i) A(i, j) = A(i, j) - W(i + m) * f / h;
        }
        for (int i = 1; i <= k; ++i) {
          double f = 0.0;
          for (int j = k; j >= n; --j) f += W(j + m) * A(i, j);
          for (int j = n; j <= k; ++j) A(i, j) = A(i, j) - W(j + m) * f / h;
        }
        W(n + m) = scale * W(n + m);
        A(n, n - 1) = scale * g;
      }
    }
    // accumulate the transformations
    for (int n = k - 2; n >= l; --n) {
      int n1 = n + 1, n2 = n + 2;
      double f = A(n1, n);
      if (f != 0.0) {
        f = f * W(n1 + m);
        for (int i = n2; i <= k; ++i) W(i + m) = A(i, n);
        if (n1 <= k) {
          for (int j = 1; j <= m; ++j) {
            double g = 0.0;
            for (int i = n1; i <= k; ++i) g += W(i + m) * E(i, j);
            g = g / f;
            for (int i = n1; i <= k; ++i) E(i, j) = E(i, j) + g * W(i + m);
          }
        }
      }
    }
  }
  {
    int n = 1;
    for (int i = 1; i <= m; ++i) {
      for (int j = n; j <= m; ++j) rnorm += std::fabs(A(i, j));
      n = i;
      if (i < l || i > k) EV(i) = A(i, i);
    }
  }
  {
    int n = k;
    double t = 0.0;
    double p = 0, q = 0, r = 0, s = 0, w = 0, x = 0, y = 0, z = 0;
    while (n >= l) {
      int in = 0, n1 = n - 1, n2 = n - 2;
      for (;;) {
        int lb = l;
        for (int i = l; i <= n; ++i) {
          lb = n + l - i;
          if (lb == l) break;
          s = std::fabs(A(lb - 1, lb - 1)) + std::fabs(A(lb, lb));
          if (s == 0.0) s = rnorm;
          if (std::fabs(A(lb, lb - 1)) <= tol * s) break;
        }
        x = A(n, n);
        if (lb == n) {  // one eigenvalue found
          A(n, n) = x + t;
          EV(n) = A(n, n);
          n = n1;
          break;
        }
        y = A(n1, n1);
        w = A(n, n1) * A(n1, n);
        if (lb == n1) {  // two eigenvalues found
          p = (y - x) * C2;
          q = p * p + w;
          z = std::sqrt(std::fabs(q));
          A(n, n) = x + t;
          x = A(n, n);
          A(n1, n1) = y + t;
          z = p + std::copysign(z, p);
          EV(n1) = x + z;
          EV(n) = EV(n1);
          if (z != 0.0) EV(n) = x - w / z;
          x = A(n, n1);
          r = std::sqrt(x * x + z * z);
          p = x / r;
          q = z / r;
          for (int j = n1; j <= m; ++j) {
            z = A(n1, j);
            A(n1, j) = q * z + p * A(n, j);
            A(n, j) = q * A(n, j) - p * z;
          }
          for (int i = 1; i <= n; ++i) {
            z = A(i, n1);
            A(i, n1) = q * z + p * A(i, n);
            A(i, n) = q * A(i, n) - p * z;
          }
          for (int i = l; i <= k; ++i) {
            z = E(i, n1);
            E(i, n1) = q * z + p * E(i, n);
            E(i, n) = q * E(i, n) - p * z;
          }
          n = n2;
          break;
        }
        if (in == 30) { ier = n; goto L670; }
        if (in == 10 || in == 20) {  // exceptional shift
          t = t + x;
          for (int i = l; i <= n; ++i) A(i, i) = A(i, i) - x;
          s = std::fabs(A(n, n1)) + std::fabs(A(n1, n2));
          x = C3 * s;
          y = x;
          w = -C1 * s * s;
        }
        in = in + 1;
        int i = lb;
        for (int j = lb; j <= n2; ++j) {  // look for two consecutive small sub-diagonal elements
          i = n2 + lb - j;
          z = A(i, i);
          r = x - z;
          s = y - z;
          p = (r * s - w) / A(i + 1, i) + A(i, i + 1);
          q = A(i + 1, i + 1) - z - r - s;
          r = A(i + 2, i + 1);
          s = std::fabs(p) + std::fabs(q) + std::fabs(r);
          p = p / s; q = q / s; r = r / s;
          if (i == lb) break;
          double uu = std::fabs(A(i, i - 1)) * (std::fabs(q) + std::fabs(r));
          double vv = std::fabs(p) * (std::fabs(A(i - 1, i - 1)) + std::fabs(z) + std::fabs(A(i + 1, i + 1)));
          if (uu <= tol * vv) break;
        }
        A(i + 2, i) = 0.0;
        for (int j = i + 3; j <= n; ++j) { A(j, j - 2) = 0.0; A(j, j - 3) = 0.0; }
        for (int ka = i; ka <= n1; ++ka) {  // double QR step
          bool notlas = ka != n1;
          if (ka == i) {
            s = std::copysign(std::sqrt(p * p + q * q + r * r), p);
            if (lb != i) A(ka, ka - 1) = -A(ka, ka - 1);
          } else {
            p = A(ka, ka - 1);
            q = A(ka + 1, ka - 1);
            r = 0.0;
            if (notlas) r = A(ka + 2, ka - 1);
            x = std::fabs(p) + std::fabs(q) + std::fabs(r);
            if (x == 0.0) continue;
            p = p / x; q = q / x; r = r / x;
            s = std::copysign(std::sqrt(p * p + q * q + r * r), p);
            A(ka, ka - 1) = -s * x;
          }
          p = p + s;
          x = p / s; y = q / s; z = r / s;
          q = q / p; r = r / p;
          for (int j = ka; j <= m; ++j) {  // row modification
            p = A(ka, j) + q * A(ka + 1, j);
            if (notlas) { p = p + r * A(ka + 2, j); A(ka + 2, j) = A(ka + 2, j) - p * z; }
            A(ka + 1, j) = A(ka + 1, j) - p * y;
            A(ka, j) = A(ka, j) - p * x;
          }
          int iimax = std::min(n, ka + 3);
          for (int ii = 1; ii <= iimax; ++ii) {  // column modification
            p = x * A(ii, ka) + y * A(ii, ka + 1);
            if (notlas) { p = p + z * A(ii, ka + 2); A(ii, ka + 2) = A(ii, ka + 2) - p * r; }
            A(ii, ka + 1) = A(ii, ka + 1) - p * q;
            A(ii, ka) = A(ii, ka) - p;
          }
          for (int ii = l; ii <= k; ++ii) {  // accumulate transformations
            p = x * E(ii, ka) + y * E(ii, ka + 1);
            if (notlas) { p = p + z * E(ii, ka + 2); E(ii, ka + 2) = E(ii, ka + 2) - p * r; }
            E(ii, ka + 1) = E(ii, ka + 1) - p * q;
            E(ii, ka) = E(ii, ka) - p;
          }
        }
      }
    }
  }
  // back substitution for the eigenvectors of the triangular form
  if (rnorm != 0.0) {
    for (int n = m; n >= 1; --n) {
      int n2 = n;
      A(n, n) = 1.0;
      for (int i = n - 1; i >= 1; --i) {
        double w = A(i, i) - EV(n);
        if (w == 0.0) w = tol * rnorm;
        double r = A(i, n);
        for (int j = n2; j <= n - 1; ++j) r += A(i, j) * A(j, n);
        A(i, n) = -r / w;
        n2 = i;
      }
    }
    for (int i = 1; i <= m; ++i)
      if (i < l || i > k)
        for (int j = i; j <= m; ++j) E(i, j) = A(i, j);
    if (k != 0) {
      for (int j = m; j >= l; --j)
        for (int i = l; i <= k; ++i) {
          double z = 0.0;
          for (int n = l; n <= std::min(j, k); ++n) z += E(i, n) * A(n, j);
          E(i, j) = z;
        }
    }
  }
  for (int i = l; i <= k; ++i)
    for (int j = 1; j <= m; ++j) E(i, j) = E(i, j) * W(i);
  for (int i = l - 1; i >= 1; --i) {
    int j = (int)W(i);
    if (i != j)
      for (int n = 1; n <= m; ++n) std::swap(E(i, n), E(j, n));
  }
  for (int i = k + 1; i <= m; ++i) {
    int j = (int)W(i);
    if (i != j)
      for (int n = 1; n <= m; ++n) std::swap(E(i, n), E(j, n));
  }
L670:
  return ier;
#undef A
#undef E
#undef W
#undef EV
}

// Banded LU with partial pivoting (LAPACK DGBTF2/DGBTRS semantics; the
// reference calls DGBTRF/DGBTRS from lapack_tools.f90:6683, 7354 inside
// vlidort_bvproblem.f90:1235 and BVP_BACKSUB).  ab is (2kl+ku+1) x n column
// major, entry A(i,j) stored at ab[kl+ku+i-j + ldab*j] (0-based).
int band_lu(int n, int kl, int ku, double* ab, int ldab, int* ipiv) {
  int kv = ku + kl;
  for (int j = ku + 2; j <= std::min(kv, n); ++j)  // zero the fill-in triangle
    for (int i = kv - j + 2; i <= kl; ++i) ab[(i - 1) + ldab * (j - 1)] = 0.0;
  int ju = 1, info = 0;
  for (int j = 1; j <= n; ++j) {
    if (j + kv <= n)
      for (int i = 1; i <= kl; ++i) ab[(i - 1) + ldab * (j + kv - 1)] = 0.0;
    int km = std::min(kl, n - j);
    int jp = 1;
    double amax = std::fabs(ab[kv + ldab * (j - 1)]);
    for (int i = 2; i <= km + 1; ++i) {
      double v = std::fabs(ab[kv + i - 1 + ldab * (j - 1)]);
      if (v > amax) { amax = v; jp = i; }
    }
    ipiv[j - 1] = jp + j - 1;
    if (ab[kv + jp - 1 + ldab * (j - 1)] != 0.0) {
      ju = std::max(ju, std::min(j + ku + jp - 1, n));
      if (jp != 1) {
        for (int c = 0; c < ju - j + 1; ++c)
          std::swap(ab[kv + jp - 1 - c + ldab * (j - 1 + c)], ab[kv - c + ldab * (j - 1 + c)]);
      }
      if (km > 0) {
        double rp = 1.0 / ab[kv + ldab * (j - 1)];
        for (int i = 1; i <= km; ++i) ab[kv + i + ldab * (j - 1)] *= rp;
        if (ju > j) {
          for (int c = 1; c <= ju - j; ++c) {
            double y = ab[kv - c + ldab * (j - 1 + c)];
            if (y != 0.0)
              for (int i = 1; i <= km; ++i)
                ab[kv - c + i + ldab * (j - 1 + c)] -= ab[kv + i + ldab * (j - 1)] * y;
          }
        }
      }
    } else if (info == 0) {
      info = j;
    }
  }
  return info;
}

void band_solve(int n, int kl, int ku, const double* ab, int ldab, const int* ipiv, double* b) {
  int kd = ku + kl + 1;
  for (int j = 1; j <= n - 1; ++j) {
    int lm = std::min(kl, n - j);
    int l = ipiv[j - 1];
    if (l != j) std::swap(b[l - 1], b[j - 1]);
    for (int i = 1; i <= lm; ++i) b[j + i - 1] -= ab[kd + i - 1 + ldab * (j - 1)] * b[j - 1];
  }
  for (int j = n; j >= 1; --j) {  // upper triangular, bandwidth kl+ku
    b[j - 1] /= ab[kd - 1 + ldab * (j - 1)];
    double t = b[j - 1];
    int lm = std::min(j - 1, kl + ku);
    for (int i = 1; i <= lm; ++i) b[j - 1 - i] -= ab[kd - 1 - i + ldab * (j - 1)] * t;
  }
}

void fo_geometry(const OracleOpts* o, int L, const double* heights, const std::vector<double>& radii,
                 const std::vector<double>& ext, const std::vector<double>& dts, double sza, double vza,
                 double raa, FoGeom& G) {
  bool enhanced = !o->do_plane_parallel && !o->do_focorr_nadir && o->do_focorr_outgoing;
  const int nf = o->nfinelayers;
  std::vector<double> tf(nf > 0 ? nf : 1), af(nf > 0 ? nf : 1);
  const double vsign = 1.0;
  double alpha_boa = vza, theta_boa = sza, phi_boa = raa;
  if (phi_boa < 0.0) phi_boa = -phi_boa;
  if (phi_boa > 360.0) phi_boa = 360.0 - phi_boa - 360.0;
  bool overhead = (theta_boa == 0.0);
  double theta_boa_R = theta_boa * DTR, ctheta_boa, stheta_boa;
  if (theta_boa == 90.0) { ctheta_boa = 0.0; stheta_boa = 1.0; }
  else { stheta_boa = std::sin(theta_boa_R); ctheta_boa = std::cos(theta_boa_R); }
  double phi_boa_R = phi_boa * DTR, cphi = std::cos(phi_boa_R), sphi = std::sin(phi_boa_R);
  std::vector<double> atten(L + 1, 0.0), suntau(L + 1, 0.0), lostrans(L, 0.0), mult(L, 0.0);
  double mu0, mu1, cosscat;
  // findsunpaths_D: paths through layers 1..nn of a ray leaving radius radstart
  auto sunpaths_D = [&](bool zero_sun_boa, double radstart, double thstart, double sthstart, int nn,
                        double* sp) {
    int n1 = nn - 1;
    if (zero_sun_boa) {
      sp[nn] = radii[n1] - radstart;
      for (int k = n1; k >= 1; --k) sp[k] = radii[k - 1] - radii[k];
      return;
    }
    double sth0 = sthstart, th0 = thstart;
    double sth1 = sth0 * radstart / radii[n1], th1 = std::asin(sth1), ks1 = th0 - th1;
    sp[nn] = std::sin(ks1) * radstart / sth1;
    sth0 = sth1; th0 = th1;
    for (int k = n1; k >= 1; --k) {
      sth1 = sth0 * radii[k] / radii[k - 1];
      th1 = std::asin(sth1);
      ks1 = th0 - th1;
      sp[k] = std::sin(ks1) * radii[k] / sth1;
      sth0 = sth1; th0 = th1;
    }
  };
  // findsunpaths_T: tangent-point paths (sun below the local horizon)
  auto sunpaths_T = [&](double radstart, double thstart, double sthstart, int nn, double* sp) -> int {
    int n1 = nn - 1, nt = nn;
    double tanr = sthstart * radstart;
    int k = n1;
    bool trawl = true;
    while (k >= n1 && trawl && k <= L) { trawl = (radii[k] > tanr); k = k + 1; }
    nt = k - 1;
    if (nt > nn) {
      double th0 = PIE - thstart, sth0 = sthstart;
      double sth1 = sth0 * radstart / radii[nn], th1 = std::asin(sth1), ks1 = th0 - th1;
      sp[nn] = 2.0 * std::sin(ks1) * radstart / sth1;
      sth0 = sth1; th0 = th1;
      for (int kk = nn + 1; kk <= nt - 1; ++kk) {
        sth1 = sth0 * radii[kk - 1] / radii[kk];
        th1 = std::asin(sth1); ks1 = th0 - th1;
        sp[kk] = 2.0 * std::sin(ks1) * radii[kk] / sth0;
        sth0 = sth1; th0 = th1;
      }
      ks1 = 0.5 * PIE - th0;
      sp[nt] = 2.0 * std::sin(ks1) * radii[nt - 1];
    } else if (nt == nn) {
      sp[nn] = -2.0 * radstart * std::cos(thstart);
    }
    double th0 = PIE - thstart, sth0 = sthstart;
    double sth1 = sth0 * radstart / radii[n1], th1 = std::asin(sth1), ks1 = th0 - th1;
    sp[nn] = sp[nn] + std::sin(ks1) * radstart / sth1;
    sth0 = sth1; th0 = th1;
    for (int kk = n1; kk >= 1; --kk) {
      sth1 = sth0 * radii[kk] / radii[kk - 1];
      th1 = std::asin(sth1); ks1 = th0 - th1;
      sp[kk] = std::sin(ks1) * radii[kk] / sth1;
      sth0 = sth1; th0 = th1;
    }
    return nt;
  };
  std::vector<double> sp(L + 2, 0.0);
  auto path_tau = [&](int nt) {
    double s = 0.0;
    for (int k = 1; k <= nt; ++k) s += ext[k - 1] * sp[k];
    return s;
  };
  if (!enhanced) {
    // regular PS (FO_WPgeometry_Routines.f90:776) or plane-parallel
    double calpha_boa, salpha_boa, alpha_boa_R = alpha_boa * DTR;
    if (alpha_boa == 90.0) { calpha_boa = 0.0; salpha_boa = 1.0; }
    else { calpha_boa = std::cos(alpha_boa_R); salpha_boa = std::sin(alpha_boa_R); }
    mu0 = ctheta_boa; mu1 = calpha_boa;
    if (overhead) { cosscat = -vsign * calpha_boa; if (calpha_boa == 0.0) cosscat = calpha_boa; }
    else cosscat = -vsign * calpha_boa * ctheta_boa + salpha_boa * stheta_boa * cphi;
    atten[0] = 1.0;
    for (int n = 1; n <= L; ++n) {
      std::fill(sp.begin(), sp.end(), 0.0);
      if (o->do_plane_parallel) {
        for (int k = 1; k <= n; ++k) sp[k] = (heights[k - 1] - heights[k]) / ctheta_boa;
      } else {
        sunpaths_D(overhead, radii[n], theta_boa_R, stheta_boa, n, sp.data());
      }
      double s = path_tau(n);
      suntau[n] = s;
      if (s < FO_CUTOFF) atten[n] = std::exp(-s);
    }
    for (int n = L; n >= 1; --n) {
      if (mu1 > 0.0) {
        double lostau = dts[n - 1] / mu1;
        if (lostau < FO_CUTOFF) lostrans[n - 1] = std::exp(-lostau);
        double f1 = atten[n - 1] - atten[n] * lostrans[n - 1];
        double f2 = 1.0 + (suntau[n] - suntau[n - 1]) / lostau;
        mult[n - 1] = f1 / f2;
      }
    }
  } else {
    // enhanced PS: LosOut_EnhancedPS_Initial_WP, _Quadrature_WP, SolarIn_..._SunPaths_WP
    bool donadir = (alpha_boa == 0.0);
    std::vector<double> losw(L + 1, 0.0), alpha(L + 1, 0.0), cosa(L + 1, 0.0), sina(L + 1, 0.0);
    double raycon = 0.0;
    if (donadir) {
      for (int n = L; n >= 1; --n) losw[n] = radii[n - 1] - radii[n];
    } else {
      double a_R = alpha_boa * DTR, salpha, calpha1;
      if (alpha_boa == 90.0) { salpha = 1.0; calpha1 = 0.0; }
      else { salpha = std::sin(a_R); calpha1 = std::cos(a_R); }
      cosa[L] = calpha1; sina[L] = salpha; alpha[L] = a_R;
      raycon = salpha * radii[L];
      for (int n = L - 1; n >= 0; --n) {
        sina[n] = raycon / radii[n];
        alpha[n] = std::asin(sina[n]);
        double calpha = std::cos(alpha[n]);
        cosa[n] = calpha;
        losw[n + 1] = radii[n] * calpha - radii[n + 1] * calpha1;
        calpha1 = calpha;
      }
    }
    // fine-layer quadrature (upwelling)
    std::vector<double> xfine(L * nf), wfine(L * nf), rfine(L * nf), afine(L * nf, 0.0);
    for (int n = L; n >= 1; --n) {
      if (donadir) {
        double difh = radii[n - 1] - radii[n];
        getquad2(0.0, difh, nf, tf.data(), af.data());
        for (int j = 0; j < nf; ++j) {
          rfine[(n - 1) * nf + j] = radii[n] + tf[j];
          xfine[(n - 1) * nf + j] = tf[j];
          wfine[(n - 1) * nf + j] = af[j];
        }
      } else {
        double rcn = radii[n] * cosa[n];
        getquad2(0.0, losw[n], nf, tf.data(), af.data());
        for (int j = 0; j < nf; ++j) {
          double tanfine = raycon / (rcn + tf[j]);
          double al = std::atan(tanfine);
          double sn = std::sin(al);
          afine[(n - 1) * nf + j] = al;
          rfine[(n - 1) * nf + j] = raycon / sn;
          xfine[(n - 1) * nf + j] = tf[j];
          wfine[(n - 1) * nf + j] = af[j];
        }
      }
    }
    double calpha_boa, salpha_boa;
    if (alpha_boa == 90.0) { calpha_boa = 0.0; salpha_boa = 1.0; }
    else { salpha_boa = std::sin(alpha[L]); calpha_boa = std::cos(alpha[L]); }
    mu1 = calpha_boa; mu0 = ctheta_boa;
    double sdir[3] = {0.0, 0.0, 0.0};
    if (!overhead) { sdir[0] = -stheta_boa * cphi * vsign; sdir[1] = -stheta_boa * sphi; sdir[2] = -ctheta_boa; }
    if (overhead) { cosscat = -vsign * calpha_boa; if (calpha_boa == 0.0) cosscat = calpha_boa; }
    else cosscat = -vsign * calpha_boa * ctheta_boa + salpha_boa * stheta_boa * cphi;
    auto findsun = [&](double radius, double cumangle, double* th, double* sth, bool* dirsun) {
      if (donadir) { *dirsun = true; *th = theta_boa_R; *sth = std::sin(theta_boa_R); return; }
      if (overhead) { *dirsun = true; *sth = std::sin(cumangle); *th = cumangle; return; }
      double px0 = -radius * std::sin(cumangle), px2 = radius * std::cos(cumangle);
      double b = px0 * sdir[0] + px2 * sdir[2];
      double ct = -b / radius;
      *dirsun = (ct >= 0.0);
      *sth = std::sqrt(1.0 - ct * ct);
      *th = std::acos(ct);
    };
    // whole-layer boundary at BOA (attenuation used by the direct bounce)
    for (int n = L; n >= 1; --n) {
      bool zero_sun_boa = overhead && (n == L || donadir);
      double th, sth; bool ds;
      if (n == L) { th = theta_boa_R; sth = stheta_boa; ds = true; }
      else findsun(radii[n], alpha[L] - alpha[n], &th, &sth, &ds);
      std::fill(sp.begin(), sp.end(), 0.0);
      int nt = n;
      if (ds) sunpaths_D(zero_sun_boa, radii[n], th, sth, n, sp.data());
      else nt = sunpaths_T(radii[n], th, sth, n, sp.data());
      double s = path_tau(nt);
      suntau[n] = s;
      if (s < FO_CUTOFF) atten[n] = std::exp(-s);
      // fine-layer attenuations and the layer multiplier
      double kn = ext[n - 1];
      double lostau = kn * losw[n];
      if (lostau < FO_CUTOFF) lostrans[n - 1] = std::exp(-lostau);
      double sum = 0.0;
      for (int j = 0; j < nf; ++j) {
        double thf, sthf; bool dsf;
        findsun(rfine[(n - 1) * nf + j], alpha[L] - afine[(n - 1) * nf + j], &thf, &sthf, &dsf);
        std::fill(sp.begin(), sp.end(), 0.0);
        int ntf = n;
        if (dsf) sunpaths_D(zero_sun_boa, rfine[(n - 1) * nf + j], thf, sthf, n, sp.data());
        else ntf = sunpaths_T(rfine[(n - 1) * nf + j], thf, sthf, n, sp.data());
        double sd = path_tau(ntf);
        double attf = sd < FO_CUTOFF ? std::exp(-sd) : 0.0;
        double dj = losw[n] - xfine[(n - 1) * nf + j];
        double tran = std::exp(-kn * dj);
        sum += attf * tran * wfine[(n - 1) * nf + j];
      }
      mult[n - 1] = sum * kn;
    }
  }
  G.mu0 = mu0; G.mu1 = mu1; G.cosscat = cosscat;
  G.atten = atten; G.lostrans = lostrans; G.mult = mult;
}

}  // namespace orc

using namespace orc;

extern "C" {

// One scalar VLIDORT solve for a single solar beam (sza) with nvza user zenith
// angles and nraa azimuths (lattice of one beam; nvza=nraa=1 is the AeroApps
// observation-geometry case).  Inputs are VLIDORT_MASTER optical inputs:
// heights[0..L] (km, TOA first), deltau[L], omega[L], greek[(ngreek+1)*L]
// (moment l of layer n at greek[l + (ngreek+1)*n]).  out[ua + nraa*um] is the
// TOA upwelling intensity STOKES(1,geom,1,UPIDX).  nfourier_out = last Fourier
// term summed.  Returns a status code.
//
// oracle_vlidort_solve_brdf: the same with a BRDF surface in place of the
// Lambertian albedo (DO_LAMBERTIAN_SURFACE = .false.): the Fourier components
// of oracle_brdf_supplement for m = 0..2N-1 (bf[(m N + i) N + j], bf0[m N + i],
// buf[(m nvza + u) N + j], buf0[m nvza + u]) and the exact direct-bounce BRDF
// bexact[u nraa + a].  bf == nullptr selects the Lambertian surface.
int oracle_vlidort_solve_brdf(const OracleOpts* o, int L, int N, int ngreek, const double* heights,
                              const double* deltau_in, const double* omega_in, const double* greek_in,
                              double albedo, double sza, int nvza, const double* vza, int nraa,
                              const double* raa, const double* bf, const double* bf0, const double* buf,
                              const double* buf0, const double* bexact, double* out, int* nfourier_out) {
  const bool brdf = bf != nullptr;
  const int order = o->taylor_order;
  const int NM = std::min(2 * N - 1, ngreek);  // vlidort_inputs.f90:4141
  const int G1 = ngreek + 1;
  const int N2 = 2 * N;
  // ---------------------------------------------------------------- derive input
  std::vector<double> qx(N), qw(N), strmwts(N), halfwts(N);
  if (N == 1) { qx[0] = std::sqrt(1.0 / 3.0); qw[0] = 1.0; }
  else getquad2(0.0, 1.0, N, qx.data(), qw.data());
  for (int i = 0; i < N; ++i) { strmwts[i] = qx[i] * qw[i]; halfwts[i] = 0.5 * qw[i]; }
  std::vector<double> mu_u(nvza), sec_u(nvza);
  for (int u = 0; u < nvza; ++u) { mu_u[u] = std::cos(DTR * vza[u]); sec_u[u] = 1.0 / mu_u[u]; }
  const double cos_sza = std::cos(sza * DTR);
  // DO_LAYER_SCATTERING(M,N), vlidort_inputs.f90:4321-4330 (solar sources)
  std::vector<char> laysc((NM + 1) * L, 1);
  for (int m = 3; m <= NM; ++m) {
    int qc = NM - m + 1;
    for (int n = 0; n < L; ++n) {
      int q = 0;
      for (int l = m; l <= NM; ++l)
        if (greek_in[l + G1 * n] == 0.0) q++;
      laysc[m + (NM + 1) * n] = (q < qc);
    }
  }
  // ---------------------------------------------------------------- Chapman factors
  // vlidort_geometry.f90:119-317 (straight-line, non-refractive)
  std::vector<double> chap(L * L, 0.0);  // chap[n*L + k], k <= n
  {
    double mu_toa = std::cos(sza * DTR);
    double sn_toa = std::sqrt(1.0 - mu_toa * mu_toa);
    std::vector<double> radii(L + 1), delz(L + 1);
    radii[0] = heights[0] + o->earth_radius;
    for (int n = 1; n <= L; ++n) { radii[n] = heights[n] + o->earth_radius; delz[n] = heights[n - 1] - heights[n]; }
    if (o->do_plane_parallel) {
      for (int n = 0; n < L; ++n) for (int k = 0; k <= n; ++k) chap[n * L + k] = 1.0 / mu_toa;
    } else if (sn_toa == 0.0) {
      for (int n = 0; n < L; ++n) for (int k = 0; k <= n; ++k) chap[n * L + k] = 1.0;
    } else {
      for (int n = 1; n <= L; ++n) {
        double sinth1 = sn_toa * radii[n] / radii[0];
        double sth1 = std::asin(sinth1);
        double re_upper = radii[0];
        for (int k = 1; k <= n; ++k) {
          double re_lower = re_upper - delz[k];
          double sinth2 = re_upper * sinth1 / re_lower;
          double sth2 = std::asin(sinth2);
          double phi = sth2 - sth1;
          double dist = re_upper * std::sin(phi) / sinth2;
          chap[(n - 1) * L + (k - 1)] = dist / delz[k];
          re_upper = re_lower; sinth1 = sinth2; sth1 = sth2;
        }
      }
    }
  }
  // ---------------------------------------------------------------- delta-M scaling
  // vlidort_miscsetups.f90:370-758
  std::vector<double> dtau(L), omg(L), fac1(L), trunc(L), greek((NM + 1) * L, 0.0);
  if (o->do_deltam) {
    int nm1 = NM + 1;
    double dnm1 = (double)(2 * nm1 + 1);
    for (int n = 0; n < L; ++n) {
      double fdel = greek_in[nm1 + G1 * n] / dnm1;
      double fac2 = 1.0 - fdel;
      fac1[n] = 1.0 - fdel * omega_in[n];
      trunc[n] = fdel;
      for (int l = 0; l <= NM; ++l) {
        double fdnl1 = fdel * (double)(2 * l + 1);
        greek[l + (NM + 1) * n] = (greek_in[l + G1 * n] - fdnl1) / fac2;
      }
      greek[0 + (NM + 1) * n] = 1.0;
      dtau[n] = deltau_in[n] * fac1[n];
      omg[n] = omega_in[n] * fac2 / fac1[n];
    }
  } else {
    for (int n = 0; n < L; ++n) {
      fac1[n] = 1.0; trunc[n] = 0.0; omg[n] = omega_in[n]; dtau[n] = deltau_in[n];
      for (int l = 0; l <= NM; ++l) greek[l + (NM + 1) * n] = greek_in[l + G1 * n];
    }
  }
  for (int n = 0; n < L; ++n) {  // :627-651 clamps on omega and the first moment
    if (omg[n] > 0.999999999) omg[n] = 0.999999999;
    else if (omg[n] < 1.0e-9) omg[n] = 1.0e-9;
    double g1 = greek[1 + (NM + 1) * n] / 3.0;
    if (g1 > 0.999999999) g1 = 0.999999999;
    else if (g1 < -0.999999999) g1 = -0.999999999;
    else if (g1 >= 0.0 && g1 < 1.0e-9) g1 = 1.0e-9;
    else if (g1 < 0.0 && g1 > -1.0e-9) g1 = -1.0e-9;
    greek[1 + (NM + 1) * n] = 3.0 * g1;
  }
  // slant optical depths (scaled)
  std::vector<double> tauslant(L + 1, 0.0);
  for (int n = 0; n < L; ++n) {
    double tau = 0.0;
    for (int k = 0; k <= n; ++k) tau += (deltau_in[k] * chap[n * L + k]) * (o->do_deltam ? fac1[k] : 1.0);
    tauslant[n + 1] = tau;
  }
  // SSALBINIT :762
  std::vector<double> og((NM + 1) * L);
  for (int n = 0; n < L; ++n)
    for (int l = 0; l <= NM; ++l) og[l + (NM + 1) * n] = omg[n] * greek[l + (NM + 1) * n];
  // ---------------------------------------------------------------- QSPREP :813-1010
  int cutoff = L;
  std::vector<double> avsec(L, 0.0), itrans(L, 0.0);
  double trans_solar_beam = 0.0;
  bool refl_directbeam = false;
  {
    std::vector<double> taugrid(L + 1, 0.0);
    for (int n = 0; n < L; ++n) taugrid[n + 1] = taugrid[n] + dtau[n];
    double tau_solar;
    if (o->do_plane_parallel) {
      double sec0 = 1.0 / cos_sza;
      for (int n = 1; n <= L; ++n) {
        double ts = taugrid[n] * sec0;
        if (n <= cutoff) {
          if (ts > MAX_TAU_SPATH) cutoff = n;
          avsec[n - 1] = sec0;
          itrans[n - 1] = std::exp(-taugrid[n - 1] * sec0);
        }
      }
      tau_solar = taugrid[L] * sec0;
    } else {
      tau_solar = tauslant[L];
      double s_t_1 = 0.0, s_t_0 = 1.0;
      for (int n = 1; n <= L; ++n) {
        if (n <= cutoff) {
          if (tauslant[n] > MAX_TAU_SPATH) cutoff = n;
          else s_t_1 = std::exp(-tauslant[n]);
          avsec[n - 1] = (tauslant[n] - tauslant[n - 1]) / dtau[n - 1];
          itrans[n - 1] = s_t_0;
          s_t_0 = s_t_1;
        }
      }
    }
    if (tau_solar < MAX_TAU_SPATH) { trans_solar_beam = std::exp(-tau_solar); refl_directbeam = true; }
  }
  // ---------------------------------------------------------------- PREPTRANS :1014-1292
  std::vector<double> t_mubar(L, 0.0), t_user(L * nvza, 0.0), itrans_u(L * nvza, 0.0);
  for (int n = 0; n < L; ++n) {
    if (n + 1 <= cutoff) {
      double sp = dtau[n] * avsec[n];
      t_mubar[n] = sp > MAX_TAU_SPATH ? 0.0 : std::exp(-sp);
    }
    for (int u = 0; u < nvza; ++u) {
      itrans_u[n + L * u] = itrans[n] * sec_u[u];
      double sp = dtau[n] * sec_u[u];
      t_user[n + L * u] = sp > MAX_TAU_UPATH ? 0.0 : std::exp(-sp);
    }
  }
  // EMULT (upwelling), miscsetups :3187 / :2936
  std::vector<double> sigma_p(L * nvza), emult_up(L * nvza, 0.0);
  for (int n = 0; n < L; ++n)
    for (int u = 0; u < nvza; ++u) {
      sigma_p[n + L * u] = avsec[n] + sec_u[u];
      if (n + 1 <= cutoff) {
        double wudel = t_mubar[n] * t_user[n + L * u];
        double su = (1.0 - wudel) / sigma_p[n + L * u];
        emult_up[n + L * u] = itrans_u[n + L * u] * su;
      }
    }
  // ---------------------------------------------------------------- FO single scatter + direct bounce
  // vlidort_vfo_interface.f90:128 -> VFO_Master.f90:123 -> FO_SSWPgeometry_master.f90:101,
  // FO_WPgeometry_Routines.f90:776 (regular PS), :1511/:1700/:2409 (enhanced PS),
  // FO_VectorSS_Spherfuncs.f90:93, FO_VectorSS_RTCalcs_I.f90:116 (SSV_Integral_I_UP)
  const int NG = nvza * nraa;
  std::vector<double> ss(NG, 0.0), db(NG, 0.0);
  if (o->do_focorr) {
    const double flux = o->flux_factor / PI4;
    std::vector<double> radii(L + 1), ext(L), dts(L), tms(L);
    for (int n = 0; n <= L; ++n) radii[n] = o->earth_radius + heights[n];
    for (int n = 0; n < L; ++n) {
      double dz = heights[n] - heights[n + 1];
      dts[n] = o->do_deltam ? dtau[n] : deltau_in[n];
      ext[n] = dts[n] / dz;
      tms[n] = o->do_deltam ? omega_in[n] / (1.0 - trunc[n] * omega_in[n]) : omega_in[n];
    }
    for (int u = 0; u < nvza; ++u)
      for (int a = 0; a < nraa; ++a) {
        const int g = a + nraa * u;
        FoGeom G;
        fo_geometry(o, L, heights, radii, ext, dts, sza, vza[u], raa[a], G);
        const double mu0 = G.mu0, cosscat = G.cosscat;
        const std::vector<double>& atten = G.atten;
        const std::vector<double>& lostrans = G.lostrans;
        const std::vector<double>& mult = G.mult;
        // scattering-angle Legendre sum (FO_VectorSS_Spherfuncs.f90, NSTOKES=1)
        std::vector<double> gs(ngreek + 1);
        gs[0] = 1.0;
        if (ngreek >= 1) gs[1] = cosscat;
        for (int l = 2; l <= ngreek; ++l)
          gs[l] = ((double)(2 * l - 1) / (double)l) * gs[l - 1] * cosscat - ((double)(l - 1) / (double)l) * gs[l - 2];
        double cum = 0.0;
        // FO direct bounce: the exact BRDF of the geometry (vlidort_vfo_interface.f90:594-617)
        const double reflec_db = brdf ? bexact[u * nraa + a] : albedo;
        double cumdb = 4.0 * mu0 * reflec_db * atten[L] * 1.0;
        for (int n = L; n >= 1; --n) {
          double fmat = 0.0;
          for (int l = 0; l <= ngreek; ++l) fmat += gs[l] * greek_in[l + G1 * (n - 1)];
          double exactscat = fmat * tms[n - 1];
          double source = exactscat * 1.0 * mult[n - 1];
          cumdb = lostrans[n - 1] * cumdb;
          cum = lostrans[n - 1] * cum + source;
        }
        ss[g] = flux * cum;
        db[g] = flux * cumdb;
      }
  }
  // ---------------------------------------------------------------- Fourier loop
  // vlidort_masters_V2p8p3.f90:2305-2700 and VLIDORT_FOURIER :3107
  const bool do_dbcorr = o->do_focorr != 0;
  const bool msmode = o->do_focorr != 0;  // FULLRAD with FO correction (inputs.f90 :3996)
  std::vector<double> stokes(NG, 0.0);
  int testconv = 0;
  bool iterate = true;
  int fourier = -1;
  // per-Fourier arrays
  std::vector<double> piq((NM + 1) * N), piu((NM + 1) * nvza), pi0(NM + 1), pimm_q(N), pimm_u(nvza), pimm_0(1);
  std::vector<double> xpos(N2 * N * L), xneg(N2 * N * L), keig(N * L), teig(N * L), norm(N * L);
  std::vector<double> uhom_dn(nvza * N * L), uhom_up(nvza * N * L), hm1(nvza * N * L), hm2(nvza * N * L);
  std::vector<double> zeta_m(nvza * N * L), zeta_p(nvza * N * L);
  std::vector<char> hsingo(nvza * N * L);
  std::vector<double> aterm(N * L), bterm(N * L), gam_p(N * L), gam_m(N * L), wupper(N2 * L), wlower(N2 * L);
  std::vector<double> upar1(nvza * L);
  const int NT = N2 * L;
  const int KL = (L == 1) ? (2 * N - 1) : (3 * N - 1), KU = KL;
  const int LDAB = 2 * KL + KU + 1;
  std::vector<double> ab(LDAB * NT), col(NT);
  std::vector<int> ipiv(NT);
  std::vector<double> sab(N * N), dab(N * N), emat(N * N), evec(N * N), eval(N), wk(4 * N), esave(N * N);
  std::vector<double> h2p((NM + 1) * N), h2m((NM + 1) * N), helpl(NM + 1);
  auto XP = [&](int i, int k, int n) -> double& { return xpos[i + N2 * (k + N * n)]; };
  auto XN = [&](int i, int k, int n) -> double& { return xneg[i + N2 * (k + N * n)]; };
  auto sgn = [](int lm) { return (lm % 2 == 0) ? 1.0 : -1.0; };
  // DO_NO_AZIMUTH (inputs.f90 :3953): scalar, nadir-only view, no FO correction
  const int n_fouriers = (nvza == 1 && vza[0] == 0.0 && !o->do_focorr) ? 0 : NM;
  while (iterate && fourier < n_fouriers) {
    fourier++;
    const int m = fourier;
    // a BRDF surface reflects in every Fourier term (vlidort_masters_V2p8p3.f90:2380-2400)
    const bool incl_surface = brdf ? true : ((m == 0) && (albedo != 0.0));
    const double surface_factor = (m == 0) ? 2.0 : 1.0;
    const double delta_factor = (m == 0) ? 1.0 : 2.0;
    const double flux_multiplier = delta_factor;
    // DIRECTRADIANCE, miscsetups :1296 (Lambertian, Fourier 0 only)
    double direct_beam = 0.0, beam_attn = 0.0;
    std::vector<double> direct_beam_q(N, 0.0);  // DIRECT_BEAM(i): per stream for a BRDF (miscsetups :1517-1545)
    bool localbeam = incl_surface ? refl_directbeam : false;
    if (incl_surface && refl_directbeam) {
      double x0_flux = 4.0 * cos_sza / delta_factor;
      x0_flux = o->flux_factor * x0_flux / PI4;
      double attn = x0_flux * trans_solar_beam;
      beam_attn = attn;
      if (brdf) {
        for (int i = 0; i < N; ++i) direct_beam_q[i] = attn * bf0[m * N + i];
      } else if (m == 0) {
        direct_beam = attn * albedo;
        for (int i = 0; i < N; ++i) direct_beam_q[i] = direct_beam;
      }
    }
    // PIMATRIX_SETUP_OMP, miscsetups :2273 (NSTOKES = 1)
    {
      double phi = 1.0, fac = 1.0;
      for (int l = 1; l <= 2 * m; ++l) fac *= (double)l;
      std::vector<double> pinorm(NM + 1, 0.0), phiv(NM + 1, 0.0);
      phiv[m] = phi / fac;
      for (int l = m + 1; l <= NM; ++l) phiv[l] = phiv[l - 1] * ((double)(l - m) / (double)(l + m));
      for (int l = m; l <= NM; ++l) pinorm[l] = std::sqrt(phiv[l]);
      auto fill = [&](double x, double* pim, double* out_pi /*stride 1*/) {
        std::vector<double> P(NM + 2, 0.0);
        double umxsq = 1.0 - x * x;
        double rt = (x == 1.0) ? 0.0 : std::sqrt(umxsq);
        if (m == 0) {
          P[0] = 1.0;
          if (NM >= 1) P[1] = x;
          if (NM >= 2) P[2] = 0.5 * (3.0 * x * x - 1.0);
          for (int l = 2; l <= NM - 1; ++l)
            P[l + 1] = (x * (double)(2 * l + 1) * P[l] - (double)l * P[l - 1]) * (1.0 / (double)(l + 1));
        } else if (m == 1) {
          P[1] = rt;
          if (NM >= 2) P[2] = 3.0 * (rt * x);
          for (int l = 2; l <= NM - 1; ++l)
            P[l + 1] = (x * (double)(2 * l + 1) * P[l] - (double)(l + 1) * P[l - 1]) * (1.0 / (double)l);
        } else {
          if (m == 2) *pim = 3.0 * umxsq;
          else *pim = (double)(2 * (m - 1) + 1) * rt * (*pim);
          P[m] = *pim;
          if (m < NM) P[m + 1] = x * (double)(2 * m + 1) * P[m] * 1.0;
          for (int l = m + 1; l <= NM - 1; ++l)
            P[l + 1] = (x * (double)(2 * l + 1) * P[l] - (double)(l + m) * P[l - 1]) * (1.0 / (double)(l + 1 - m));
        }
        for (int l = m; l <= NM; ++l) out_pi[l] = P[l] * pinorm[l];
      };
      std::vector<double> tmp(NM + 1);
      for (int i = 0; i < N; ++i) {
        fill(qx[i], &pimm_q[i], tmp.data());
        for (int l = 0; l <= NM; ++l) piq[l + (NM + 1) * i] = (l >= m) ? tmp[l] : 0.0;
      }
      for (int u = 0; u < nvza; ++u) {
        fill(mu_u[u], &pimm_u[u], tmp.data());
        for (int l = 0; l <= NM; ++l) piu[l + (NM + 1) * u] = (l >= m) ? tmp[l] : 0.0;
      }
      fill(cos_sza, &pimm_0[0], tmp.data());
      for (int l = 0; l <= NM; ++l) pi0[l] = (l >= m) ? tmp[l] : 0.0;
    }
    // ------------------------------------------------ homogeneous solutions per layer
    for (int n = 0; n < L; ++n) {
      const double* OG = &og[(NM + 1) * n];
      // QHOM_SOLUTION, solutions.f90:150 (SAB/DAB contraction, eigenmatrix)
      for (int j = 0; j < N; ++j)
        for (int l = m; l <= NM; ++l) {
          double p = piq[l + (NM + 1) * j];
          h2p[l + (NM + 1) * j] = OG[l] * p;
          h2m[l + (NM + 1) * j] = OG[l] * (p * sgn(l - m));
        }
      for (int i = 0; i < N; ++i) {
        double xinv = -1.0 / qx[i];
        for (int j = 0; j < N; ++j) {
          double f = xinv * halfwts[j];
          double dp = 0.0, dm = 0.0;
          for (int l = m; l <= NM; ++l) {
            dp += piq[l + (NM + 1) * i] * h2p[l + (NM + 1) * j];
            dm += piq[l + (NM + 1) * i] * h2m[l + (NM + 1) * j];
          }
          sab[i + N * j] = f * (dp + dm);
          dab[i + N * j] = f * (dp - dm);
        }
        sab[i + N * i] -= xinv;
        dab[i + N * i] -= xinv;
      }
      for (int i = 0; i < N; ++i)
        for (int j = 0; j < N; ++j) {
          double s = 0.0;
          for (int k = 0; k < N; ++k) s += dab[i + N * k] * sab[k + N * j];
          emat[i + N * j] = s;
        }
      esave = emat;
      bool bad;
      int ier = asymtx(o->asymtx_tol, emat.data(), N, N, evec.data(), eval.data(), wk.data(), &bad);
      if (bad) return ORC_EIGEN_FAIL;
      if (ier > 0) {
        emat = esave;
        ier = asymtx(1.0e-10, emat.data(), N, N, evec.data(), eval.data(), wk.data(), &bad);
        if (ier > 0) {
          emat = esave;
          ier = asymtx(1.0e-8, emat.data(), N, N, evec.data(), eval.data(), wk.data(), &bad);
          if (ier > 0 || bad) return ORC_EIGEN_FAIL;
        }
      }
      for (int a = 0; a < N; ++a) {
        double s = 0.0;
        for (int i = 0; i < N; ++i) s += evec[i + N * a] * evec[i + N * a];
        s = std::sqrt(s);
        for (int i = 0; i < N; ++i) evec[i + N * a] /= s;
      }
      for (int k = 0; k < N; ++k) {
        if (!(eval[k] > 0.0)) return ORC_EIGEN_FAIL;
        double kv = std::sqrt(eval[k]);
        keig[k + N * n] = kv;
        double sc = 1.0 / kv;
        double nr = 0.0;
        for (int i = 0; i < N; ++i) nr += evec[i + N * k] * evec[i + N * k];
        nr = std::sqrt(nr);
        std::vector<double> sumv(N), difv(N);
        for (int i = 0; i < N; ++i) sumv[i] = evec[i + N * k] / nr;
        for (int i = 0; i < N; ++i) {
          double h = 0.0;
          for (int j = 0; j < N; ++j) h += sab[i + N * j] * sumv[j];
          difv[i] = h * sc;
        }
        for (int i = 0; i < N; ++i) {
          double fpd = 0.5 * (sumv[i] + difv[i]);
          double fnd = 0.5 * (sumv[i] - difv[i]);
          XP(i, k, n) = fpd; XP(i + N, k, n) = fnd;
          XN(i, k, n) = fnd; XN(i + N, k, n) = fpd;
        }
        double help = kv * dtau[n];
        teig[k + N * n] = help > MAX_TAU_QPATH ? 0.0 : std::exp(-help);
      }
      // UHOM_SOLUTION, solutions.f90:1167 (upwelling user streams)
      for (int u = 0; u < nvza; ++u)
        for (int k = 0; k < N; ++k) {
          int idx = u + nvza * (k + N * n);
          double rho_p = sec_u[u] + keig[k + N * n];
          double rho_m = sec_u[u] - keig[k + N * n];
          zeta_p[idx] = 1.0 / rho_p;
          hsingo[idx] = std::fabs(rho_m) < TAYLOR_SMALL;
          zeta_m[idx] = hsingo[idx] ? rho_m : 1.0 / rho_m;
        }
      const bool lsc = laysc[m + (NM + 1) * n];
      for (int k = 0; k < N; ++k) {
        for (int l = m; l <= NM; ++l) {
          double sps = 0.0;
          for (int j = 0; j < N; ++j) {
            double a5 = halfwts[j];
            double p = piq[l + (NM + 1) * j];
            double sp = p * a5 * XP(j, k, n);
            double sm = (p * sgn(l - m)) * a5 * XN(j, k, n);
            sps = sps + sp + sm;
          }
          helpl[l] = OG[l] * sps;
        }
        for (int u = 0; u < nvza; ++u) {
          double dn = 0.0, up = 0.0;
          for (int l = m; l <= NM; ++l) {
            double pu = piu[l + (NM + 1) * u];
            dn += (pu * sgn(l - m)) * helpl[l];
            up += pu * helpl[l];
          }
          uhom_dn[u + nvza * (k + N * n)] = lsc ? dn : 0.0;
          uhom_up[u + nvza * (k + N * n)] = lsc ? up : 0.0;
        }
      }
      // QHOM_NORMS :1051
      for (int k = 0; k < N; ++k) {
        double s = 0.0;
        for (int j = 0; j < N; ++j) s += strmwts[j] * (XP(j, k, n) * XP(j, k, n) - XN(j, k, n) * XN(j, k, n));
        norm[k + N * n] = s;
      }
      // HMULT (whole layer) :1651
      for (int u = 0; u < nvza; ++u) {
        double udel = t_user[n + L * u], smu = sec_u[u];
        for (int k = 0; k < N; ++k) {
          int idx = u + nvza * (k + N * n);
          double zdel = teig[k + N * n], zudel = zdel * udel;
          double th2 = 1.0 - zudel, th1 = zdel - udel;
          if (hsingo[idx]) hm1[idx] = taylor1(order, zeta_m[idx], dtau[n], udel, smu);
          else hm1[idx] = smu * th1 * zeta_m[idx];
          hm2[idx] = smu * th2 * zeta_p[idx];
        }
      }
    }
    // ------------------------------------------------ BVP matrix (bvproblem.f90:627) + LU (:1180)
    std::fill(ab.begin(), ab.end(), 0.0);
    auto AB = [&](int i, int j) -> double& { return ab[(KL + KU + i - j) + LDAB * j]; };  // 0-based i,j
    double r2homp_fac = incl_surface ? surface_factor * albedo : 0.0;
    {
      for (int i = 0; i < N; ++i)
        for (int k = 0; k < N; ++k) {
          AB(i, k) = XP(i, k, 0);
          AB(i, k + N) = XN(i, k, 0) * teig[k];
        }
      for (int n = 1; n < L; ++n) {
        int c0 = n * N2 - N;       // first row of interface n-1/n
        int ce = c0 - N;           // first column of layer n-1
        for (int i = 0; i < N2; ++i) {
          int cm = c0 + i;
          for (int k = 0; k < N; ++k) {
            AB(cm, ce + k) = teig[k + N * (n - 1)] * XP(i, k, n - 1);
            AB(cm, ce + k + N) = XN(i, k, n - 1);
            AB(cm, ce + k + N2) = -XP(i, k, n);
            AB(cm, ce + k + N + N2) = -teig[k + N * n] * XN(i, k, n);
          }
        }
      }
      int c0 = N2 * L - N, ce = N2 * (L - 1);
      // R2_HOMP/R2_HOMM (bvproblem.f90:538-614): one row for every stream i
      // (Lambertian: the same for all i; BRDF: AXBID_F = QUAD_STRMWTS(j) BRDF_F(i, j))
      std::vector<double> r2p(N * N, 0.0), r2m(N * N, 0.0);
      if (incl_surface)
        for (int i = 0; i < N; ++i)
          for (int k = 0; k < N; ++k) {
            double sp = 0.0, sm = 0.0;
            if (brdf) {
              for (int j = 0; j < N; ++j) {
                const double ax = strmwts[j] * bf[(m * N + i) * N + j];
                sp += ax * XP(j, k, L - 1);
                sm += ax * XN(j, k, L - 1);
              }
              r2p[i + N * k] = surface_factor * sp; r2m[i + N * k] = surface_factor * sm;
            } else {
              for (int j = 0; j < N; ++j) { sp += strmwts[j] * XP(j, k, L - 1); sm += strmwts[j] * XN(j, k, L - 1); }
              r2p[i + N * k] = sp * r2homp_fac; r2m[i + N * k] = sm * r2homp_fac;
            }
          }
      for (int i = 0; i < N; ++i)
        for (int k = 0; k < N; ++k) {
          double xpnet = XP(i + N, k, L - 1) - r2p[i + N * k];
          double xmnet = XN(i + N, k, L - 1) - r2m[i + N * k];
          AB(c0 + i, ce + k) = teig[k + N * (L - 1)] * xpnet;
          AB(c0 + i, ce + k + N) = xmnet;
        }
    }
    if (band_lu(NT, KL, KU, ab.data(), LDAB, ipiv.data()) != 0) return ORC_BVP_SINGULAR;
    // ------------------------------------------------ beam particular solutions (Green's function)
    const double F1 = o->flux_factor / PI4;
    std::vector<double> dpi(N), dmi(N), hq(NM + 1);
    for (int n = 0; n < L; ++n) {
      bool active = (n + 1 <= cutoff) && laysc[m + (NM + 1) * n];
      for (int i = 0; i < N2; ++i) { wupper[i + N2 * n] = 0.0; wlower[i + N2 * n] = 0.0; }
      for (int u = 0; u < nvza; ++u) upar1[u + nvza * n] = 0.0;
      if (!active) continue;
      // GBEAM_SOLUTION :2649
      double secbar = avsec[n], cnst = itrans[n], wdel = t_mubar[n];
      std::vector<double> cfunc(N), dfunc(N);
      for (int k = 0; k < N; ++k) {
        double zdel = teig[k + N * n], zwdel = zdel * wdel;
        gam_p[k + N * n] = secbar + keig[k + N * n];
        gam_m[k + N * n] = secbar - keig[k + N * n];
        double eps = gam_m[k + N * n];
        if (std::fabs(eps) < TAYLOR_SMALL) cfunc[k] = taylor1(order, eps, dtau[n], wdel, cnst);
        else cfunc[k] = cnst * (zdel - wdel) / gam_m[k + N * n];
        dfunc[k] = cnst * (1.0 - zwdel) / gam_p[k + N * n];
      }
      const double* OG = &og[(NM + 1) * n];
      for (int l = m; l <= NM; ++l) hq[l] = OG[l] * (pi0[l] * 1.0);
      for (int i = 0; i < N; ++i) {
        double sp = 0.0, sm = 0.0;
        for (int l = m; l <= NM; ++l) {
          sp += piq[l + (NM + 1) * i] * hq[l];
          sm += (piq[l + (NM + 1) * i] * sgn(l - m)) * hq[l];
        }
        dpi[i] = F1 * sp; dmi[i] = F1 * sm;
      }
      std::vector<double> gdn(N), gup(N);
      for (int k = 0; k < N; ++k) {
        double s1 = 0.0, s2 = 0.0;
        for (int i = 0; i < N; ++i) {
          double h1 = dpi[i] * XP(i, k, n) + dmi[i] * XN(i, k, n);
          double h2 = dmi[i] * XP(i, k, n) + dpi[i] * XN(i, k, n);
          s1 += qw[i] * h1; s2 += qw[i] * h2;
        }
        aterm[k + N * n] = s1 / norm[k + N * n];
        bterm[k + N * n] = s2 / norm[k + N * n];
        gdn[k] = cfunc[k] * aterm[k + N * n];
        gup[k] = dfunc[k] * bterm[k + N * n];
      }
      for (int i = 0; i < N; ++i) {
        double wu1 = 0, wu2 = 0, wl1 = 0, wl2 = 0;
        for (int k = 0; k < N; ++k) {
          wu1 += gup[k] * XN(i, k, n); wu2 += gup[k] * XP(i, k, n);
          wl1 += gdn[k] * XN(i, k, n); wl2 += gdn[k] * XP(i, k, n);
        }
        wupper[i + N2 * n] = wu1; wupper[i + N + N2 * n] = wu2;
        wlower[i + N + N2 * n] = wl1; wlower[i + N2 * n] = wl2;
      }
      // GUSER_SOLUTION :2936 (upwelling, needed when single scatter is not FO-corrected)
      for (int u = 0; u < nvza; ++u) {
        double s = 0.0;
        for (int l = m; l <= NM; ++l) s += (F1 * hq[l]) * (piu[l + (NM + 1) * u] * sgn(l - m));
        upar1[u + nvza * n] = s;
      }
    }
    // BVP column (bvproblem.f90:1743) and back substitution
    std::fill(col.begin(), col.end(), 0.0);
    for (int i = 0; i < N; ++i) col[i] = -wupper[i];
    for (int n = 1; n < L; ++n) {
      int c0 = n * N2 - N;
      for (int i = 0; i < N2; ++i) col[c0 + i] = wupper[i + N2 * n] - wlower[i + N2 * (n - 1)];
    }
    {
      int c0 = (L - 1) * N2 + N;
      // R2_BEAM (bvproblem.f90:1680-1736) and the direct beam (:1903-1913)
      double r2b = 0.0;
      if (incl_surface && !brdf) {
        for (int j = 0; j < N; ++j) r2b += strmwts[j] * wlower[j + N2 * (L - 1)];
        r2b = r2b * surface_factor * albedo;
      }
      for (int i = 0; i < N; ++i) {
        double r2bi = r2b;
        if (incl_surface && brdf) {
          double s = 0.0;
          for (int j = 0; j < N; ++j) s += strmwts[j] * bf[(m * N + i) * N + j] * wlower[j + N2 * (L - 1)];
          r2bi = surface_factor * s;
        }
        col[c0 + i] = -wlower[i + N + N2 * (L - 1)] + (incl_surface ? r2bi : 0.0);
        if (localbeam && incl_surface) col[c0 + i] += direct_beam_q[i];
      }
    }
    band_solve(NT, KL, KU, ab.data(), LDAB, ipiv.data(), col.data());
    auto LCON = [&](int k, int n) { return col[n * N2 + k]; };
    auto MCON = [&](int k, int n) { return col[n * N2 + N + k]; };
    // ------------------------------------------------ UPUSER_INTENSITY (intensity.f90:145), TOA only
    std::vector<double> stokes_f(nvza, 0.0);
    {
      const bool incl_directrf = (localbeam && !do_dbcorr) && !msmode;
      // BOA surface source (intensity.f90:1300-1420): STOKES_DOWNSURF(i) =
      // QUAD_STRMWTS(i) * downwelling; Lambertian: albedo times their sum;
      // BRDF: their product with USER_BRDF_F(u, i)
      double reflec = 0.0;
      std::vector<double> downsurf(N, 0.0);
      if (incl_surface) {
        double s = 0.0;
        for (int i = 0; i < N; ++i) {
          double shom = 0.0;
          for (int k = 0; k < N; ++k) {
            double lxr = LCON(k, L - 1) * XP(i, k, L - 1);
            double mxr = MCON(k, L - 1) * XN(i, k, L - 1);
            shom = shom + lxr * teig[k + N * (L - 1)] + mxr;
          }
          downsurf[i] = strmwts[i] * (wlower[i + N2 * (L - 1)] + shom);
          s += downsurf[i];
        }
        reflec = surface_factor * albedo * s;
      }
      for (int u = 0; u < nvza; ++u) {
        double cum = 0.0;
        if (incl_surface) {
          if (brdf) {
            double s = 0.0;
            for (int j = 0; j < N; ++j) s += downsurf[j] * buf[(m * nvza + u) * N + j];
            cum = surface_factor * s;
          } else {
            cum = reflec;
          }
        }
        if (incl_surface && incl_directrf && !do_dbcorr) cum += brdf ? beam_attn * buf0[m * nvza + u] : direct_beam;
        for (int n = L - 1; n >= 0; --n) {
          double src = 0.0;
          if (laysc[m + (NM + 1) * n]) {
            double h = 0.0;
            for (int k = 0; k < N; ++k) {
              int idx = u + nvza * (k + N * n);
              double luxr = LCON(k, n) * uhom_dn[idx];
              double muxr = MCON(k, n) * uhom_up[idx];
              h = h + luxr * hm2[idx] + muxr * hm1[idx];
            }
            src = h;
            if (n + 1 <= cutoff) {
              double wdel = t_mubar[n], it = itrans[n], itw = -it * wdel;
              double spar = 0.0;
              double em = emult_up[n + L * u];
              for (int k = 0; k < N; ++k) {
                int idx = u + nvza * (k + N * n);
                double sd;
                if (std::fabs(gam_m[k + N * n]) < TAYLOR_SMALL) {
                  double mult = taylor2(order, gam_m[k + N * n], sigma_p[n + L * u], dtau[n], 1.0,
                                        wdel * t_user[n + L * u], 1.0);
                  sd = itrans_u[n + L * u] * mult;
                } else {
                  sd = (it * hm2[idx] - em) / gam_m[k + N * n];
                }
                double su = (itw * hm1[idx] + em) / gam_p[k + N * n];
                spar += uhom_dn[idx] * sd * aterm[k + N * n] + uhom_up[idx] * su * bterm[k + N * n];
              }
              src += spar;
              if (!msmode) src += upar1[u + nvza * n] * em;
            }
          }
          cum = src + t_user[n + L * u] * cum;
        }
        stokes_f[u] = flux_multiplier * cum;
      }
    }
    // ------------------------------------------------ convergence (converge.f90:128 / :825)
    if (m == 0) {
      for (int u = 0; u < nvza; ++u)
        for (int a = 0; a < nraa; ++a) {
          int g = a + nraa * u;
          stokes[g] = stokes_f[u];
          if (o->do_focorr) stokes[g] += ss[g];
          if (o->do_focorr || do_dbcorr) stokes[g] += db[g];
        }
    } else {
      int count = 0;
      for (int a = 0; a < nraa; ++a)
        for (int u = 0; u < nvza; ++u) {
          int g = a + nraa * u;
          double azmfac = std::cos(raa[a] * (double)m * DTR);
          double told = stokes[g], tazm = azmfac * stokes_f[u], tnew = told + tazm;
          if (tazm != 0.0) {
            if (std::fabs(tazm / tnew) < o->accuracy) count++;
          } else {
            count++;
          }
          stokes[g] = tnew;
        }
      if (count == NG) {
        testconv++;
        if (o->do_double_convtest) { if (testconv == 2) iterate = false; }
        else iterate = false;
      } else {
        testconv = 0;
      }
    }
  }
  for (int g = 0; g < NG; ++g) out[g] = stokes[g];
  if (nfourier_out) *nfourier_out = fourier;
  return ORC_OK;
}

}  // extern "C"

// ------------------------------------------------------------------------------------------
// The AeroApps glue: VLIDORT_Scalar_Lambert (geo_vlidort/VLIDORT_LAMBERT.F90:34-168) calling
// VLIDORT_Init (VLIDORT2p8p3/VLIDORT_Mod.F90:65-383) and VLIDORT_Run_Scalar
// (VLIDORT2p8p3/VLIDORT_ScatMod.F90:975-1247) per (observation, channel).
// Arrays are Fortran column-major exactly as the reference declares them.
// Pixels are independent apart from the sticky nadir-FO flag, which is resolved
// up front in loop order, so the loop runs with OpenMP over pixels.
// nfourier (nobs,nch) and status (nobs,nch) are optional diagnostics.
// ASYMTX tolerance used by oracle_scalar_lambert: AeroApps sets 1.0d-12
// (VLIDORT2p8p3/VLIDORT_Mod.F90:355); tests may tighten it to check how far
// that tolerance moves the reference algorithm from the converged solution.
static double g_asymtx_tol = 1.0e-12;
extern "C" int oracle_vlidort_solve(const OracleOpts* o, int L, int N, int ngreek, const double* heights,
                                    const double* deltau_in, const double* omega_in, const double* greek_in,
                                    double albedo, double sza, int nvza, const double* vza, int nraa,
                                    const double* raa, double* out, int* nfourier_out) {
  return oracle_vlidort_solve_brdf(o, L, N, ngreek, heights, deltau_in, omega_in, greek_in, albedo, sza, nvza, vza,
                                   nraa, raa, nullptr, nullptr, nullptr, nullptr, nullptr, out, nfourier_out);
}

extern "C" void oracle_set_asymtx_tol(double tol) { g_asymtx_tol = tol; }
extern "C" double oracle_get_asymtx_tol() { return g_asymtx_tol; }

// Threads of the OpenMP loop over pixels (n <= 0: every host core).
extern "C" void oracle_set_threads(int n) { omp_set_num_threads(n > 0 ? n : omp_get_num_procs()); }

extern "C" int oracle_scalar_lambert(int km, int nch, int nobs, const double* channels, int nstreams,
                                     int plane_parallel, int nMom, int nPol, const double* ROT,
                                     const double* depol, const double* tau, const double* ssa,
                                     const double* g, const double* pmom, const double* pe, const double* he,
                                     const double* te, const double* albedo, const double* solar_zenith,
                                     const double* relat_azymuth, const double* sensor_zenith, double MISSING,
                                     int verbose, double* radiance, double* reflectance, int* nfourier,
                                     int* status, const int* nlay) {
  (void)channels; (void)nPol; (void)pe; (void)te; (void)verbose; (void)g;
  // VLIDORT_Init error checks (VLIDORT_Mod.F90:365-374): MAXSTREAMS=25, MAXLAYERS=72
  if (nstreams > 25) return 2;
  if (km > 72) return 3;
  if (nMom > 1000) return 5;
  auto is_missing = [&](double x) { return std::fabs(x / MISSING - 1.0) < 0.001; };
  // sticky DO_FOCORR_NADIR (VLIDORT_ScatMod.F90:1123-1126): set by the first call that reaches
  // Run_Scalar with solar_zenith == 0 and stays set for every later call of the loop
  std::vector<char> nadir(nobs, 0);
  {
    bool flag = false;
    for (int j = 0; j < nobs; ++j) {
      bool geo_ok = !(is_missing(solar_zenith[j]) || is_missing(sensor_zenith[j]) || is_missing(relat_azymuth[j]));
      if (geo_ok && solar_zenith[j] == 0.0) {
        for (int i = 0; i < nch; ++i)
          if (!is_missing(albedo[j + nobs * i])) { flag = true; break; }
      }
      nadir[j] = flag;
    }
  }
  const double pi_sp = (double)(4.0f * std::atan(1.0f));  // single-precision pi (ScatMod :1036)
  const double height_scale = (double)1.0e-3f;           // ze * 1.E-3 (ScatMod :1128)
  const double ssa_cap = (double)0.99999f;                // ScatMod :1169
#pragma omp parallel for schedule(dynamic, 1)
  for (int p = 0; p < nobs * nch; ++p) {
    int j = p / nch, i = p % nch;
    size_t o = (size_t)j + (size_t)nobs * i;
    if (nfourier) nfourier[o] = -1;
    if (status) status[o] = 0;
    if (is_missing(solar_zenith[j]) || is_missing(sensor_zenith[j]) || is_missing(relat_azymuth[j]) ||
        is_missing(albedo[o])) {
      radiance[o] = MISSING; reflectance[o] = MISSING;
      continue;
    }
    const int L = nlay ? nlay[j] : km;  // column uses its first L layers (extension for ragged batches)
    std::vector<double> dt(L), om(L), gr((size_t)(nMom + 1) * L, 0.0), hg(L + 1);
    const double dep = depol[i];
    const double raysmom2 = (1.0 - dep) / (2.0 + dep);
    for (int k = 0; k < L; ++k) {
      double ray_l = ROT[k + (size_t)km * (j + (size_t)nobs * i)];
      size_t a = k + (size_t)km * (i + (size_t)nch * j);
      double tau_l = tau[a], ssa_l = ssa[a];
      double tau_ext = 0.0 + ray_l + tau_l;
      double tau_scat = ray_l + ssa_l * tau_l;
      double ssa_tot = tau_scat / tau_ext;
      if (ssa_tot > ssa_cap) ssa_tot = ssa_cap;
      dt[k] = tau_ext; om[k] = ssa_tot;
      double aerswt = ssa_l * tau_l / tau_scat;
      double rayswt = ray_l / tau_scat;
      size_t nk = (size_t)km * nch * nobs;
      auto aersmom = [&](int l) { return l < nMom ? pmom[a + nk * (size_t)l] : 0.0; };
      double* G = &gr[(size_t)(nMom + 1) * k];
      G[0] = 1.0;
      G[1] = aersmom(1) * aerswt;
      G[2] = raysmom2 * rayswt + aersmom(2) * aerswt;
      for (int l = 3; l <= nMom; ++l) G[l] = aersmom(l) * aerswt;
    }
    for (int k = 0; k <= L; ++k) hg[k] = he[k + (size_t)(km + 1) * j] * height_scale;
    OracleOpts op;
    op.do_focorr = 1;
    op.do_focorr_nadir = nadir[j] ? 1 : 0;
    op.do_focorr_outgoing = nadir[j] ? 0 : 1;
    op.do_deltam = 1;
    op.do_plane_parallel = plane_parallel;
    op.do_double_convtest = 1;
    op.nfinelayers = 3;
    op.taylor_order = 3;
    op.accuracy = (double)0.0001f;  // VLIDORT_Mod.F90: VLIDORT_ACCURACY = 0.0001 (REAL literal)
    op.asymtx_tol = g_asymtx_tol;
    op.earth_radius = 6371.0;
    op.flux_factor = 1.0;
    double sza = solar_zenith[j], vz = sensor_zenith[j], az = relat_azymuth[j], rad = 0.0;
    int nf = -1;
    int rc = oracle_vlidort_solve(&op, L, nstreams, nMom, hg.data(), dt.data(), om.data(), gr.data(),
                                  albedo[o], sza, 1, &vz, 1, &az, &rad, &nf);
    if (nfourier) nfourier[o] = nf;
    if (status) status[o] = rc;
    if (rc != 0) { radiance[o] = MISSING; reflectance[o] = MISSING; continue; }
    radiance[o] = rad;
    reflectance[o] = (pi_sp * rad) / (std::cos(sza * pi_sp / 180.0) * 1.0);
  }
  return 0;
}

// VLIDORT_Scalar_LandMODIS (geo_vlidort/VLIDORT_BRDF_MODIS.F90:34-200): the
// scalar solve of VLIDORT_Scalar_Lambert (same layer mixing and
// VLIDORT_Init settings) over the MODIS RTLS surface of
// VLIDORT_LANDMODIS_SingleGeom (VLIDORT_SurfaceMod.F90:1376-1596):
// kernel_wt(3, nch, nobs) = (fiso, fgeo, fvol) on the Lambertian, Li-sparse
// and Ross-thick kernels, param(2, nch, nobs) = Li-sparse (h/b, b/r), 50
// azimuth streams, observation geometry.  BR(nobs, nch) is the exact
// direct-bounce BRDF (BS_DBOUNCE_BRDFUNC); a negative one gives -500 in the
// three outputs and skips the solve (:168-174).  The reference's checks of
// MISSING kernel weights and parameters (:136-149) end with a CYCLE of their
// own inner loop, so they never skip a pixel: restated as no check.  Pixels
// with MISSING angles get MISSING radiance, reflectance and BR.
extern "C" int oracle_scalar_landmodis(int km, int nch, int nobs, const double* channels, int nstreams,
                                       int plane_parallel, int nMom, int nPol, const double* ROT,
                                       const double* depol, const double* tau, const double* ssa, const double* g,
                                       const double* pmom, const double* pe, const double* he, const double* te,
                                       const double* kernel_wt, const double* param, const double* solar_zenith,
                                       const double* relat_azymuth, const double* sensor_zenith, double MISSING,
                                       int verbose, double* radiance, double* reflectance, double* BR,
                                       int* nfourier, int* status, const int* nlay) {
  (void)channels; (void)nPol; (void)pe; (void)te; (void)verbose; (void)g;
  if (nstreams > 25) return 2;
  if (km > 72) return 3;
  if (nMom > 1000) return 5;
  auto is_missing = [&](double x) { return std::fabs(x / MISSING - 1.0) < 0.001; };
  auto geo_ok = [&](int j) {
    return !(is_missing(solar_zenith[j]) || is_missing(sensor_zenith[j]) || is_missing(relat_azymuth[j]));
  };
  auto kernels = [&](int j, int i, int* which, double* fac, double* pars) {
    const size_t w = 3 * ((size_t)i + (size_t)nch * j), q = 2 * ((size_t)i + (size_t)nch * j);
    // kernel_wt = (fiso, fgeo, fvol) (VLIDORT_BRDF_MODIS.F90:152-156 into
    // VLIDORT_LANDMODIS(..., fiso, fgeo, fvol, ...)); the supplement sums the
    // kernels as Lambertian (fiso), Ross-thick (fvol), Li-sparse (fgeo)
    which[0] = 1; which[1] = 3; which[2] = 4;
    fac[0] = kernel_wt[w]; fac[1] = kernel_wt[w + 2]; fac[2] = kernel_wt[w + 1];
    for (int n = 0; n < 9; ++n) pars[n] = 0.0;
    pars[6] = param[q]; pars[7] = param[q + 1];
  };
  // exact direct-bounce BRDF of every (pixel, channel) first: it decides
  // which calls reach Run_Scalar, hence the sticky nadir FO flag
  for (int j = 0; j < nobs; ++j)
    for (int i = 0; i < nch; ++i) {
      const size_t o = (size_t)j + (size_t)nobs * i;
      if (!geo_ok(j)) { BR[o] = MISSING; continue; }
      int which[3]; double fac[3], pars[9];
      kernels(j, i, which, fac, pars);
      const double mu0 = std::cos(solar_zenith[j] * DTR), mu = std::cos(sensor_zenith[j] * DTR);
      const double phi = relat_azymuth[j] * DTR;
      double br = 0.0;
      for (int n = 0; n < 3; ++n)
        br += fac[n] * brdf_kernel(which[n], &pars[3 * n], mu0, std::sqrt(1.0 - mu0 * mu0), mu,
                                   std::sqrt(1.0 - mu * mu), std::cos(phi), std::sin(phi));
      BR[o] = br;
    }
  std::vector<char> nadir(nobs, 0);
  {
    bool flag = false;
    for (int j = 0; j < nobs; ++j) {
      if (geo_ok(j) && solar_zenith[j] == 0.0)
        for (int i = 0; i < nch; ++i)
          if (!(BR[(size_t)j + (size_t)nobs * i] < 0.0)) { flag = true; break; }
      nadir[j] = flag;
    }
  }
  const double pi_sp = (double)(4.0f * std::atan(1.0f));
  const double height_scale = (double)1.0e-3f;
  const double ssa_cap = (double)0.99999f;
  const int NMOM = 2 * nstreams - 1;
#pragma omp parallel for schedule(dynamic, 1)
  for (int p = 0; p < nobs * nch; ++p) {
    int j = p / nch, i = p % nch;
    size_t o = (size_t)j + (size_t)nobs * i;
    if (nfourier) nfourier[o] = -1;
    if (status) status[o] = 0;
    if (!geo_ok(j)) { radiance[o] = MISSING; reflectance[o] = MISSING; continue; }
    if (BR[o] < 0.0) { radiance[o] = -500.0; reflectance[o] = -500.0; BR[o] = -500.0; continue; }
    const int L = nlay ? nlay[j] : km;
    std::vector<double> dt(L), om(L), gr((size_t)(nMom + 1) * L, 0.0), hg(L + 1);
    const double dep = depol[i];
    const double raysmom2 = (1.0 - dep) / (2.0 + dep);
    for (int k = 0; k < L; ++k) {
      double ray_l = ROT[k + (size_t)km * (j + (size_t)nobs * i)];
      size_t a = k + (size_t)km * (i + (size_t)nch * j);
      double tau_l = tau[a], ssa_l = ssa[a];
      double tau_ext = 0.0 + ray_l + tau_l;
      double tau_scat = ray_l + ssa_l * tau_l;
      double ssa_tot = tau_scat / tau_ext;
      if (ssa_tot > ssa_cap) ssa_tot = ssa_cap;
      dt[k] = tau_ext; om[k] = ssa_tot;
      double aerswt = ssa_l * tau_l / tau_scat;
      double rayswt = ray_l / tau_scat;
      size_t nk = (size_t)km * nch * nobs;
      auto aersmom = [&](int l) { return l < nMom ? pmom[a + nk * (size_t)l] : 0.0; };
      double* G = &gr[(size_t)(nMom + 1) * k];
      G[0] = 1.0;
      G[1] = aersmom(1) * aerswt;
      G[2] = raysmom2 * rayswt + aersmom(2) * aerswt;
      for (int l = 3; l <= nMom; ++l) G[l] = aersmom(l) * aerswt;
    }
    for (int k = 0; k <= L; ++k) hg[k] = he[k + (size_t)(km + 1) * j] * height_scale;
    OracleOpts op;
    op.do_focorr = 1;
    op.do_focorr_nadir = nadir[j] ? 1 : 0;
    op.do_focorr_outgoing = nadir[j] ? 0 : 1;
    op.do_deltam = 1;
    op.do_plane_parallel = plane_parallel;
    op.do_double_convtest = 1;
    op.nfinelayers = 3;
    op.taylor_order = 3;
    op.accuracy = (double)0.0001f;
    op.asymtx_tol = g_asymtx_tol;
    op.earth_radius = 6371.0;
    op.flux_factor = 1.0;
    double sza = solar_zenith[j], vz = sensor_zenith[j], az = relat_azymuth[j], rad = 0.0;
    int which[3]; double fac[3], pars[9];
    kernels(j, i, which, fac, pars);
    const int N = nstreams, M1 = NMOM + 1;
    std::vector<double> bf((size_t)M1 * N * N), bf0((size_t)M1 * N), buf((size_t)M1 * N), buf0(M1), bex(1);
    oracle_brdf_supplement(3, which, fac, pars, 0, 50, N, NMOM, sza, 1, &vz, 1, &az, bf.data(), bf0.data(),
                           buf.data(), buf0.data(), bex.data());
    int nf = -1;
    int rc = oracle_vlidort_solve_brdf(&op, L, nstreams, nMom, hg.data(), dt.data(), om.data(), gr.data(), 0.0, sza,
                                       1, &vz, 1, &az, bf.data(), bf0.data(), buf.data(), buf0.data(), bex.data(),
                                       &rad, &nf);
    if (nfourier) nfourier[o] = nf;
    if (status) status[o] = rc;
    if (rc != 0) { radiance[o] = MISSING; reflectance[o] = MISSING; continue; }
    radiance[o] = rad;
    reflectance[o] = (pi_sp * rad) / (std::cos(sza * pi_sp / 180.0) * 1.0);
  }
  return 0;
}

// VLIDORT_Scalar_CX (geo_vlidort/VLIDORT_BRDF_CX.F90:420-584): the scalar
// solve of VLIDORT_Scalar_Lambert (same layer mixing and VLIDORT_Init
// settings) over the Cox-Munk glint surface of VLIDORT_CoxMunk_SingleGeom
// (VLIDORT_SurfaceMod.F90:816-1042): one Cox-Munk kernel (factor 1) with
// shadowing, slope variance sigma2 = 0.003 + 0.00512 W from the wind speed
// W = |(U10m, V10m)| clamped to [0, 50] m/s (:893-898), refractive index
// squared mr(ch)^2, 100 azimuth streams, observation geometry.  BR(nobs, nch)
// is the exact direct-bounce BRDF (BS_DBOUNCE_BRDFUNC).  Pixels with MISSING
// angles, and channels with a MISSING wind component or refractive index,
// get MISSING radiance and reflectance (the reference leaves its BRDF output
// unset there; here it is MISSING too).
// VLIDORT_Scalar_GissCX (VLIDORT_BRDF_CX.F90:1553-1716) is the same wrapper
// over the GISS Cox-Munk kernel of VLIDORT_GissCoxMunk_SingleGeom
// (VLIDORT_SurfaceMod.F90:586-814): index 10, parameters (sigma2 / 2, mr(ch),
// shadowing) (:680-697); `giss` selects it.
static int scalar_cx_impl(int giss, int km, int nch, int nobs, const double* channels, int nstreams,
                          int plane_parallel, int nMom, int nPol, const double* ROT, const double* depol,
                          const double* tau, const double* ssa, const double* g, const double* pmom, const double* pe,
                          const double* he, const double* te, const double* U10m, const double* V10m, const double* mr,
                          const double* solar_zenith, const double* relat_azymuth, const double* sensor_zenith,
                          double MISSING, int verbose, double* radiance, double* reflectance, double* BR,
                          int* nfourier, int* status, const int* nlay) {
  (void)channels; (void)nPol; (void)pe; (void)te; (void)verbose; (void)g;
  if (nstreams > 25) return 2;
  if (km > 72) return 3;
  if (nMom > 1000) return 5;
  auto is_missing = [&](double x) { return std::fabs(x / MISSING - 1.0) < 0.001; };
  auto geo_ok = [&](int j) {
    return !(is_missing(solar_zenith[j]) || is_missing(sensor_zenith[j]) || is_missing(relat_azymuth[j]));
  };
  auto surf_ok = [&](int j, int i) { return !(is_missing(U10m[j]) || is_missing(V10m[j]) || is_missing(mr[i])); };
  auto kernel = [&](int j, int i, double* pars) {
    double w = std::sqrt(U10m[j] * U10m[j] + V10m[j] * V10m[j]);
    if (w < 0.0) w = 0.0;
    if (w > 50.0) w = 50.0;
    const double sigma2 = 0.003 + 0.00512 * w;
    pars[0] = giss ? 0.5 * sigma2 : sigma2;
    pars[1] = giss ? mr[i] : mr[i] * mr[i];
    pars[2] = 1.0;  // shadowing
  };
  const int which = giss ? 10 : 9;
  for (int j = 0; j < nobs; ++j)
    for (int i = 0; i < nch; ++i) {
      const size_t o = (size_t)j + (size_t)nobs * i;
      if (!geo_ok(j) || !surf_ok(j, i)) { BR[o] = MISSING; continue; }
      double pars[3];
      kernel(j, i, pars);
      const double mu0 = std::cos(solar_zenith[j] * DTR), mu = std::cos(sensor_zenith[j] * DTR);
      const double phi = relat_azymuth[j] * DTR;
      BR[o] = brdf_kernel(which, pars, mu0, std::sqrt(1.0 - mu0 * mu0), mu, std::sqrt(1.0 - mu * mu),
                          std::cos(phi), std::sin(phi));
    }
  // the sticky nadir FO flag: set by the first Run_Scalar call at SZA = 0
  std::vector<char> nadir(nobs, 0);
  {
    bool flag = false;
    for (int j = 0; j < nobs; ++j) {
      if (geo_ok(j) && solar_zenith[j] == 0.0)
        for (int i = 0; i < nch; ++i)
          if (surf_ok(j, i)) { flag = true; break; }
      nadir[j] = flag;
    }
  }
  const double pi_sp = (double)(4.0f * std::atan(1.0f));
  const double height_scale = (double)1.0e-3f;
  const double ssa_cap = (double)0.99999f;
  const int NMOM = 2 * nstreams - 1;
#pragma omp parallel for schedule(dynamic, 1)
  for (int p = 0; p < nobs * nch; ++p) {
    int j = p / nch, i = p % nch;
    size_t o = (size_t)j + (size_t)nobs * i;
    if (nfourier) nfourier[o] = -1;
    if (status) status[o] = 0;
    if (!geo_ok(j) || !surf_ok(j, i)) { radiance[o] = MISSING; reflectance[o] = MISSING; continue; }
    const int L = nlay ? nlay[j] : km;
    std::vector<double> dt(L), om(L), gr((size_t)(nMom + 1) * L, 0.0), hg(L + 1);
    const double dep = depol[i];
    const double raysmom2 = (1.0 - dep) / (2.0 + dep);
    for (int k = 0; k < L; ++k) {
      double ray_l = ROT[k + (size_t)km * (j + (size_t)nobs * i)];
      size_t a = k + (size_t)km * (i + (size_t)nch * j);
      double tau_l = tau[a], ssa_l = ssa[a];
      double tau_ext = 0.0 + ray_l + tau_l;
      double tau_scat = ray_l + ssa_l * tau_l;
      double ssa_tot = tau_scat / tau_ext;
      if (ssa_tot > ssa_cap) ssa_tot = ssa_cap;
      dt[k] = tau_ext; om[k] = ssa_tot;
      double aerswt = ssa_l * tau_l / tau_scat;
      double rayswt = ray_l / tau_scat;
      size_t nk = (size_t)km * nch * nobs;
      auto aersmom = [&](int l) { return l < nMom ? pmom[a + nk * (size_t)l] : 0.0; };
      double* G = &gr[(size_t)(nMom + 1) * k];
      G[0] = 1.0;
      G[1] = aersmom(1) * aerswt;
      G[2] = raysmom2 * rayswt + aersmom(2) * aerswt;
      for (int l = 3; l <= nMom; ++l) G[l] = aersmom(l) * aerswt;
    }
    for (int k = 0; k <= L; ++k) hg[k] = he[k + (size_t)(km + 1) * j] * height_scale;
    OracleOpts op;
    op.do_focorr = 1;
    op.do_focorr_nadir = nadir[j] ? 1 : 0;
    op.do_focorr_outgoing = nadir[j] ? 0 : 1;
    op.do_deltam = 1;
    op.do_plane_parallel = plane_parallel;
    op.do_double_convtest = 1;
    op.nfinelayers = 3;
    op.taylor_order = 3;
    op.accuracy = (double)0.0001f;
    op.asymtx_tol = g_asymtx_tol;
    op.earth_radius = 6371.0;
    op.flux_factor = 1.0;
    double sza = solar_zenith[j], vz = sensor_zenith[j], az = relat_azymuth[j], rad = 0.0;
    const double fac = 1.0;
    double pars[3];
    kernel(j, i, pars);
    const int N = nstreams, M1 = NMOM + 1;
    std::vector<double> bf((size_t)M1 * N * N), bf0((size_t)M1 * N), buf((size_t)M1 * N), buf0(M1), bex(1);
    oracle_brdf_supplement(1, &which, &fac, pars, 1, 100, N, NMOM, sza, 1, &vz, 1, &az, bf.data(), bf0.data(),
                           buf.data(), buf0.data(), bex.data());
    int nf = -1;
    int rc = oracle_vlidort_solve_brdf(&op, L, nstreams, nMom, hg.data(), dt.data(), om.data(), gr.data(), 0.0, sza,
                                       1, &vz, 1, &az, bf.data(), bf0.data(), buf.data(), buf0.data(), bex.data(),
                                       &rad, &nf);
    if (nfourier) nfourier[o] = nf;
    if (status) status[o] = rc;
    if (rc != 0) { radiance[o] = MISSING; reflectance[o] = MISSING; continue; }
    radiance[o] = rad;
    reflectance[o] = (pi_sp * rad) / (std::cos(sza * pi_sp / 180.0) * 1.0);
  }
  return 0;
}

extern "C" int oracle_scalar_cx(int km, int nch, int nobs, const double* channels, int nstreams, int plane_parallel,
                                int nMom, int nPol, const double* ROT, const double* depol, const double* tau,
                                const double* ssa, const double* g, const double* pmom, const double* pe,
                                const double* he, const double* te, const double* U10m, const double* V10m,
                                const double* mr, const double* solar_zenith, const double* relat_azymuth,
                                const double* sensor_zenith, double MISSING, int verbose, double* radiance,
                                double* reflectance, double* BR, int* nfourier, int* status, const int* nlay) {
  return scalar_cx_impl(0, km, nch, nobs, channels, nstreams, plane_parallel, nMom, nPol, ROT, depol, tau, ssa, g,
                        pmom, pe, he, te, U10m, V10m, mr, solar_zenith, relat_azymuth, sensor_zenith, MISSING,
                        verbose, radiance, reflectance, BR, nfourier, status, nlay);
}

extern "C" int oracle_scalar_gisscx(int km, int nch, int nobs, const double* channels, int nstreams,
                                    int plane_parallel, int nMom, int nPol, const double* ROT, const double* depol,
                                    const double* tau, const double* ssa, const double* g, const double* pmom,
                                    const double* pe, const double* he, const double* te, const double* U10m,
                                    const double* V10m, const double* mr, const double* solar_zenith,
                                    const double* relat_azymuth, const double* sensor_zenith, double MISSING,
                                    int verbose, double* radiance, double* reflectance, double* BR, int* nfourier,
                                    int* status, const int* nlay) {
  return scalar_cx_impl(1, km, nch, nobs, channels, nstreams, plane_parallel, nMom, nPol, ROT, depol, tau, ssa, g,
                        pmom, pe, he, te, U10m, V10m, mr, solar_zenith, relat_azymuth, sensor_zenith, MISSING,
                        verbose, radiance, reflectance, BR, nfourier, status, nlay);
}
