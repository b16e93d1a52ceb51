// Team-cooperative Fourier series: the 32 lanes of one warp run the Fourier
// series of one solve together, with the layer matrices in shared memory.
//
// Why: the thread-per-solve series keeps ~15 N^2 values per solve live (layer
// eigen-solution, two layer solutions, the 2N x 2N interface system); at 12-16
// streams that is 20-45 KB per thread, far beyond what an SM can hold for the
// thread count that hides FP64 latency, so the working set streams from L2 or
// HBM.  With one solve per warp the same working set (per solve) sits in
// shared memory, and every step is parallel over matrix elements, matrix rows,
// eigenvectors or Jacobi rotation pairs, so the FP64/FP32 pipes stay busy with
// a handful of warps per SM.  The arithmetic is that of rt_solve.cuh (same
// formulation, same pivot choices); only the schedule over lanes differs.
//
// The per-solve set-up (layer mixing, delta-M, single scatter, beam
// attenuation) stays thread-per-solve (solve_setup); its per-layer outputs are
// read from the set-up thread's scratch.
#pragma once
#include "rt_solve.cuh"

namespace aerort {

constexpr int kTeam = 32;

// Lane index and warp barrier of a team.  On the host (the CPU test harness
// runs one std::thread per lane) the barrier and the lane exchange go through
// a callback and shared memory.
struct Team {
  int lane;
  void (*host_sync)(void*);
  void* host_arg;
  RT_HD void sync() const {
#ifdef __CUDA_ARCH__
    __syncwarp();
#else
    host_sync(host_arg);
#endif
  }
};

// Sum of v over aligned groups of G lanes (G a power of two); every lane of a
// group gets the group's sum.  red: kTeam scratch values in shared memory.
template <int G, typename T>
RT_HD T group_sum(const Team& tm, T v, T* red) {
#ifdef __CUDA_ARCH__
  (void)red;
  for (int o = 1; o < G; o <<= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
#else
  red[tm.lane] = v;
  tm.sync();
  T s = 0;
  const int b = tm.lane & ~(G - 1);
  for (int k = 0; k < G; ++k) s += red[b + k];
  tm.sync();
  return s;
#endif
}

// Whether the team splits its per-row and per-eigenvector sums (particular
// solution, user-angle solutions) across both half-warps, two lanes per row.
// Measured on GB300: faster in FP64 (4%) and for the 16-stream FP32 kernel
// (6%), slower for the 12-stream FP32 kernel (17%).
template <int NS, typename T>
constexpr bool kTeamSplitSums = sizeof(T) == sizeof(double) || NS >= 16;

// v of this lane plus v of lane + h (lanes < h get the sum of the pair; the
// others keep their own v).  Every lane must call it.
template <typename T>
RT_HD T pair_sum(const Team& tm, T v, int h, T* red) {
#ifdef __CUDA_ARCH__
  (void)red;
  return v + __shfl_down_sync(0xffffffffu, v, h);
#else
  red[tm.lane] = v;
  tm.sync();
  const T r = (tm.lane + h < kTeam) ? v + red[tm.lane + h] : v;
  tm.sync();
  return r;
#endif
}

// Whether pred holds on any lane (every lane gets the answer).
RT_HD bool team_any(const Team& tm, bool pred, int* flag) {
#ifdef __CUDA_ARCH__
  (void)flag;
  return __any_sync(0xffffffffu, pred) != 0;
#else
  if (tm.lane == 0) *flag = 0;
  tm.sync();
  if (pred) *flag = 1;
  tm.sync();
  bool r = *flag != 0;
  tm.sync();
  return r;
#endif
}

// Lane holding the largest v, the lowest lane among equals (the first maximum
// of a serial scan when the candidates sit on lanes in index order); every
// lane gets it and *vmax.  v >= 0 on lanes with a candidate, v < 0 elsewhere.
// On the device, non-negative floats order as their bit patterns, so the
// maximum is one warp reduction (two for FP64: high word, then low word).
template <typename T>
RT_HD int team_argmax_lane(const Team& tm, T v, T* red, T* vmax) {
#ifdef __CUDA_ARCH__
  (void)red;
  const unsigned full = 0xffffffffu;
  if constexpr (sizeof(T) == sizeof(float)) {
    const unsigned key = (v >= (T)0) ? __float_as_uint(v) : 0u;
    const unsigned mx = __reduce_max_sync(full, key);
    const int src = __ffs(__ballot_sync(full, key == mx)) - 1;
    *vmax = __uint_as_float(mx);
    return src;
  } else {
    const unsigned hi = (v >= (T)0) ? (unsigned)__double2hiint(v) : 0u;
    const unsigned lo = (v >= (T)0) ? (unsigned)__double2loint(v) : 0u;
    const unsigned mh = __reduce_max_sync(full, hi);
    const unsigned cand = __ballot_sync(full, hi == mh);
    unsigned ml = 0;
    if (cand & (1u << tm.lane)) ml = __reduce_max_sync(cand, lo);
    ml = __shfl_sync(full, ml, __ffs(cand) - 1);
    const int src = __ffs(__ballot_sync(full, hi == mh && lo == ml)) - 1;
    *vmax = __hiloint2double((int)mh, (int)ml);
    return src;
  }
#else
  red[tm.lane] = v;
  tm.sync();
  T bv = red[0];
  int bi = 0;
  for (int k = 1; k < kTeam; ++k)
    if (red[k] > bv) { bv = red[k]; bi = k; }
  tm.sync();
  *vmax = bv < (T)0 ? (T)0 : bv;
  return bi;
#endif
}

// Shared-memory working set of one team.  The layer matrices are
// column-major with a padded leading dimension (LD = N + 1) so that lanes
// working on different columns hit different banks.  The interface systems
// are row-major, [A | pad | B] per row with a row stride of LR words: a lane
// owns a row in the elimination and moves it 16 bytes at a time; LR is an
// odd number of 16-byte units, so 8 lanes' 16-byte accesses at the same
// column fall in 8 different bank groups.
template <int NS, typename T>
struct TeamMem {
  static constexpr int LD = NS + 1;
  static constexpr int V = 16 / (int)sizeof(T);                  // words per 16 bytes
  static constexpr int LRQ = (3 * NS + 1 + V - 1) / V;           // 16-byte units for 2N + (N + 1) columns
  static constexpr int LR = (LRQ % 2 == 1 ? LRQ : LRQ + 1) * V;  // row stride of the interface systems
  // eigen phase: Sp, Bs, H, G, V (N x LD each); interface: 2N rows of LR
  static constexpr int NWORK = (5 * NS * LD > 2 * NS * LR) ? 5 * NS * LD : 2 * NS * LR;
  T piq[NS][2 * NS + 1];             // P~_l^m at the quadrature cosines (row padded against bank conflicts)
  T piu[2 * NS], pi0[2 * NS];        // at the user and solar cosines
  T pimq[NS], pimu, pim0;            // P~_m^m carried across terms
  T lra[2 * NS], lrb[2 * NS], lr1;   // Legendre recurrence coefficients of term m
  T og[2 * NS];                      // omega * beta_l of the current layer
  T lsc[8];                          // dtau, 1 - omega, tuser, secbar, itrans, tmubar, emult, lnz
  alignas(16) T work[NWORK];         // eigen phase: Sp Bs H G V | interface system
  T kv[NS], norm[NS], uhd[NS], uhu[NS], hm1[NS], hm2[NS], gup[NS], gdn[NS], dpi[NS], dmi[NS], rv[NS];
  T rbeta;
  T la[NS], lb[NS], ls;              // source coefficients a, b, s of the current layer
  T adj[NS];                         // TOA source per unit of the current layer's M (adjoint of the sweep)
  T P[2][NS * LD], Q[2][NS * LD];    // layer solutions (prev / cur)
  T t[2][NS], wt[2][2 * NS], wb[2][2 * NS];
  T F[NS * LD], f[NS];               // L = F M + f of the current interface
  T Vp[NS * LD];                     // previous layer's Jacobi rotations (warm start)
  T cqx[NS], cqw[NS], csqw[NS], csin[NS];  // quadrature cosines, weights, sqrt(weights), sines
  int vp_valid;
  T red[2 * kTeam];
  int flag;
};

// ---------------------------------------------------------------------------------- dense steps
// Cholesky A = L L^T (lower triangle, leading dimension LDA, n <= 32),
// right-looking; lane r owns row r of the trailing update (the column below
// the pivot is a shared-memory broadcast).  Returns false (on every lane) if a
// pivot is not positive.
template <int LDA, typename T>
RT_HD bool team_cholesky(const Team& tm, int n, T* A) {
  const int r = tm.lane;
  for (int j = 0; j < n; ++j) {
    const T d = A[j + LDA * j];
    if (!(d > (T)0)) return false;
    const T ljj = sqrt(d), inv = (T)1 / ljj;
    tm.sync();
    if (r == 0) A[j + LDA * j] = ljj;
    if (r > j && r < n) A[r + LDA * j] *= inv;
    tm.sync();
    if (r > j && r < n) {
      const T lrj = A[r + LDA * j];
      for (int k = j + 1; k <= r; ++k) A[r + LDA * k] -= lrj * A[k + LDA * j];
    }
    tm.sync();
  }
  return true;
}

// y[0..V) -= a x[0..V) for the 16 bytes at y and x (both 16-byte aligned).
template <typename T>
RT_HD void axpy16(T* y, const T* x, T a) {
#ifdef __CUDA_ARCH__
  if constexpr (sizeof(T) == sizeof(float)) {
    const float4 xv = *reinterpret_cast<const float4*>(x);
    float4 yv = *reinterpret_cast<float4*>(y);
    yv.x -= a * xv.x; yv.y -= a * xv.y; yv.z -= a * xv.z; yv.w -= a * xv.w;
    *reinterpret_cast<float4*>(y) = yv;
  } else {
    const double2 xv = *reinterpret_cast<const double2*>(x);
    double2 yv = *reinterpret_cast<double2*>(y);
    yv.x -= a * xv.x; yv.y -= a * xv.y;
    *reinterpret_cast<double2*>(y) = yv;
  }
#else
  for (int v = 0; v < 16 / (int)sizeof(T); ++v) y[v] -= a * x[v];
#endif
}

// First column of the right-hand sides of an n-row interface system.
RT_HD int rhs_col(int n) { return (n + 3) & ~3; }

// Solution of A X = B by Gaussian elimination with partial pivoting, n <= 32
// rows.  Row r of the system is S[r * LR ...]: A in columns 0..n-1, B in
// columns rhs_col(n).. (nrhs of them); X overwrites B.  Pivots and the
// arithmetic on every element of U and B as lu_solve.  Lane r owns row r: its
// multiplier stays in a register and the pivot row is a broadcast.  A row is
// updated 16 bytes at a time from the 16-byte boundary at or below the pivot
// column; the entries this also touches (the eliminated column, the padding)
// are not read again, since the solve needs no L.
template <int LR, typename T>
RT_HD bool team_lu_solve(const Team& tm, int n, T* S, int nrhs, T* red) {
  constexpr int V = 16 / (int)sizeof(T);
  const int r = tm.lane, nb = rhs_col(n), ncol = nb + nrhs;
  T* row = S + LR * r;
  for (int k = 0; k < n; ++k) {
    T vmax;
    const int piv = team_argmax_lane(tm, (r >= k && r < n) ? fabs(row[k]) : (T)-1, red, &vmax);
    if (vmax == (T)0) return false;
    if (piv != k) {
      for (int j = tm.lane; j < ncol; j += kTeam) {
        const T tmp = S[LR * k + j];
        S[LR * k + j] = S[LR * piv + j];
        S[LR * piv + j] = tmp;
      }
      tm.sync();
    }
    if (r > k && r < n) {
      const T* rk = S + LR * k;
      const T inv = (T)1 / rk[k];
      const T fm = row[k] * inv;
      for (int j = (k + 1) & ~(V - 1); j < ncol; j += V) axpy16(row + j, rk + j, fm);
    }
    tm.sync();
  }
  for (int i = n - 1; i >= 0; --i) {
    T* ri = S + LR * i;
    const T inv = (T)1 / ri[i];
    for (int j = tm.lane; j < nrhs; j += kTeam) ri[nb + j] *= inv;
    tm.sync();
    if (r < i) {
      const T a = row[i];
      for (int j = nb; j < ncol; j += V) axpy16(row + j, ri + j, a);
    }
    tm.sync();
  }
  return true;
}

// One-sided Jacobi on the columns of G (leading dimension LD) with rotations
// accumulated in V, in round-robin order: each round rotates n/2 disjoint
// column pairs at once, LPP lanes per pair.  sigma[a] = |G e_a| on return.
// warm = true: V already holds a starting rotation, applied to G by the caller.
template <int NS, int LD, typename T>
RT_HD bool team_jacobi(const Team& tm, int n, T* G, T* V, T* sigma, T* red, int* flag, bool warm = false) {
  constexpr int NP = NS / 2;
  constexpr int LPP = (kTeam / NP >= 16) ? 16 : (kTeam / NP >= 8) ? 8 : (kTeam / NP >= 4) ? 4 : 2;
  if (!warm)
    for (int e = tm.lane; e < n * n; e += kTeam) V[e % n + LD * (e / n)] = (e % n == e / n) ? (T)1 : (T)0;
  tm.sync();
  const int pr = tm.lane / LPP, sub = tm.lane % LPP;
  const bool act = pr < NP;
  const T tol = Eps<T>::v * (T)n;
  bool done = false;
  for (int sweep = 0; sweep < 30 && !done; ++sweep) {
    bool unconverged = false;  // see jacobi_svd
    for (int round = 0; round < n - 1; ++round) {
      int p = 0, q = 0;
      if (act) {
        p = (pr == 0) ? 0 : 1 + (pr - 1 + round) % (n - 1);
        q = 1 + (n - 2 - pr + round) % (n - 1);
        if (pr == 0) q = 1 + (n - 2 + round) % (n - 1);
      }
      T al = 0, be = 0, ga = 0;
      if (act)
        for (int i = sub; i < n; i += LPP) {
          const T gp = G[i + LD * p], gq = G[i + LD * q];
          al += gp * gp; be += gq * gq; ga += gp * gq;
        }
      al = group_sum<LPP>(tm, al, red);
      be = group_sum<LPP>(tm, be, red);
      ga = group_sum<LPP>(tm, ga, red);
      const Rotation<T> rot(al, be, ga, tol);
      if (act && rot.rotate) {
        unconverged = unconverged || rot.unconverged;
        const T cs = rot.cs, sn = rot.sn;
        for (int i = sub; i < n; i += LPP) {
          const T gp = G[i + LD * p], gq = G[i + LD * q];
          G[i + LD * p] = cs * gp - sn * gq;
          G[i + LD * q] = sn * gp + cs * gq;
          const T vp = V[i + LD * p], vq = V[i + LD * q];
          V[i + LD * p] = cs * vp - sn * vq;
          V[i + LD * q] = sn * vp + cs * vq;
        }
      }
      tm.sync();
    }
    done = !team_any(tm, unconverged, flag);
  }
  if (tm.lane < n) {
    T s = 0;
    for (int i = 0; i < n; ++i) s += G[i + LD * tm.lane] * G[i + LD * tm.lane];
    sigma[tm.lane] = sqrt(s);
  }
  tm.sync();
  return done;
}

// ---------------------------------------------------------------------------------- layer solution
// Legendre functions of term m at the N quadrature cosines (lanes 0..N-1), the
// user cosine (lane N) and the solar cosine (lane N+1).
template <int NS, typename T>
RT_HD void team_legendre(const Team& tm, TeamMem<NS, T>& M, const SolveCtx<NS, T>& c, int m) {
  const int NM = c.NM;
  for (int l = m + 2 + tm.lane; l <= NM; l += kTeam) {
    const T d = (T)1 / sqrt((T)(l * l - m * m));
    M.lra[l] = (T)(2 * l - 1) * d;
    M.lrb[l] = sqrt((T)((l - 1) * (l - 1) - m * m)) * d;
  }
  if (tm.lane == 0) M.lr1 = sqrt((T)(2 * m + 1));
  tm.sync();
  const int i = tm.lane;
  if (i < NS + 2) {
    T x, s, *pim, *out;
    if (i < NS) { x = M.cqx[i]; s = M.csin[i]; pim = &M.pimq[i]; out = M.piq[i]; }
    else if (i == NS) { x = c.mu_u; s = c.sin_u; pim = &M.pimu; out = M.piu; }
    else { x = c.cos_sza; s = c.sin_0; pim = &M.pim0; out = M.pi0; }
    for (int l = 0; l < m && l <= NM; ++l) out[l] = 0;
    if (m <= NM) {
      const T pmm = (m == 0) ? (T)1 : *pim * s * sqrt((T)(2 * m - 1) / (T)(2 * m));
      *pim = pmm;
      out[m] = pmm;
      if (m + 1 <= NM) out[m + 1] = x * M.lr1 * pmm;
      for (int l = m + 2; l <= NM; ++l) out[l] = M.lra[l] * x * out[l - 1] - M.lrb[l] * out[l - 2];
    }
  }
  tm.sync();
}

#ifdef __CUDA_ARCH__
// The moment contraction of team_layer_eigen on the tensor cores, for the FP32
// solve: mma.sync m16n8k8 with TF32 operands and FP32 accumulation, and the
// 3xTF32 split x = hi + lo (hi = x rounded to TF32, lo = the remainder rounded
// to TF32), x y ~ lo_x hi_y + hi_x lo_y + hi_x hi_y, which drops only lo_x lo_y
// (below 2^-22 |x y|).  Per k-step of 8 moments l: A (16 x 8) = og_l P_l(mu_i)
// for the rows i < N (zero above) and l of one parity (even, then odd l - m
// into a second accumulator), B (8 x 8 per tile of columns j) = P_l(mu_j).
// Fragments as the PTX ISA lays out m16n8k8 .tf32: lane = 4 g + t, A rows g
// and g + 8 at columns t and t + 4, B rows t and t + 4 at column g, D rows g
// and g + 8 at columns 2t and 2t + 1.  Writes the lower triangle of Sp
// (mirrored) and of Bs as the CUDA-core loop does.
__device__ __forceinline__ unsigned tf32_rna(float x) {
  unsigned r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return r;
}

__device__ __forceinline__ void tf32_split(float x, unsigned& hi, unsigned& lo) {
  hi = tf32_rna(x);
  lo = tf32_rna(x - __uint_as_float(hi));
}

__device__ __forceinline__ void mma_tf32_m16n8k8(float (&d)[4], const unsigned (&a)[4], unsigned b0, unsigned b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k8.row.col.f32.tf32.tf32.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

template <int NS>
__device__ void team_contract_tf32x3(const Team& tm, TeamMem<NS, float>& M, int m, int NM, float* Sp, float* Bs) {
  constexpr int LD = TeamMem<NS, float>::LD;
  constexpr int NT = (NS + 7) / 8;
  static_assert(NS <= 16, "one 16-row tile");
  const int g = tm.lane >> 2, t4 = tm.lane & 3;
  float ce[NT][4], co[NT][4];
#pragma unroll
  for (int jt = 0; jt < NT; ++jt)
#pragma unroll
    for (int r = 0; r < 4; ++r) { ce[jt][r] = 0.0f; co[jt][r] = 0.0f; }
  auto pq = [&](int i, int l) -> float { return (i < NS && l <= NM) ? M.piq[i][l] : 0.0f; };
  for (int l0 = m & ~7; l0 <= NM; l0 += 8) {
    const int la = l0 + t4, lb = la + 4;
    const float oa = (la >= m && la <= NM) ? M.og[la] : 0.0f;
    const float ob = (lb >= m && lb <= NM) ? M.og[lb] : 0.0f;
    const bool eva = ((la - m) & 1) == 0, evb = ((lb - m) & 1) == 0;
    const float x[4] = {oa * pq(g, la), oa * pq(g + 8, la), ob * pq(g, lb), ob * pq(g + 8, lb)};
    const bool ev[4] = {eva, eva, evb, evb};
    unsigned aeh[4], ael[4], aoh[4], aol[4];
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      tf32_split(ev[r] ? x[r] : 0.0f, aeh[r], ael[r]);
      tf32_split(ev[r] ? 0.0f : x[r], aoh[r], aol[r]);
    }
#pragma unroll
    for (int jt = 0; jt < NT; ++jt) {
      unsigned bh0, bl0, bh1, bl1;
      tf32_split(pq(8 * jt + g, la), bh0, bl0);
      tf32_split(pq(8 * jt + g, lb), bh1, bl1);
      mma_tf32_m16n8k8(ce[jt], ael, bh0, bh1);
      mma_tf32_m16n8k8(ce[jt], aeh, bl0, bl1);
      mma_tf32_m16n8k8(ce[jt], aeh, bh0, bh1);
      mma_tf32_m16n8k8(co[jt], aol, bh0, bh1);
      mma_tf32_m16n8k8(co[jt], aoh, bl0, bl1);
      mma_tf32_m16n8k8(co[jt], aoh, bh0, bh1);
    }
  }
#pragma unroll
  for (int jt = 0; jt < NT; ++jt)
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      const int i = g + (r >= 2 ? 8 : 0), j = 8 * jt + 2 * t4 + (r & 1);
      if (i < NS && j <= i) {
        Sp[i + LD * j] = ce[jt][r];
        Sp[j + LD * i] = ce[jt][r];
        float b = -M.csqw[i] * M.csqw[j] * co[jt][r];
        if (i == j) b += 1.0f;
        Bs[i + LD * j] = b;
      }
    }
}
#endif

// P~_k^k, which team_legendre carries from term to term, advanced over the
// terms after `last` and before m (the same products in the same order), for
// a warp that runs only some of a solve's terms (k_refine_terms).
template <int NS, typename T>
RT_HD void team_skip_terms(const Team& tm, TeamMem<NS, T>& M, const SolveCtx<NS, T>& c, int last, int m) {
  const int i = tm.lane;
  if (i < NS + 2) {
    T s, *pim;
    if (i < NS) { s = M.csin[i]; pim = &M.pimq[i]; }
    else if (i == NS) { s = c.sin_u; pim = &M.pimu; }
    else { s = c.sin_0; pim = &M.pim0; }
    for (int k = last + 1; k < m; ++k)
      if (k <= c.NM) *pim = (k == 0) ? (T)1 : *pim * s * sqrt((T)(2 * k - 1) / (T)(2 * k));
  }
  tm.sync();
}

// Eigen-solution of layer n for term m into P/Q/t of slot `cur`, with the
// Green's-function norms and user-angle homogeneous solutions (layer_eigen).
// tc: the FP32 solve forms the moment contraction on the tensor cores
// (team_contract_tf32x3; device only).
template <int NS, typename T>
RT_HD int team_layer_eigen(const Team& tm, TeamMem<NS, T>& M, const SolveCtx<NS, T>& c, int m, int cur,
                           bool tc = false) {
  constexpr int LD = TeamMem<NS, T>::LD;
  const int N = NS, NM = c.NM;
  T* Sp = M.work;
  T* Bs = M.work + NS * LD;
  T* H = M.work + 2 * NS * LD;
  T* G = M.work + 3 * NS * LD;
  T* V = M.work + 4 * NS * LD;
  const T dtau = M.lsc[0], om1 = M.lsc[1];
  // Sp (even l-m) and Sm (odd l-m) contractions of omega*beta_l P_l(mu_i) P_l(mu_j),
  // symmetric: the lower triangle only (Sp mirrored; Bs is read below its
  // diagonal only).  Element e of the folded triangle: row pairs (r, N-1-r)
  // hold N+1 elements together (N even).
  // Each lane keeps its U elements' sums in registers (U independent chains).
#ifdef __CUDA_ARCH__
  const bool use_tc = sizeof(T) == sizeof(float) && tc;
  if constexpr (sizeof(T) == sizeof(float)) {
    if (use_tc) team_contract_tf32x3<NS>(tm, M, m, NM, Sp, Bs);
  }
#else
  const bool use_tc = false;
  (void)tc;
#endif
  if (!use_tc) {
    constexpr int NE = (NS / 2) * (NS + 1), U = (NE + kTeam - 1) / kTeam;
    int ii[U], jj[U];
    T se[U], so[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int e = tm.lane + kTeam * u, r = e / (N + 1), cc = e % (N + 1);
      ii[u] = (cc <= r) ? r : N - 1 - r;
      jj[u] = (cc <= r) ? cc : cc - r - 1;
      se[u] = 0;
      so[u] = 0;
    }
    for (int l = m; l <= NM; ++l) {
      const T og = M.og[l];
      const bool even = ((l - m) & 1) == 0;
#pragma unroll
      for (int u = 0; u < U; ++u) {
        if (tm.lane + kTeam * u < NE) {
          const T t = og * M.piq[ii[u]][l] * M.piq[jj[u]][l];
          if (even) se[u] += t; else so[u] += t;
        }
      }
    }
#pragma unroll
    for (int u = 0; u < U; ++u) {
      if (tm.lane + kTeam * u < NE) {
        const int i = ii[u], j = jj[u];
        Sp[i + LD * j] = se[u];
        Sp[j + LD * i] = se[u];
        T b = -M.csqw[i] * M.csqw[j] * so[u];
        if (i == j) b += (T)1;
        Bs[i + LD * j] = b;
      }
    }
  }
  tm.sync();
  if (!team_cholesky<LD>(tm, N, Bs)) return RT_EIGEN_FAIL;
  // R = M^-1 Lb
  for (int e = tm.lane; e < N * N; e += kTeam) {
    const int i = e % N, j = e / N;
    if (i >= j) Bs[i + LD * j] /= M.cqx[i];
  }
  // As = I - W^1/2 Sp W^1/2 (full)
  for (int e = tm.lane; e < N * N; e += kTeam) {
    const int i = e % N, j = e / N;
    T a = -M.csqw[i] * Sp[i + LD * j] * M.csqw[j];
    if (i == j) a += (T)1;
    H[i + LD * j] = a;
  }
  tm.sync();
  if (m == 0) {
    // exact split of the conservative mode (see layer_eigen): Q As Q, reflector v
    T ns = 0;
    for (int i = 0; i < N; ++i) ns += M.csqw[i] * M.csqw[i];
    ns = sqrt(ns);
    T vv = 0;
    for (int i = 0; i < N; ++i) {
      const T vi = M.csqw[i] + (i == 0 ? ns : (T)0);
      vv += vi * vi;
    }
    const T beta = (T)2 / vv;
    if (tm.lane < N) M.rv[tm.lane] = M.csqw[tm.lane] + (tm.lane == 0 ? ns : (T)0);
    if (tm.lane == 0) M.rbeta = beta;
    tm.sync();
    // p = beta A v ; w = p - (beta/2)(p.v) v ; A -= v w^T + w v^T
    if (tm.lane < N) {
      T s = 0;
      for (int j = 0; j < N; ++j) s += H[tm.lane + LD * j] * M.rv[j];
      M.dpi[tm.lane] = beta * s;
    }
    tm.sync();
    T pv = 0;
    for (int i = 0; i < N; ++i) pv += M.dpi[i] * M.rv[i];
    const T half = (T)0.5 * beta * pv;
    for (int e = tm.lane; e < N * N; e += kTeam) {
      const int i = e % N, j = e / N;
      const T wi = M.dpi[i] - half * M.rv[i], wj = M.dpi[j] - half * M.rv[j];
      H[i + LD * j] -= M.rv[i] * wj + wi * M.rv[j];
    }
    tm.sync();
    if (tm.lane == 0) H[0] = om1;
    if (tm.lane >= 1 && tm.lane < N) { H[tm.lane] = 0; H[LD * tm.lane] = 0; }
    tm.sync();
    if (!(om1 > (T)0)) return RT_EIGEN_FAIL;
  }
  if (!team_cholesky<LD>(tm, N, H)) return RT_EIGEN_FAIL;
  if (m == 0) {
    // QR = Q R into V (temporary), then G = L~^T QR
    const T beta = M.rbeta;
    if (tm.lane < N) {
      const int j = tm.lane;
      T d = 0;
      for (int k = j; k < N; ++k) d += M.rv[k] * Bs[k + LD * j];
      M.dmi[j] = d * beta;
    }
    tm.sync();
    for (int e = tm.lane; e < N * N; e += kTeam) {
      const int i = e % N, j = e / N;
      V[i + LD * j] = ((i >= j) ? Bs[i + LD * j] : (T)0) - M.dmi[j] * M.rv[i];
    }
    tm.sync();
    for (int e = tm.lane; e < N * N; e += kTeam) {
      const int i = e % N, j = e / N;
      T s = 0;
      for (int k = i; k < N; ++k) s += H[k + LD * i] * V[k + LD * j];
      G[i + LD * j] = s;
    }
  } else {
    for (int e = tm.lane; e < N * N; e += kTeam) {
      const int i = e % N, j = e / N;
      T s = 0;
      for (int k = (i > j ? i : j); k < N; ++k) s += H[k + LD * i] * Bs[k + LD * j];
      G[i + LD * j] = s;
    }
  }
  tm.sync();
  // FP64: warm start from the previous layer of this term; its eigenvectors
  // are usually close, so G V_prev is nearly column-orthogonal and few sweeps
  // remain.  Not in FP32: V is then a product of the rotations of every layer
  // so far, and its loss of orthogonality (a few ulp per rotation) grows along
  // the layer chain to 1e-4 and more; the eigenvectors taken from it, and a
  // radiance, go wrong by that much.
  const bool warm = M.vp_valid != 0 && sizeof(T) == sizeof(double);
  if (warm) {
    T* Wt = M.work + 4 * NS * LD;  // V slot as temporary for G V_prev
    for (int e = tm.lane; e < N * N; e += kTeam) {
      const int i = e % N, j = e / N;
      T s = 0;
      for (int k = 0; k < N; ++k) s += G[i + LD * k] * M.Vp[k + LD * j];
      Wt[i + LD * j] = s;
    }
    tm.sync();
    for (int e = tm.lane; e < N * N; e += kTeam) {
      const int i = e % N, j = e / N;
      G[i + LD * j] = Wt[i + LD * j];
      V[i + LD * j] = M.Vp[i + LD * j];
    }
  }
  if (!team_jacobi<NS, LD>(tm, N, G, V, M.kv, M.red, &M.flag, warm)) return RT_EIGEN_FAIL;
  for (int e = tm.lane; e < N * N; e += kTeam) M.Vp[e % N + LD * (e / N)] = V[e % N + LD * (e / N)];
  if (tm.lane == 0) M.vp_valid = 1;
  // per eigenvector a (lane a): La u_a in place of G[:, a], x, dif, X+, norm, user solutions
  int fail = 0;
  const int a = tm.lane;
  if (a < N) {
    const T k = M.kv[a];
    if (!(k > (T)0)) {
      fail = 1;
    } else {
      T* g = G + LD * a;
      const T inv = (T)1 / k;
      for (int i = N - 1; i >= 0; --i) {  // lower-triangular product in place, bottom up
        T s = 0;
        for (int kk = 0; kk <= i; ++kk) s += H[i + LD * kk] * g[kk];
        g[i] = s * inv;
      }
      if (m == 0) {
        T d = 0;
        for (int i = 0; i < N; ++i) d += M.rv[i] * g[i];
        d *= M.rbeta;
        for (int i = 0; i < N; ++i) g[i] -= d * M.rv[i];
      }
      T x[NS], nrm = 0;
      for (int i = 0; i < N; ++i) {
        T s = 0;
        for (int j = 0; j <= i; ++j) s += Bs[i + LD * j] * V[j + LD * a];
        x[i] = s / M.csqw[i];
        nrm += x[i] * x[i];
      }
      nrm = (T)1 / sqrt(nrm);
      T nr = 0;
      for (int i = 0; i < N; ++i) {
        x[i] *= nrm;
        const T dif = g[i] / (M.cqx[i] * M.csqw[i]) * nrm;
        g[i] = dif;  // keep dif for the user-angle solutions
        M.P[cur][i + LD * a] = (T)0.5 * (x[i] + dif);
        M.Q[cur][i + LD * a] = (T)0.5 * (x[i] - dif);
        nr += M.cqx[i] * M.cqw[i] * x[i] * dif;
      }
      M.norm[a] = nr;
      const T help = k * dtau;
      M.t[cur][a] = help > (T)kMaxTau ? (T)0 : exp(-help);
      if constexpr (!kTeamSplitSums<NS, T>) {
        T dn = 0, up = 0;
        for (int l = m; l <= NM; ++l) {
          const bool even = ((l - m) & 1) == 0;
          T sps = 0;
          for (int j = 0; j < N; ++j) sps += M.cqw[j] * M.piq[j][l] * (even ? x[j] : g[j]);
          const T h = (T)0.5 * M.og[l] * sps;
          dn += (even ? M.piu[l] : -M.piu[l]) * h;
          up += M.piu[l] * h;
        }
        M.uhd[a] = dn;
        M.uhu[a] = up;
      } else {
        for (int i = 0; i < N; ++i) Sp[i + LD * a] = x[i];  // Sp is free: x for the user solutions
      }
    }
  }
  if (team_any(tm, fail != 0, &M.flag)) return RT_EIGEN_FAIL;
  if constexpr (kTeamSplitSums<NS, T>) {
    tm.sync();
    // user-angle solutions: lanes a and a + N share eigenvector a, each summing
    // half of the moments (x in Sp, dif in G)
    const int ea = tm.lane % N, half = tm.lane / N;
    const int nl = NM - m + 1, l0 = m + (half == 0 ? 0 : (nl + 1) / 2), l1 = (half == 0) ? m + (nl + 1) / 2 : NM + 1;
    T dn = 0, up = 0;
    if (half < 2) {
      const T* xa = Sp + LD * ea;
      const T* da = G + LD * ea;
      for (int l = l0; l < l1; ++l) {
        const bool even = ((l - m) & 1) == 0;
        const T* v = even ? xa : da;
        T sps = 0;
        for (int j = 0; j < N; ++j) sps += M.cqw[j] * M.piq[j][l] * v[j];
        const T h = (T)0.5 * M.og[l] * sps;
        dn += (even ? M.piu[l] : -M.piu[l]) * h;
        up += M.piu[l] * h;
      }
    }
    dn = pair_sum(tm, dn, N, M.red);
    up = pair_sum(tm, up, N, M.red);
    if (tm.lane < N) {
      M.uhd[ea] = dn;
      M.uhu[ea] = up;
    }
  }
  return RT_OK;
}

// Layer n of term m: eigen-solution, multipliers, Green's particular solution,
// source coefficients a, b, s of the layer into M.la, M.lb, M.ls (layer_solution).
template <int NS, typename T>
RT_HD int team_layer_solution(const Team& tm, TeamMem<NS, T>& M, const SolveCtx<NS, T>& c, const RtOptions& opt,
                              int m, int n, bool laysc, int cur) {
  constexpr int LD = TeamMem<NS, T>::LD;
  const int N = NS, NM = c.NM;
  int st = team_layer_eigen<NS, T>(tm, M, c, m, cur, opt.moment_contraction != 0);
  if (st != RT_OK) return st;
  const T dtau = M.lsc[0], tuser = M.lsc[2], smu = c.sec_u;
  const int a = tm.lane;
  if (a < N) {
    if (!laysc) { M.uhd[a] = 0; M.uhu[a] = 0; }
    const T zdel = M.t[cur][a], kk = M.kv[a];
    const T rho_p = smu + kk, rho_m = smu - kk;
    if constexpr (sizeof(T) == sizeof(float)) {
      M.hm2[a] = smu * dtau * e1_fn(rho_p * dtau);
      M.hm1[a] = smu * dd1_neg(kk, smu, dtau);
    } else {
      M.hm2[a] = smu * (1.0 - zdel * tuser) * (1.0 / rho_p);
      if (fabs(rho_m) < kTaylorSmall) M.hm1[a] = taylor1<T>(opt.taylor_order, rho_m, dtau, tuser, smu);
      else M.hm1[a] = smu * (zdel - tuser) * (1.0 / rho_m);
    }
    M.la[a] = M.uhd[a] * M.hm2[a];
    M.lb[a] = M.uhu[a] * M.hm1[a];
  }
  for (int e = tm.lane; e < 2 * N; e += kTeam) { M.wt[cur][e] = 0; M.wb[cur][e] = 0; }
  tm.sync();
  const bool active = (n < c.cutoff) && laysc;
  T spart = 0;
  if (active) {
    const T F1 = (T)(opt.flux_factor / kPI4);
    const T secbar = M.lsc[3], cnst = M.lsc[4], wdel = M.lsc[5], emult = M.lsc[6];
    const int hq = tm.lane % N, half = tm.lane / N;
    if constexpr (!kTeamSplitSums<NS, T>) {
      // dpi/dmi: lanes over quadrature rows
      if (tm.lane < N) {
        const int i = tm.lane;
        T sp = 0, sm = 0;
        for (int l = m; l <= NM; ++l) {
          const T t = M.piq[i][l] * (M.og[l] * M.pi0[l]);
          sp += t;
          sm += (((l - m) & 1) ? -t : t);
        }
        M.dpi[i] = F1 * sp;
        M.dmi[i] = F1 * sm;
      }
      tm.sync();
    } else {
      // dpi/dmi: lanes i and i + N over quadrature row i, each half of the moments
      {
        const int nl = NM - m + 1, l0 = m + (half == 0 ? 0 : (nl + 1) / 2), l1 = (half == 0) ? m + (nl + 1) / 2 : NM + 1;
        T sp = 0, sm = 0;
        if (half < 2)
          for (int l = l0; l < l1; ++l) {
            const T t = M.piq[hq][l] * (M.og[l] * M.pi0[l]);
            sp += t;
            sm += (((l - m) & 1) ? -t : t);
          }
        sp = pair_sum(tm, sp, N, M.red);
        sm = pair_sum(tm, sm, N, M.red);
        if (tm.lane < N) {
          M.dpi[hq] = F1 * sp;
          M.dmi[hq] = F1 * sm;
        }
      }
      tm.sync();
    }
    T part = 0;
    if (a < N) {
      const T zdel = M.t[cur][a], kk = M.kv[a];
      const T gp = secbar + kk, gm = secbar - kk, sigp = secbar + smu, itw = -cnst * wdel;
      const bool tay = fabs(gm) < (T)kTaylorSmall;
      T cf, df, sd, su;
      if constexpr (sizeof(T) == sizeof(float)) {
        cf = cnst * dd1_neg(kk, secbar, dtau);
        df = cnst * dtau * e1_fn(gp * dtau);
        sd = cnst * smu * dd2(kk + smu, sigp, dtau);
        su = cnst * smu * dd2(gp, sigp, dtau);
      } else {
        cf = tay ? taylor1<T>(opt.taylor_order, gm, dtau, wdel, cnst) : cnst * (zdel - wdel) / gm;
        df = cnst * (1.0 - zdel * wdel) / gp;
        if (tay) sd = (cnst * smu) * taylor2<T>(opt.taylor_order, gm, sigp, dtau, (T)1, wdel * tuser, (T)1);
        else sd = (cnst * M.hm2[a] - emult) / gm;
        su = (itw * M.hm1[a] + emult) / gp;
      }
      if constexpr (!kTeamSplitSums<NS, T>) {
        T s1 = 0, s2 = 0;
        for (int i = 0; i < N; ++i) {
          s1 += M.cqw[i] * (M.dpi[i] * M.P[cur][i + LD * a] + M.dmi[i] * M.Q[cur][i + LD * a]);
          s2 += M.cqw[i] * (M.dmi[i] * M.P[cur][i + LD * a] + M.dpi[i] * M.Q[cur][i + LD * a]);
        }
        const T at = s1 / M.norm[a], bt = s2 / M.norm[a];
        M.gdn[a] = cf * at;
        M.gup[a] = df * bt;
        part = M.uhd[a] * sd * at + M.uhu[a] * su * bt;
      } else {
        M.hm2[a] = cf;  // multipliers of eigenvector a, until at and bt are known
        M.gdn[a] = df;
        M.gup[a] = sd;
        M.red[a] = su;
      }
    }
    if constexpr (kTeamSplitSums<NS, T>) {
      tm.sync();
      // projections at, bt of the beam source on eigenvector hq: lanes hq and
      // hq + N, each half of the quadrature rows
      {
        const int i0 = half == 0 ? 0 : N / 2, i1 = half == 0 ? N / 2 : N;
        T s1 = 0, s2 = 0;
        if (half < 2)
          for (int i = i0; i < i1; ++i) {
            s1 += M.cqw[i] * (M.dpi[i] * M.P[cur][i + LD * hq] + M.dmi[i] * M.Q[cur][i + LD * hq]);
            s2 += M.cqw[i] * (M.dmi[i] * M.P[cur][i + LD * hq] + M.dpi[i] * M.Q[cur][i + LD * hq]);
          }
        s1 = pair_sum(tm, s1, N, M.red + kTeam);
        s2 = pair_sum(tm, s2, N, M.red + kTeam);
        if (a < N) {
          const T cf = M.hm2[a], df = M.gdn[a], sd = M.gup[a], su = M.red[a];
          const T at = s1 / M.norm[a], bt = s2 / M.norm[a];
          part = M.uhd[a] * sd * at + M.uhu[a] * su * bt;
          M.gdn[a] = cf * at;
          M.gup[a] = df * bt;
        }
      }
    }
    tm.sync();
    M.red[tm.lane] = part;
    tm.sync();
    for (int k = 0; k < N; ++k) spart += M.red[k];
    if constexpr (!kTeamSplitSums<NS, T>) {
      if (tm.lane < N) {
        const int i = tm.lane;
        T wu1 = 0, wu2 = 0, wl1 = 0, wl2 = 0;
        for (int k = 0; k < N; ++k) {
          wu1 += M.gup[k] * M.Q[cur][i + LD * k]; wu2 += M.gup[k] * M.P[cur][i + LD * k];
          wl1 += M.gdn[k] * M.P[cur][i + LD * k]; wl2 += M.gdn[k] * M.Q[cur][i + LD * k];
        }
        M.wt[cur][i] = wu1; M.wt[cur][N + i] = wu2;
        M.wb[cur][i] = wl1; M.wb[cur][N + i] = wl2;
      }
    } else {
      // particular solution at the layer boundaries, row hq: lanes hq and hq + N, half of the eigenvectors each
      const int k0 = half == 0 ? 0 : N / 2, k1 = half == 0 ? N / 2 : N;
      T wu1 = 0, wu2 = 0, wl1 = 0, wl2 = 0;
      if (half < 2)
        for (int k = k0; k < k1; ++k) {
          wu1 += M.gup[k] * M.Q[cur][hq + LD * k]; wu2 += M.gup[k] * M.P[cur][hq + LD * k];
          wl1 += M.gdn[k] * M.P[cur][hq + LD * k]; wl2 += M.gdn[k] * M.Q[cur][hq + LD * k];
        }
      wu1 = pair_sum(tm, wu1, N, M.red + kTeam);
      wu2 = pair_sum(tm, wu2, N, M.red + kTeam);
      wl1 = pair_sum(tm, wl1, N, M.red + kTeam);
      wl2 = pair_sum(tm, wl2, N, M.red + kTeam);
      if (tm.lane < N) {
        M.wt[cur][hq] = wu1; M.wt[cur][N + hq] = wu2;
        M.wb[cur][hq] = wl1; M.wb[cur][N + hq] = wl2;
      }
    }
    if (!c.msmode) {
      T upar = 0;
      for (int l = m; l <= NM; ++l) upar += (F1 * M.og[l] * M.pi0[l]) * ((((l - m) & 1) ? (T)-1 : (T)1) * M.piu[l]);
      spart += upar * emult;
    }
  }
  if (tm.lane == 0) M.ls = laysc ? spart : (T)0;
  tm.sync();
  return RT_OK;
}

// One Fourier term (fourier_term): layer solutions, block interface sweep,
// surface closure, TOA source.  Per-layer inputs come from the set-up
// thread's scratch W.
//
// The sweep leaves, per interface, M_{n-1} = c_{n-1} + C_{n-1} M_n and
// L_n = f_n + F_n M_n, and the TOA source is the recursion
// cum_n = s_n + a_n.L_n + b_n.M_n + tuser_n cum_{n+1} (the back-substitution
// and UPUSER_INTENSITY of the reference).  That value is linear in the
// M_n, so it is accumulated top-down during the sweep instead:
//   out = sum_n T_n (s_n + a_n.f_n) + sum_{n<L-1} v_n.c_n + v_{L-1}.M_{L-1} + T_L cum_L,
//   v_n = C_{n-1}^T v_{n-1} + T_n (F_n^T a_n + b_n),   T_n = prod_{k<n} tuser_k,
// with cum_L the surface term.  Nothing per layer is stored, so the term's
// memory traffic is its inputs W alone.  Every lane returns the same status
// and *out.
//
// BRDF = true (the RTLS surface of VLIDORT_Scalar_LandMODIS, FP64): the
// surface reflects in every term, with the Fourier components of rt_brdf.cuh
// in place of the albedo -- BVP rows R2_HOMP/R2_HOMM and R2_BEAM with
// QUAD_STRMWTS(j) BRDF_F(m, i, j) (vlidort_bvproblem.f90:558-614, 1680-1736),
// direct beam ATTN BRDF_F_0(m, i) per stream (vlidort_miscsetups.f90:1517-1545),
// and the view-angle surface source sum_j STOKES_DOWNSURF(j) USER_BRDF_F(m, j)
// (vlidort_intensity.f90:1378-1396).  `brdf` holds the launch's tables and
// `bidx` is this solve's block.
template <int NS, typename T, bool BRDF = false>
RT_HD int team_fourier_term(const Team& tm, TeamMem<NS, T>& M, SolveCtx<NS, T>& c, const RtOptions& opt, int m,
                            const ScratchT<T>& W, const ScratchLayout<NS>& lay, T* out,
                            const BrdfInputs* brdf = nullptr, long bidx = 0) {
  static_assert(!BRDF || sizeof(T) == sizeof(double), "the BRDF surface runs in FP64");
  constexpr int LD = TeamMem<NS, T>::LD;
  constexpr int LR = TeamMem<NS, T>::LR;
  const int N = NS, NM = c.NM, L = c.L;
  const bool incl_surface = BRDF ? true : ((m == 0) && (c.albedo != (T)0));
  const T surface_factor = (m == 0) ? (T)2 : (T)1;
  const T delta_factor = (m == 0) ? (T)1 : (T)2;
  const bool localbeam = incl_surface && c.refl_directbeam;
  T direct_beam = 0, beam_attn = 0;
  if (localbeam) {
    T x0 = (T)4 * c.cos_sza / delta_factor;
    x0 = (T)opt.flux_factor * x0 / (T)kPI4;
    beam_attn = x0 * c.trans_solar_beam;
    direct_beam = beam_attn * c.albedo;
  }
  team_legendre<NS, T>(tm, M, c, m);
  T* K = M.work;  // interface systems, row-major (team_lu_solve)
  int cur = 1, prev = 0;
  if (tm.lane == 0) M.vp_valid = 0;
  for (int i = tm.lane; i < N; i += kTeam) M.adj[i] = 0;
  T acc = 0, tcum = 1;  // the TOA source so far and T_n (every lane the same)
  tm.sync();
  for (int n = 0; n < L; ++n) {
    // per-layer inputs of layer n
    for (int l = tm.lane; l <= NM; l += kTeam) M.og[l] = (l >= m) ? W[lay.og + l + 2 * NS * (long)n] : (T)0;
    if (tm.lane < 8) {
      const long src[8] = {lay.tdtau, lay.om1, lay.tuser, lay.tavsec, lay.titrans, lay.tmubar, lay.emult, lay.lnz};
      M.lsc[tm.lane] = W[src[tm.lane] + n];
    }
    tm.sync();
    const bool lsc = (m < 3) || ((T)m <= M.lsc[7]);
    int st = team_layer_solution<NS, T>(tm, M, c, opt, m, n, lsc, cur);
    if (st != RT_OK) return st;
    if (n == 0) {
      const int nb = rhs_col(N);
      for (int e = tm.lane; e < N * N; e += kTeam) {
        const int j = e % N, i = e / N;
        K[LR * i + j] = M.P[cur][i + LD * j];
        K[LR * i + nb + j] = -M.Q[cur][i + LD * j] * M.t[cur][j];
      }
      for (int i = tm.lane; i < N; i += kTeam) K[LR * i + nb + N] = -M.wt[cur][i];
      tm.sync();
      if (!team_lu_solve<LR>(tm, N, K, N + 1, M.red)) return RT_BVP_SINGULAR;
      for (int e = tm.lane; e < N * N; e += kTeam) {
        const int i = e % N, j = e / N;
        M.F[i + LD * j] = K[LR * i + nb + j];
      }
      for (int i = tm.lane; i < N; i += kTeam) M.f[i] = K[LR * i + nb + N];
      tm.sync();
    } else {
      const int nb = rhs_col(2 * N);
      {
        // U elements per lane, their 2U sums in registers (independent chains)
        constexpr int NE = NS * NS, U = (NE + kTeam - 1) / kTeam;
        T gt[U], gb[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
          const int e = tm.lane + kTeam * u;
          if (e < NE) {
            const int j = e % N, i = e / N;
            gt[u] = M.Q[prev][i + LD * j];
            gb[u] = M.P[prev][i + LD * j];
          }
        }
        for (int k = 0; k < N; ++k) {
          const T tk = M.t[prev][k];
#pragma unroll
          for (int u = 0; u < U; ++u) {
            const int e = tm.lane + kTeam * u;
            if (e < NE) {
              const int j = e % N, i = e / N;
              const T tf = tk * M.F[k + LD * j];
              gt[u] += M.P[prev][i + LD * k] * tf;
              gb[u] += M.Q[prev][i + LD * k] * tf;
            }
          }
        }
#pragma unroll
        for (int u = 0; u < U; ++u) {
          const int e = tm.lane + kTeam * u;
          if (e < NE) {
            const int j = e % N, i = e / N;
            K[LR * i + j] = gt[u];
            K[LR * (N + i) + j] = gb[u];
            K[LR * i + N + j] = -M.P[cur][i + LD * j];
            K[LR * (N + i) + N + j] = -M.Q[cur][i + LD * j];
            K[LR * i + nb + j] = M.Q[cur][i + LD * j] * M.t[cur][j];
            K[LR * (N + i) + nb + j] = M.P[cur][i + LD * j] * M.t[cur][j];
          }
        }
      }
      for (int i = tm.lane; i < N; i += kTeam) {
        T gt = 0, gb = 0;
        for (int k = 0; k < N; ++k) {
          const T tf = M.t[prev][k] * M.f[k];
          gt += M.P[prev][i + LD * k] * tf;
          gb += M.Q[prev][i + LD * k] * tf;
        }
        K[LR * i + nb + N] = M.wt[cur][i] - M.wb[prev][i] - gt;
        K[LR * (N + i) + nb + N] = M.wt[cur][N + i] - M.wb[prev][N + i] - gb;
      }
      tm.sync();
      if (!team_lu_solve<LR>(tm, 2 * N, K, N + 1, M.red)) return RT_BVP_SINGULAR;
      // through M_{n-1} = c_{n-1} + C_{n-1} M_n (C, c in the upper rows of the solution)
      T d = 0;
      for (int k = 0; k < N; ++k) d += M.adj[k] * K[LR * k + nb + N];
      acc += d;
      T vn = 0;
      if (tm.lane < N)
        for (int i = 0; i < N; ++i) vn += M.adj[i] * K[LR * i + nb + tm.lane];
      for (int e = tm.lane; e < N * N; e += kTeam) {
        const int i = e % N, j = e / N;
        M.F[i + LD * j] = K[LR * (N + i) + nb + j];
      }
      for (int i = tm.lane; i < N; i += kTeam) M.f[i] = K[LR * (N + i) + nb + N];
      tm.sync();
      if (tm.lane < N) M.adj[tm.lane] = vn;
    }
    // source of layer n: T_n (s_n + a_n.(f_n + F_n M_n) + b_n.M_n)
    {
      T d = M.ls;
      for (int k = 0; k < N; ++k) d += M.la[k] * M.f[k];
      acc += tcum * d;
      if (tm.lane < N) {
        const int k = tm.lane;
        T v = M.lb[k];
        for (int i = 0; i < N; ++i) v += M.F[i + LD * k] * M.la[i];
        M.adj[k] += tcum * v;
      }
      tcum *= M.lsc[2];
      tm.sync();
    }
    prev = cur;
    cur = 1 - cur;
  }
  // surface closure on the bottom layer (slot prev)
  const int bl = prev;
  const T kmult = incl_surface ? surface_factor * c.albedo : (T)0;
  const int nbc = rhs_col(N);
  Scratch Bb{nullptr, 0};
  if constexpr (BRDF) {
    // R(i, l) = BRDF_F(m, i, l) in M.Vp, R2P / R2M in the free layer slot,
    // R2_BEAM(i) in M.dpi, DIRECT_BEAM(i) in M.dmi
    const int fr = 1 - bl;
    using BB = BrdfBlock<NS>;
    Bb = Scratch{brdf->terms + bidx, brdf->stride};
    if (brdf->kind != kBrdfRTLS) {  // a glint solve's own components
      for (int e = tm.lane; e < N * N; e += kTeam) {
        const int i = e / N, l = e % N;
        M.Vp[i + LD * l] = (T)Bb[BB::qq + ((long)m * NS + i) * NS + l];
      }
    } else {
      const double fiso = Bb[BB::w], fvol = Bb[BB::w + 1], fgeo = Bb[BB::w + 2];
      const int t = (int)Bb[BB::w + 3];
      const double* qv = brdf->qq + (long)m * NS * NS;
      const double* qg = brdf->qq + ((long)(1 + t) * 2 * NS + m) * NS * NS;
      for (int e = tm.lane; e < N * N; e += kTeam) {
        const int i = e / N, l = e % N;
        double r = (m == 0) ? fiso : 0.0;
        r += fvol * qv[i * NS + l];
        r += fgeo * qg[i * NS + l];
        M.Vp[i + LD * l] = (T)r;
      }
    }
    tm.sync();
    for (int e = tm.lane; e < N * N; e += kTeam) {
      const int i = e % N, k = e / N;
      T sp = 0, sm = 0;
      for (int l = 0; l < N; ++l) {
        const T ax = M.cqx[l] * M.cqw[l] * M.Vp[i + LD * l];
        sp += ax * M.P[bl][l + LD * k];
        sm += ax * M.Q[bl][l + LD * k];
      }
      M.P[fr][i + LD * k] = surface_factor * sp;
      M.Q[fr][i + LD * k] = surface_factor * sm;
    }
    if (tm.lane < N) {
      const int i = tm.lane;
      T s = 0;
      for (int l = 0; l < N; ++l) s += M.cqx[l] * M.cqw[l] * M.Vp[i + LD * l] * M.wb[bl][l];
      M.dpi[i] = surface_factor * s;
      M.dmi[i] = localbeam ? beam_attn * (T)Bb[BB::r0 + (long)m * NS + i] : (T)0;
    }
    tm.sync();
    for (int e = tm.lane; e < N * N; e += kTeam) {
      const int j = e % N, i = e / N;
      T s = M.P[bl][i + LD * j] - M.Q[fr][i + LD * j];
      for (int k = 0; k < N; ++k) s += (M.Q[bl][i + LD * k] - M.P[fr][i + LD * k]) * M.t[bl][k] * M.F[k + LD * j];
      K[LR * i + j] = s;
    }
    if (tm.lane < N) {
      const int i = tm.lane;
      T s = -M.wb[bl][N + i] + M.dpi[i] + M.dmi[i];
      for (int k = 0; k < N; ++k) s -= (M.Q[bl][i + LD * k] - M.P[fr][i + LD * k]) * M.t[bl][k] * M.f[k];
      K[LR * i + nbc] = s;
    }
    tm.sync();
  } else {
    if (tm.lane < N) {
      const int k = tm.lane;
      T sp = 0, sm = 0;
      for (int j = 0; j < N; ++j) {
        sp += M.cqx[j] * M.cqw[j] * M.P[bl][j + LD * k];
        sm += M.cqx[j] * M.cqw[j] * M.Q[bl][j + LD * k];
      }
      M.dpi[k] = sp * kmult;   // r2p
      M.dmi[k] = sm * kmult;   // r2m
    }
    T r2b = 0;
    for (int j = 0; j < N; ++j) r2b += M.cqx[j] * M.cqw[j] * M.wb[bl][j];
    r2b *= kmult;
    tm.sync();
    for (int e = tm.lane; e < N * N; e += kTeam) {
      const int j = e % N, i = e / N;
      T s = M.P[bl][i + LD * j] - M.dmi[j];
      for (int k = 0; k < N; ++k) s += (M.Q[bl][i + LD * k] - M.dpi[k]) * M.t[bl][k] * M.F[k + LD * j];
      K[LR * i + j] = s;
    }
    if (tm.lane < N) {
      const int i = tm.lane;
      T s = -M.wb[bl][N + i] + r2b + (localbeam ? direct_beam : (T)0);
      for (int k = 0; k < N; ++k) s -= (M.Q[bl][i + LD * k] - M.dpi[k]) * M.t[bl][k] * M.f[k];
      K[LR * i + nbc] = s;
    }
    tm.sync();
  }
  if (!team_lu_solve<LR>(tm, N, K, 1, M.red)) return RT_BVP_SINGULAR;
  // M_{L-1} (Mc) from the solved right-hand side, L_{L-1} (Lc) in M.gup
  T* Mc = M.hm1;
  T* Lc = M.gup;
  if (tm.lane < N) Mc[tm.lane] = K[LR * tm.lane + nbc];
  tm.sync();
  if (tm.lane < N) {
    const int i = tm.lane;
    T s = M.f[i];
    for (int k = 0; k < N; ++k) s += M.F[i + LD * k] * Mc[k];
    Lc[i] = s;
  }
  tm.sync();
  T cum = 0;
  if (incl_surface) {
    if (tm.lane < N) {
      const int i = tm.lane;
      T h = M.wb[bl][i];
      for (int k = 0; k < N; ++k) h += Lc[k] * M.P[bl][i + LD * k] * M.t[bl][k] + Mc[k] * M.Q[bl][i + LD * k];
      M.red[i] = M.cqx[i] * M.cqw[i] * h;
    }
    tm.sync();
    T s = 0;
    const bool incl_directrf = localbeam && !opt.do_focorr && !c.msmode;
    if constexpr (BRDF) {
      using BB = BrdfBlock<NS>;
      for (int i = 0; i < N; ++i) s += M.red[i] * (T)Bb[BB::ur + (long)m * NS + i];
      cum = surface_factor * s;
      if (incl_directrf) cum += beam_attn * (T)Bb[BB::ur0 + m];
    } else {
      for (int i = 0; i < N; ++i) s += M.red[i];
      cum = kmult * s;
      if (incl_directrf) cum += direct_beam;
    }
    tm.sync();
  }
  T d = 0;
  for (int k = 0; k < N; ++k) d += M.adj[k] * Mc[k];
  const T total = acc + d + tcum * cum;
  tm.sync();
  *out = delta_factor * total;
  return RT_OK;
}

// The Fourier series of one set-up solve, run by the whole team; lane 0 writes
// the outputs.
// The team's per-solve state before term 0: the solve context and, in shared
// memory for lane-indexed access, the quadrature arrays of make_ctx and the
// Legendre P~_m^m carried across terms.
template <int NS, typename T>
RT_HD void team_series_init(const Team& tm, TeamMem<NS, T>& M, const SetupRecord& r, const double* qx,
                            const double* qw, SolveCtx<NS, T>& c) {
  make_ctx<NS, T>(r, qx, qw, c);
  if (tm.lane < NS) {
    const int q = tm.lane;
    M.cqx[q] = (T)qx[q];
    M.cqw[q] = (T)qw[q];
    M.csqw[q] = (T)sqrt(qw[q]);
    M.csin[q] = (T)quad_sine(qx[q]);
    M.pimq[q] = 0;
  }
  if (tm.lane == 0) { M.pimu = 0; M.pim0 = 0; }
  tm.sync();
}

template <int NS, typename T, bool BRDF = false>
RT_HD void team_fourier_series(const Team& tm, TeamMem<NS, T>& M, const RtOptions& opt, const LambertInputs& in,
                               const SetupRecord& r, const double* qx, const double* qw, const ScratchT<T>& W,
                               const ScratchLayout<NS>& lay, double* radiance, double* reflectance,
                               int* nfourier, int* status, const Worklist& wl = Worklist(), int sidx = 0,
                               const BrdfInputs* brdf = nullptr, long bidx = 0) {
  SolveCtx<NS, T> c;
  team_series_init<NS, T>(tm, M, r, qx, qw, c);
  FourierSum sum;
  int m = 0, st = RT_OK;
  for (m = 0; m <= r.n_fouriers; ++m) {
    T sf = 0;
    st = team_fourier_term<NS, T, BRDF>(tm, M, c, opt, m, W, lay, &sf, brdf, bidx);
    if (st != RT_OK || sum.add(opt, r, m, (double)sf)) break;
  }
  if (tm.lane == 0) {
    solve_finish(opt, in, r, st, m, sum.stokes, radiance, reflectance, nfourier, status);
    wl.flag(sum, st, sidx);
  }
  tm.sync();
}

}  // namespace aerort
