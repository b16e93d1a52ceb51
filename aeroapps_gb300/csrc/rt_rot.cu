// Rayleigh optical thickness and depolarisation on the device: the
// reference's VLIDORT_ROT_CALC (geo_vlidort/VLIDORT_ROT.F90:19-86), i.e.
// VLIDORT_Rayleigh, A(), coef_depol and F_air
// (RTSI/VLIDORT2p8p3/VLIDORT_ScatMod.F90:145-283) for every pixel and channel.
//
// Bit-identical to the reference arithmetic: every operation is an explicitly
// rounded FP64 intrinsic (no FMA contraction) in the Fortran evaluation order;
// the reference's default-REAL literals enter as the nearest float, and its
// all-literal subexpressions are evaluated in single precision.
//
// Layout: blocks walk groups of pixels; per group the channel-independent
// edge quotients and layer height differences go to shared memory once, then
// every channel's km layer values are written.  Reads pe/he/te once (3 x
// (km+1) doubles per pixel), writes km doubles per pixel and channel.  On
// GB300 the FP64 divisions (two per edge) and multiplications set the pace
// rather than HBM.
#include "aerort_internal.cuh"

namespace aerort_internal {
namespace {

#define LIT(x) ((double)(x##f))  // a default-REAL literal widened to REAL*8

__host__ __device__ inline double dm(double a, double b) {
#ifdef __CUDA_ARCH__
  return __dmul_rn(a, b);
#else
  return a * b;
#endif
}
__host__ __device__ inline double da(double a, double b) {
#ifdef __CUDA_ARCH__
  return __dadd_rn(a, b);
#else
  return a + b;
#endif
}
__host__ __device__ inline double ds(double a, double b) {
#ifdef __CUDA_ARCH__
  return __dsub_rn(a, b);
#else
  return a - b;
#endif
}
__host__ __device__ inline double dd(double a, double b) {
#ifdef __CUDA_ARCH__
  return __ddiv_rn(a, b);
#else
  return a / b;
#endif
}

// F_air (ScatMod.F90:267-283): King factor of the air mixture; c = CO2 ratio.
__host__ __device__ inline double king_factor(double xx2, double c) {
  const double d1 = da(LIT(1.034), dm(LIT(3.17E-4), xx2));
  const double d2 = da(da(LIT(1.096), dm(LIT(1.385E-3), xx2)), dm(dm(LIT(1.448E-4), xx2), xx2));
  const double d3 = 1.0, d4 = LIT(1.15);
  const double c100 = dm(c, LIT(100.0));
  const double num = da(da(da(dm(LIT(78.084), d1), dm(LIT(20.946), d2)), dm(LIT(0.934), d3)), dm(c100, d4));
  const float lit_sum = (78.084f + 20.946f) + 0.934f;  // REAL*4 in the reference
  return dd(num, da((double)lit_sum, c100));
}

__host__ __device__ inline double co2_ratio() { return (double)(360.0f * 1e-6f); }  // `360.0*1e-6`, REAL*4

// Ns = (Av/22.4141)*(273.15/Ts)*(1.0/1000) [molecules/cm^3]
__host__ __device__ inline double ns_standard() {
  return dm(dm(dd(LIT(6.0221367e23), LIT(22.4141)), dd(LIT(273.15), LIT(288.15))), (double)(1.0f / 1000.0f));
}

// A(X): Rayleigh cross section [cm^2/molecule] at X micron (ScatMod.F90:211-247).
__host__ __device__ inline double rayleigh_cross_section(double x) {
  const double pi = (double)3.14159274101257324f;  // 4.*atan(1.0) in REAL*4
  const double xx = dd(1.0, x);
  const double xx2 = dm(xx, xx);
  const double cm = dd(x, LIT(10000.0));
  const double pi3 = dm(dm(pi, pi), pi);
  double ri = da(da(LIT(8060.51), dd(LIT(2480990.0), ds(LIT(132.274), xx2))), dd(LIT(17455.7), ds(LIT(39.32957), xx2)));
  ri = da(dm(ri, LIT(1e-8)), 1.0);
  const double c = co2_ratio();
  ri = da(dm(ds(ri, 1.0), da(1.0, dm(LIT(0.54), ds(c, LIT(0.0003))))), 1.0);
  const double ri2 = dm(ri, ri);
  const double ns = ns_standard();
  const double num = dm(dm(dm(24.0, pi3), king_factor(xx2, c)), dm(ds(ri2, 1.0), ds(ri2, 1.0)));
  double den = dm(ns, ns);
  den = dm(den, cm);
  den = dm(den, cm);
  den = dm(den, cm);
  den = dm(den, cm);
  den = dm(den, da(ri2, 2.0));
  den = dm(den, da(ri2, 2.0));
  return dd(num, den);
}

// coef_depol (ScatMod.F90:251-265), x in micron.
__host__ __device__ inline double depolarisation(double x) {
  const double xx = dd(1.0, x);
  const double xx2 = dm(xx, xx);
  const double c = co2_ratio();
  const double f = king_factor(xx2, c);
  return dd(dm(6.0, ds(f, 1.0)), da(dm(7.0, f), 3.0));
}

// Each block iteration takes cpb pixels, whose (km+1)-edge profiles are
// contiguous: thread t reads edge word t of the group (coalesced).  The two
// divisions of an edge, (p/Ps) and (Ts/T), and the height difference of a
// layer do not depend on the channel, so they are formed once per pixel; per
// channel only the products with A(lambda) Ns remain.  The reference's
// evaluation order ((A Ns) (p/Ps)) (Ts/T) 1e5 allows exactly this split.
// Division by 2 is the exact product with 0.5.
__global__ void k_rot_calc(int km, int nch, int nobs, const double* __restrict__ channels,
                           const double* __restrict__ pe, const double* __restrict__ he,
                           const double* __restrict__ te, double* __restrict__ rot, double* __restrict__ depol) {
  // shared: A(lambda) Ns per channel; cpb x (km+1) p/Ps and Ts/T; cpb x km layer height differences
  extern __shared__ double sm[];
  const double ps = LIT(1013.25), ts = LIT(288.15);
  const int ne = km + 1;
  const int cpb = blockDim.x / ne > 0 ? blockDim.x / ne : 1;
  double* ans = sm;
  double* qp = sm + nch;
  double* qt = qp + cpb * ne;
  double* dz = qt + cpb * ne;
  for (int i = threadIdx.x; i < nch; i += blockDim.x) {
    const double wmicron = dm(channels[i], LIT(1.E-3));
    ans[i] = dm(rayleigh_cross_section(wmicron), ns_standard());
    if (blockIdx.x == 0) depol[i] = depolarisation(wmicron);
  }
  __syncthreads();
  for (long j0 = (long)blockIdx.x * cpb; j0 < nobs; j0 += (long)gridDim.x * cpb) {
    const long nj = (nobs - j0 < cpb) ? nobs - j0 : cpb;
    const long base = (long)ne * j0;
    for (int t = threadIdx.x; t < nj * ne; t += blockDim.x) {
      qp[t] = dd(dm(pe[base + t], LIT(1.E-2)), ps);
      qt[t] = dd(ts, te[base + t]);
    }
    for (int t = threadIdx.x; t < nj * km; t += blockDim.x) {
      const int c = t / km, k = t - c * km;
      const double* z = he + base + (long)ne * c;
      dz[t] = ds(dm(z[k], LIT(1.E-3)), dm(z[k + 1], LIT(1.E-3)));
    }
    __syncthreads();
    for (int i = 0; i < nch; ++i) {
      const double a_ns = ans[i];
      double* out = rot + (long)km * (j0 + (long)nobs * i);
      for (int t = threadIdx.x; t < nj * km; t += blockDim.x) {
        const int c = t / km, k = t - c * km;
        const int e = ne * c + k;
        const double v0 = dm(dm(dm(a_ns, qp[e]), qt[e]), LIT(1.E5));
        const double v1 = dm(dm(dm(a_ns, qp[e + 1]), qt[e + 1]), LIT(1.E5));
        out[t] = dm(dm(dz[t], da(v0, v1)), 0.5);
      }
    }
    __syncthreads();
  }
}

int rot_checks(int km, int nch, int nobs) {
  if (km <= 0 || nch <= 0 || nobs < 0) return set_error(AERORT_RC_ARG, "rot_calc: bad sizes");
  if (((size_t)3 * (km + 1) + nch) * sizeof(double) > 200 * 1024)
    return set_error(AERORT_RC_NLAYERS, "rot_calc: km or nch too large");
  return 0;
}

int launch_rot(int km, int nch, int nobs, const double* channels, const double* pe, const double* he,
               const double* te, double* rot, double* depol, cudaStream_t s, int num_sms) {
  if (nobs == 0) return 0;
  constexpr int kThreads = 256;
  const int ne = km + 1, cpb = kThreads / ne > 0 ? kThreads / ne : 1;
  const size_t smem = ((size_t)cpb * (3 * ne) + nch) * sizeof(double);
  if (smem > 48 * 1024)
    CUDA_TRY(cudaFuncSetAttribute(k_rot_calc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  long blocks = (nobs + cpb - 1) / cpb;
  const long cap = (long)num_sms * 8;  // about 8 resident 256-thread blocks per SM
  if (blocks > cap) blocks = cap;
  k_rot_calc<<<(unsigned)blocks, kThreads, smem, s>>>(km, nch, nobs, channels, pe, he, te, rot, depol);
  CUDA_TRY(cudaGetLastError());
  count_launches(1);
  return 0;
}

}  // namespace
}  // namespace aerort_internal

using namespace aerort_internal;

extern "C" int aerort_vlidort_rot_calc_dev(int km, int nch, int nobs, const double* channels, const double* pe,
                                           const double* he, const double* te, double* ROT, double* depol,
                                           void* stream) {
  if (int rc = rot_checks(km, nch, nobs)) return rc;
  if (!channels || !pe || !he || !te || !ROT || !depol) return set_error(AERORT_RC_ARG, "rot_calc_dev: null array");
  Context& c = ctx();
  int num_sms = 0;
  {
    std::lock_guard<std::mutex> lk(c.mu);
    if (int rc = c.setup()) return rc;
    num_sms = c.num_sms;
  }
  return launch_rot(km, nch, nobs, channels, pe, he, te, ROT, depol, (cudaStream_t)stream, num_sms);
}

extern "C" int aerort_vlidort_rot_calc(int km, int nch, int nobs, const double* channels, const double* pe,
                                       const double* he, const double* te, double MISSING, int verbose, double* ROT,
                                       double* depol) {
  (void)MISSING;  // VLIDORT_Rayleigh cannot fail, so no layer is ever set to MISSING
  (void)verbose;
  if (int rc = rot_checks(km, nch, nobs)) return rc;
  if (!channels || !pe || !he || !te || !ROT || !depol) return set_error(AERORT_RC_ARG, "rot_calc: null array");
  Context& c = ctx();
  std::lock_guard<std::mutex> lk(c.mu);
  if (int rc = c.setup()) return rc;
  cudaStream_t s = c.stream;
  const size_t ne = (size_t)(km + 1) * nobs, nr = (size_t)km * nobs * nch;
  // staging buffers 16..20 are this entry point's
  if (int rc = c.stage[16].ensure(8 * (size_t)nch)) return rc;
  if (int rc = c.stage[17].ensure(8 * ne + 8)) return rc;
  if (int rc = c.stage[18].ensure(8 * ne + 8)) return rc;
  if (int rc = c.stage[19].ensure(8 * ne + 8)) return rc;
  if (int rc = c.stage[20].ensure(8 * (nr + nch) + 8)) return rc;
  double* dch = (double*)c.stage[16].p;
  double* dpe = (double*)c.stage[17].p;
  double* dhe = (double*)c.stage[18].p;
  double* dte = (double*)c.stage[19].p;
  double* drot = (double*)c.stage[20].p;
  double* ddep = drot + nr;
  CUDA_TRY(cudaMemcpyAsync(dch, channels, 8 * (size_t)nch, cudaMemcpyHostToDevice, s));
  CUDA_TRY(cudaMemcpyAsync(dpe, pe, 8 * ne, cudaMemcpyHostToDevice, s));
  CUDA_TRY(cudaMemcpyAsync(dhe, he, 8 * ne, cudaMemcpyHostToDevice, s));
  CUDA_TRY(cudaMemcpyAsync(dte, te, 8 * ne, cudaMemcpyHostToDevice, s));
  if (int rc = launch_rot(km, nch, nobs, dch, dpe, dhe, dte, drot, ddep, s, c.num_sms)) return rc;
  if (nobs > 0) {
    CUDA_TRY(cudaMemcpyAsync(ROT, drot, 8 * nr, cudaMemcpyDeviceToHost, s));
    CUDA_TRY(cudaMemcpyAsync(depol, ddep, 8 * (size_t)nch, cudaMemcpyDeviceToHost, s));
  }
  CUDA_TRY(cudaStreamSynchronize(s));
  return AERORT_OK;
}
