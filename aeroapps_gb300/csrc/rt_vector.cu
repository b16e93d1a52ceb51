// Polarized RT (VLIDORT_Vector_Lambert, NSTOKES = 3): kernel, launcher and C ABI.
//
// k_vector_lambert<N>: one warp per (column, wavelength) solve, a persistent
// grid pulling solves from an atomic work counter; each warp owns one global
// working region (VecLayout) and one shared-memory working set (VecShared).
// The solve itself is vec_solve (rt_vector.cuh).
#include "aerort_internal.cuh"
#include "rt_vector.cuh"

using namespace aerort;
using namespace aerort_internal;

namespace aerort_internal {

// defined in aerort.cu (shared with the scalar launchers)
__global__ void k_nadir_first(int nobs, int nch, const double* sza, const double* raa, const double* vza,
                              const double* albedo, double missing, int* first);
__global__ void k_init_sched(int* counter, int* first, int nobs, int* zero);

template <int N>
__global__ void __launch_bounds__(32) k_vector_lambert(RtOptions opt, VectorInputs vin, Quad q, double* scratch,
                                                       long per_warp, int nsolve, int* counter, double* rad,
                                                       double* refl, double* Qo, double* Uo, int* nf, int* st) {
  extern __shared__ __align__(16) unsigned char vec_smem[];
  VecShared<N>& sh = *reinterpret_cast<VecShared<N>*>(vec_smem);
  const Team tm{(int)(threadIdx.x & 31), nullptr, nullptr};
  double* ws = scratch + (long)blockIdx.x * per_warp;
  for (;;) {
    int s = 0;
    if (tm.lane == 0) s = atomicAdd(counter, 1);
    s = __shfl_sync(0xffffffffu, s, 0);
    if (s >= nsolve) break;
    vec_solve<N>(tm, sh, opt, vin, s, q.qx, q.qw, q.tu, q.wu, ws, rad, refl, Qo, Uo, nf, st);
  }
}

namespace {

template <int N>
int launch_vector(Context& c, const RtOptions& opt, const VectorInputs& vin, double* rad, double* refl, double* Qo,
                  double* Uo, int* nf, int* st, cudaStream_t s) {
  const LambertInputs& in = vin.base;
  const int nsolve = in.nobs * in.nch;
  if (nsolve == 0) return 0;
  Quad q;
  std::memset(&q, 0, sizeof(q));
  gauss_legendre01(N, q.qx, q.qw);
  if (opt.nfine > 0) gauss_legendre01(opt.nfine, q.tu, q.wu);
  const size_t smem = sizeof(VecShared<N>);
  CUDA_TRY(cudaFuncSetAttribute(k_vector_lambert<N>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  int per_sm = 0;
  CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_vector_lambert<N>, 32, smem));
  if (per_sm < 1) return set_error(AERORT_RC_CUDA, "vector kernel does not fit on an SM");
  long nblocks = (long)per_sm * c.num_sms;
  if (nblocks > nsolve) nblocks = nsolve;
  const VecLayout<N> lay(in.km);
  const long per_warp = (lay.total + 31) / 32 * 32;
  if (int rc = c.pad->scratch.ensure(sizeof(double) * (size_t)per_warp * (size_t)nblocks)) return rc;
  if (int rc = c.pad->counter.ensure(4 * sizeof(int))) return rc;
  int* counter = (int*)c.pad->counter.p;
  int* first = counter + 1;
  k_init_sched<<<1, 1, 0, s>>>(counter, first, in.nobs, nullptr);
  k_nadir_first<<<(in.nobs + 127) / 128, 128, 0, s>>>(in.nobs, in.nch, in.sza, in.raa, in.vza, in.albedo, in.missing,
                                                       first);
  CUDA_TRY(cudaGetLastError());
  VectorInputs v2 = vin;
  v2.base.nadir_first = first;
  k_vector_lambert<N><<<(unsigned)nblocks, 32, smem, s>>>(opt, v2, q, (double*)c.pad->scratch.p, per_warp, nsolve,
                                                          counter, rad, refl, Qo, Uo, nf, st);
  CUDA_TRY(cudaGetLastError());
  count_launches(3);
  return 0;
}

int dispatch_vector(Context& c, int nstreams, const RtOptions& opt, const VectorInputs& vin, double* rad,
                    double* refl, double* Qo, double* Uo, int* nf, int* st, cudaStream_t s) {
  if (int rc = c.bind(s)) return rc;
  int rc = 0;
  switch (nstreams) {
    case 4: rc = launch_vector<4>(c, opt, vin, rad, refl, Qo, Uo, nf, st, s); break;
    case 6: rc = launch_vector<6>(c, opt, vin, rad, refl, Qo, Uo, nf, st, s); break;
    case 8: rc = launch_vector<8>(c, opt, vin, rad, refl, Qo, Uo, nf, st, s); break;
    case 12: rc = launch_vector<12>(c, opt, vin, rad, refl, Qo, Uo, nf, st, s); break;
    case 16: rc = launch_vector<16>(c, opt, vin, rad, refl, Qo, Uo, nf, st, s); break;
    default: rc = set_error(AERORT_RC_UNSUPPORTED, "vector_lambert: nstreams must be one of 4, 6, 8, 12, 16");
  }
  const int rc2 = c.unbind(s);
  return rc ? rc : rc2;
}

RtOptions vector_options(int plane_parallel) {
  RtOptions o;
  o.do_focorr = 1;            // VLIDORT_Mod.F90: DO_FOCORR / DO_FOCORR_OUTGOING
  o.do_deltam = 1;            // DO_DELTAM_SCALING
  o.do_plane_parallel = plane_parallel ? 1 : 0;
  o.do_double_convtest = 1;   // DO_DOUBLE_CONVTEST
  o.nfine = 3;                // NFINELAYERS
  o.taylor_order = 3;         // TAYLOR_ORDER
  o.accuracy = kAccuracySingle;
  o.earth_radius = 6371.0;
  o.flux_factor = 1.0;        // per pixel and channel from flux_factor(nch, nobs)
  o.max_fourier = -1;
  return o;
}

int vector_checks(int km, int nch, int nobs, int nstreams, int nMom, int nPol) {
  if (km <= 0 || nch <= 0 || nobs < 0) return set_error(AERORT_RC_ARG, "vector_lambert: bad sizes");
  if ((long long)nobs * nch > 0x7f000000LL)
    return set_error(AERORT_RC_ARG, "vector_lambert: nobs * nch too large (at most 2130706432 solves per call)");
  if (nstreams > 25) return set_error(AERORT_RC_NSTREAMS, "NSTREAMS > MAXSTREAMS");
  if (km > kMaxLayers) return set_error(AERORT_RC_NLAYERS, "NLAYERS > MAXLAYERS");
  if (nMom > 1000) return set_error(AERORT_RC_NMOMENTS, "nmom > MAXMOMENTS_INPUT");
  if (nMom < 1) return set_error(AERORT_RC_ARG, "vector_lambert: nMom must be >= 1");
  if (nPol != 6)
    return set_error(AERORT_RC_ARG, "vector_lambert: pmom must carry the 6 elements P11, P12, P33, P34, P22, P44");
  return 0;
}

}  // namespace
}  // namespace aerort_internal

extern "C" int aerort_vlidort_vector_lambert_batch_dev(
    int km, int nch, int nobs, int nstreams, int plane_parallel, int nMom, const int* nlay, const double* ROT,
    const double* depol, const double* alpha, const double* tau, const double* ssa, const double* pmom,
    const float* tau_f, const float* ssa_f, const float* pmom_f, const double* he, const double* albedo,
    const double* solar_zenith, const double* relat_azymuth, const double* sensor_zenith, const double* flux_factor,
    double MISSING, double* radiance_VL, double* reflectance_VL, double* Q, double* U, int* nfourier, int* status,
    void* stream) {
  if (int rc = vector_checks(km, nch, nobs, nstreams, nMom, 6)) return rc;
  if ((!tau_f && (!tau || !ssa || !pmom)) || (tau_f && (!ssa_f || !pmom_f)))
    return set_error(AERORT_RC_ARG, "vector_lambert_batch_dev: optics missing");
  if (!ROT || !depol || !he || !albedo || !solar_zenith || !relat_azymuth || !sensor_zenith || !radiance_VL ||
      !reflectance_VL || !Q || !U)
    return set_error(AERORT_RC_ARG, "vector_lambert_batch_dev: null array");
  Context& c = ctx();
  std::lock_guard<std::mutex> lk(c.mu);
  if (int rc = c.setup()) return rc;
  VectorInputs vin;
  vin.base = LambertInputs{km, nch, nobs, nMom, ROT, depol, tau, ssa, pmom, he, albedo, solar_zenith, relat_azymuth,
                           sensor_zenith, nlay, tau_f, ssa_f, pmom_f, nullptr, MISSING, alpha};
  vin.flux_factor = flux_factor;
  return dispatch_vector(c, nstreams, vector_options(plane_parallel), vin, radiance_VL, reflectance_VL, Q, U, nfourier,
                         status, (cudaStream_t)stream);
}

extern "C" int aerort_vlidort_vector_lambert_ex(int km, int nch, int nobs, const double* channels, int nstreams,
                                                int plane_parallel, int nMom, int nPol, const double* ROT,
                                                const double* depol, const double* alpha, const double* tau,
                                                const double* ssa, const double* pmom, const double* pe,
                                                const double* he, const double* te, const double* albedo,
                                                const double* solar_zenith, const double* relat_azymuth,
                                                const double* sensor_zenith, const double* flux_factor,
                                                double MISSING, int verbose, double* radiance_VL,
                                                double* reflectance_VL, double* Q, double* U, int* nfourier,
                                                int* status) {
  (void)channels; (void)pe; (void)te; (void)verbose;
  if (int rc = vector_checks(km, nch, nobs, nstreams, nMom, nPol)) return rc;
  if (!ROT || !depol || !tau || !ssa || !pmom || !he || !albedo || !solar_zenith || !relat_azymuth ||
      !sensor_zenith || !flux_factor || !radiance_VL || !reflectance_VL || !Q || !U)
    return set_error(AERORT_RC_ARG, "vector_lambert: null array");
  Context& c = ctx();
  std::lock_guard<std::mutex> lk(c.mu);
  if (int rc = c.setup()) return rc;
  cudaStream_t s = c.stream;
  const size_t nl = (size_t)km * nobs * nch, np = nl * nMom * 6, nh = (size_t)(km + 1) * nobs, nx = (size_t)nobs * nch;
  struct { const void* src; size_t bytes; } ins[] = {
      {ROT, 8 * nl}, {depol, 8 * (size_t)nch}, {alpha, alpha ? 8 * nl : 0}, {tau, 8 * nl}, {ssa, 8 * nl},
      {pmom, 8 * np}, {he, 8 * nh}, {albedo, 8 * nx}, {solar_zenith, 8 * (size_t)nobs},
      {relat_azymuth, 8 * (size_t)nobs}, {sensor_zenith, 8 * (size_t)nobs}, {flux_factor, 8 * nx}};
  const double* d[12];
  for (int k = 0; k < 12; ++k) {
    d[k] = nullptr;
    if (!ins[k].src) continue;
    if (int rc = c.stage[k].ensure(ins[k].bytes + 8)) return rc;
    CUDA_TRY(cudaMemcpyAsync(c.stage[k].p, ins[k].src, ins[k].bytes, cudaMemcpyHostToDevice, s));
    d[k] = (const double*)c.stage[k].p;
  }
  if (int rc = c.stage[12].ensure(32 * nx + 8 * nx + 8)) return rc;
  double* drad = (double*)c.stage[12].p;
  double* drefl = drad + nx;
  double* dq = drefl + nx;
  double* du = dq + nx;
  int* dnf = (int*)(du + nx);
  int* dst = dnf + nx;
  VectorInputs vin;
  vin.base = LambertInputs{km, nch, nobs, nMom, d[0], d[1], d[3], d[4], d[5], d[6], d[7], d[8], d[9], d[10],
                           nullptr, nullptr, nullptr, nullptr, nullptr, MISSING, d[2]};
  vin.flux_factor = d[11];
  if (int rc = dispatch_vector(c, nstreams, vector_options(plane_parallel), vin, drad, drefl, dq, du, dnf, dst, s))
    return rc;
  CUDA_TRY(cudaMemcpyAsync(radiance_VL, drad, 8 * nx, cudaMemcpyDeviceToHost, s));
  CUDA_TRY(cudaMemcpyAsync(reflectance_VL, drefl, 8 * nx, cudaMemcpyDeviceToHost, s));
  CUDA_TRY(cudaMemcpyAsync(Q, dq, 8 * nx, cudaMemcpyDeviceToHost, s));
  CUDA_TRY(cudaMemcpyAsync(U, du, 8 * nx, cudaMemcpyDeviceToHost, s));
  if (nfourier) CUDA_TRY(cudaMemcpyAsync(nfourier, dnf, 4 * nx, cudaMemcpyDeviceToHost, s));
  if (status) CUDA_TRY(cudaMemcpyAsync(status, dst, 4 * nx, cudaMemcpyDeviceToHost, s));
  CUDA_TRY(cudaStreamSynchronize(s));
  return AERORT_OK;
}

extern "C" int aerort_vlidort_vector_lambert(int km, int nch, int nobs, const double* channels, int nstreams,
                                             int plane_parallel, int nMom, int nPol, const double* ROT,
                                             const double* depol, const double* alpha, const double* tau,
                                             const double* ssa, const double* pmom, const double* pe,
                                             const double* he, const double* te, const double* albedo,
                                             const double* solar_zenith, const double* relat_azymuth,
                                             const double* sensor_zenith, const double* flux_factor, double MISSING,
                                             int verbose, double* radiance_VL, double* reflectance_VL, double* Q,
                                             double* U) {
  return aerort_vlidort_vector_lambert_ex(km, nch, nobs, channels, nstreams, plane_parallel, nMom, nPol, ROT, depol,
                                          alpha, tau, ssa, pmom, pe, he, te, albedo, solar_zenith, relat_azymuth,
                                          sensor_zenith, flux_factor, MISSING, verbose, radiance_VL, reflectance_VL, Q,
                                          U, nullptr, nullptr);
}
