// BRDF-surface entry points: VLIDORT_Scalar_LandMODIS
// (geo_vlidort/VLIDORT_BRDF_MODIS.F90:34-200), the scalar solve of
// VLIDORT_Scalar_Lambert over the MODIS RTLS BRDF, and VLIDORT_Scalar_CX /
// VLIDORT_Scalar_GissCX (geo_vlidort/VLIDORT_BRDF_CX.F90:420-584, :1553-1716),
// the same solve over the Cox-Munk / GISS Cox-Munk ocean glint (rt_brdf.cuh;
// kernels in rt_launch.cuh, one instantiation per stream count).
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <map>
#include <utility>
#include <vector>

#include "aerort_internal.cuh"

using namespace aerort;
using namespace aerort_internal;

namespace {

constexpr int kMaxBrdfTables = 256;

RtOptions brdf_options(int plane_parallel) {
  RtOptions o;
  o.do_focorr = 1;  // the VLIDORT_Init settings of the Lambertian wrapper (VLIDORT_Mod.F90:65-383)
  o.do_deltam = 1;
  o.do_plane_parallel = plane_parallel ? 1 : 0;
  o.do_double_convtest = 1;
  o.nfine = 3;
  o.taylor_order = 3;
  o.accuracy = kAccuracySingle;
  o.earth_radius = 6371.0;
  o.flux_factor = 1.0;
  o.max_fourier = -1;
  return o;
}

// Distinct Li-sparse parameter pairs of param(2, nch, nobs) (host): tab[i + nch j]
// is the table of solve (j, i); returns the number of tables or -1 if there
// are more than kMaxBrdfTables.
int brdf_param_tables(int nch, int nobs, const double* param, std::vector<int>& tab, std::vector<double>& tpar) {
  std::map<std::pair<double, double>, int> seen;
  const size_t n = (size_t)nch * nobs;
  tab.resize(n);
  tpar.clear();
  for (size_t w = 0; w < n; ++w) {
    const std::pair<double, double> key(param[2 * w], param[2 * w + 1]);
    auto it = seen.find(key);
    if (it == seen.end()) {
      if ((int)seen.size() == kMaxBrdfTables) return -1;
      it = seen.emplace(key, (int)seen.size()).first;
      tpar.push_back(key.first);
      tpar.push_back(key.second);
    }
    tab[w] = it->second;
  }
  return (int)seen.size();
}

int dispatch_brdf(Context& c, int nstreams, const RtOptions& opt, const LambertInputs& in, const BrdfSurface& sf,
                  double* rad, double* refl, double* br, int* nf, int* st, cudaStream_t s) {
  if (int rc = c.bind(s)) return rc;
  int rc = 0;
  switch (nstreams) {
    case 4: rc = launch_scalar_brdf<4>(c, opt, in, sf, rad, refl, br, nf, st, s); break;
    case 6: rc = launch_scalar_brdf<6>(c, opt, in, sf, rad, refl, br, nf, st, s); break;
    case 8: rc = launch_scalar_brdf<8>(c, opt, in, sf, rad, refl, br, nf, st, s); break;
    case 12: rc = launch_scalar_brdf<12>(c, opt, in, sf, rad, refl, br, nf, st, s); break;
    case 16: rc = launch_scalar_brdf<16>(c, opt, in, sf, rad, refl, br, nf, st, s); break;
    default: rc = set_error(AERORT_RC_UNSUPPORTED, "nstreams must be one of 4, 6, 8, 12, 16");
  }
  const int rc2 = c.unbind(s);
  return rc ? rc : rc2;
}

int dispatch_landmodis(Context& c, int nstreams, const RtOptions& opt, const LambertInputs& in, const double* kw,
                       const double* param_host, double* rad, double* refl, double* br, int* nf, int* st,
                       cudaStream_t s) {
  std::vector<int> tab;
  std::vector<double> tpar;
  const int ntab = brdf_param_tables(in.nch, in.nobs, param_host, tab, tpar);
  if (ntab < 0)
    return set_error(AERORT_RC_ARG, "scalar_landmodis: more than 256 distinct Li-sparse parameter pairs in one call");
  if (ntab == 0) tpar.assign(2, 0.0);  // no solves
  BrdfSurface sf;
  sf.kind = kBrdfRTLS;
  sf.kw = kw;
  sf.tab_host = ntab > 1 ? tab.data() : nullptr;
  sf.tpar_host = tpar.data();
  sf.ntab = ntab ? ntab : 1;
  return dispatch_brdf(c, nstreams, opt, in, sf, rad, refl, br, nf, st, s);
}

}  // namespace

extern "C" int aerort_vlidort_scalar_landmodis_batch_dev(
    int km, int nch, int nobs, int nstreams, int plane_parallel, int nMom, const int* nlay, const double* ROT,
    const double* depol, const double* tau, const double* ssa, const double* pmom, const float* tau_f,
    const float* ssa_f, const float* pmom_f, const double* he, const double* kernel_wt, const double* param_host,
    const double* solar_zenith, const double* relat_azymuth, const double* sensor_zenith, double MISSING,
    double* radiance_VL_SURF, double* reflectance_VL_SURF, double* BR, int* nfourier, int* status, void* stream) {
  if (int rc = lambert_checks(km, nch, nobs, nstreams, nMom)) return rc;
  if ((!tau_f && (!tau || !ssa || !pmom)) || (tau_f && (!ssa_f || !pmom_f)))
    return set_error(AERORT_RC_ARG, "scalar_landmodis_batch_dev: optics missing");
  if (!kernel_wt || !param_host || !BR) return set_error(AERORT_RC_ARG, "scalar_landmodis_batch_dev: null array");
  Context& c = ctx();
  std::lock_guard<std::mutex> lk(c.mu);
  if (int rc = c.setup()) return rc;
  LambertInputs in{km, nch, nobs, nMom, ROT, depol, tau, ssa, pmom, he, nullptr, solar_zenith, relat_azymuth,
                   sensor_zenith, nlay, tau_f, ssa_f, pmom_f, nullptr, MISSING};
  return dispatch_landmodis(c, nstreams, brdf_options(plane_parallel), in, kernel_wt, param_host,
                            radiance_VL_SURF, reflectance_VL_SURF, BR, nfourier, status, (cudaStream_t)stream);
}

extern "C" int aerort_vlidort_scalar_landmodis_ex(
    int km, int nch, int nobs, const double* channels, int nstreams, int plane_parallel, int nMom, int nPol,
    const double* ROT, const double* depol, const double* tau, const double* ssa, const double* g,
    const double* pmom, const double* pe, const double* he, const double* te, const double* kernel_wt,
    const double* param, const double* solar_zenith, const double* relat_azymuth, const double* sensor_zenith,
    double MISSING, int verbose, double* radiance_VL_SURF, double* reflectance_VL_SURF, double* BR, int* nfourier,
    int* status) {
  (void)channels; (void)nPol; (void)g; (void)pe; (void)te; (void)verbose;
  if (int rc = lambert_checks(km, nch, nobs, nstreams, nMom)) return rc;
  if (!ROT || !depol || !tau || !ssa || !pmom || !he || !kernel_wt || !param || !solar_zenith || !relat_azymuth ||
      !sensor_zenith || !radiance_VL_SURF || !reflectance_VL_SURF || !BR)
    return set_error(AERORT_RC_ARG, "scalar_landmodis: null array");
  Context& c = ctx();
  std::lock_guard<std::mutex> lk(c.mu);
  if (int rc = c.setup()) return rc;
  cudaStream_t s = c.stream;
  const size_t nl = (size_t)km * nobs * nch, np = nl * nMom, nh = (size_t)(km + 1) * nobs, nx = (size_t)nobs * nch;
  struct { const void* src; size_t bytes; } ins[] = {
      {ROT, 8 * nl}, {depol, 8 * (size_t)nch}, {tau, 8 * nl}, {ssa, 8 * nl}, {pmom, 8 * np}, {he, 8 * nh},
      {kernel_wt, 8 * 3 * nx}, {solar_zenith, 8 * (size_t)nobs}, {relat_azymuth, 8 * (size_t)nobs},
      {sensor_zenith, 8 * (size_t)nobs}};
  const double* d[10];
  for (int k = 0; k < 10; ++k) {
    if (int rc = c.stage[k].ensure(ins[k].bytes + 8)) return rc;
    CUDA_TRY(cudaMemcpyAsync(c.stage[k].p, ins[k].src, ins[k].bytes, cudaMemcpyHostToDevice, s));
    d[k] = (const double*)c.stage[k].p;
  }
  if (int rc = c.stage[10].ensure(24 * nx + 8 * nx + 8)) return rc;
  double* drad = (double*)c.stage[10].p;
  double* drefl = drad + nx;
  double* dbr = drefl + nx;
  int* dnf = (int*)(dbr + nx);
  int* dst = dnf + nx;
  LambertInputs in{km, nch, nobs, nMom, d[0], d[1], d[2], d[3], d[4], d[5], nullptr, d[7], d[8], d[9],
                   nullptr, nullptr, nullptr, nullptr, nullptr, MISSING};
  if (int rc = dispatch_landmodis(c, nstreams, brdf_options(plane_parallel), in, d[6], param, drad, drefl, dbr,
                                  dnf, dst, s))
    return rc;
  CUDA_TRY(cudaMemcpyAsync(radiance_VL_SURF, drad, 8 * nx, cudaMemcpyDeviceToHost, s));
  CUDA_TRY(cudaMemcpyAsync(reflectance_VL_SURF, drefl, 8 * nx, cudaMemcpyDeviceToHost, s));
  CUDA_TRY(cudaMemcpyAsync(BR, dbr, 8 * nx, cudaMemcpyDeviceToHost, s));
  if (nfourier) CUDA_TRY(cudaMemcpyAsync(nfourier, dnf, 4 * nx, cudaMemcpyDeviceToHost, s));
  if (status) CUDA_TRY(cudaMemcpyAsync(status, dst, 4 * nx, cudaMemcpyDeviceToHost, s));
  CUDA_TRY(cudaStreamSynchronize(s));
  return AERORT_OK;
}

extern "C" int aerort_vlidort_scalar_landmodis(
    int km, int nch, int nobs, const double* channels, int nstreams, int plane_parallel, int nMom, int nPol,
    const double* ROT, const double* depol, const double* tau, const double* ssa, const double* g,
    const double* pmom, const double* pe, const double* he, const double* te, const double* kernel_wt,
    const double* param, const double* solar_zenith, const double* relat_azymuth, const double* sensor_zenith,
    double MISSING, int verbose, double* radiance_VL_SURF, double* reflectance_VL_SURF, double* BR) {
  return aerort_vlidort_scalar_landmodis_ex(km, nch, nobs, channels, nstreams, plane_parallel, nMom, nPol, ROT, depol,
                                            tau, ssa, g, pmom, pe, he, te, kernel_wt, param, solar_zenith,
                                            relat_azymuth, sensor_zenith, MISSING, verbose, radiance_VL_SURF,
                                            reflectance_VL_SURF, BR, nullptr, nullptr);
}

namespace {

int glint_batch_dev(
    int kind, int km, int nch, int nobs, int nstreams, int plane_parallel, int nMom, const int* nlay, const double* ROT,
    const double* depol, const double* tau, const double* ssa, const double* pmom, const float* tau_f,
    const float* ssa_f, const float* pmom_f, const double* he, const double* U10m, const double* V10m,
    const double* mr, const double* solar_zenith, const double* relat_azymuth, const double* sensor_zenith,
    double MISSING, double* radiance_VL_SURF, double* reflectance_VL_SURF, double* BRDF, int* nfourier, int* status,
    void* stream) {
  if (int rc = lambert_checks(km, nch, nobs, nstreams, nMom)) return rc;
  if ((!tau_f && (!tau || !ssa || !pmom)) || (tau_f && (!ssa_f || !pmom_f)))
    return set_error(AERORT_RC_ARG, "scalar_(giss)cx_batch_dev: optics missing");
  if (!U10m || !V10m || !mr || !BRDF) return set_error(AERORT_RC_ARG, "scalar_(giss)cx_batch_dev: null array");
  Context& c = ctx();
  std::lock_guard<std::mutex> lk(c.mu);
  if (int rc = c.setup()) return rc;
  LambertInputs in{km, nch, nobs, nMom, ROT, depol, tau, ssa, pmom, he, nullptr, solar_zenith, relat_azymuth,
                   sensor_zenith, nlay, tau_f, ssa_f, pmom_f, nullptr, MISSING};
  BrdfSurface sf;
  sf.kind = kind;
  sf.u10 = U10m;
  sf.v10 = V10m;
  sf.mr = mr;
  return dispatch_brdf(c, nstreams, brdf_options(plane_parallel), in, sf, radiance_VL_SURF, reflectance_VL_SURF,
                       BRDF, nfourier, status, (cudaStream_t)stream);
}

int glint_ex(
    int kind, int km, int nch, int nobs, const double* channels, int nstreams, int plane_parallel, int nMom, int nPol,
    const double* ROT, const double* depol, const double* tau, const double* ssa, const double* g,
    const double* pmom, const double* pe, const double* he, const double* te, const double* U10m,
    const double* V10m, const double* mr, const double* solar_zenith, const double* relat_azymuth,
    const double* sensor_zenith, double MISSING, int verbose, double* radiance_VL_SURF, double* reflectance_VL_SURF,
    double* BRDF, int* nfourier, int* status) {
  (void)channels; (void)nPol; (void)g; (void)pe; (void)te; (void)verbose;
  if (int rc = lambert_checks(km, nch, nobs, nstreams, nMom)) return rc;
  if (!ROT || !depol || !tau || !ssa || !pmom || !he || !U10m || !V10m || !mr || !solar_zenith || !relat_azymuth ||
      !sensor_zenith || !radiance_VL_SURF || !reflectance_VL_SURF || !BRDF)
    return set_error(AERORT_RC_ARG, "scalar_(giss)cx: null array");
  Context& c = ctx();
  std::lock_guard<std::mutex> lk(c.mu);
  if (int rc = c.setup()) return rc;
  cudaStream_t s = c.stream;
  const size_t nl = (size_t)km * nobs * nch, np = nl * nMom, nh = (size_t)(km + 1) * nobs, nx = (size_t)nobs * nch;
  struct { const void* src; size_t bytes; } ins[] = {
      {ROT, 8 * nl}, {depol, 8 * (size_t)nch}, {tau, 8 * nl}, {ssa, 8 * nl}, {pmom, 8 * np}, {he, 8 * nh},
      {solar_zenith, 8 * (size_t)nobs}, {relat_azymuth, 8 * (size_t)nobs}, {sensor_zenith, 8 * (size_t)nobs},
      {U10m, 8 * (size_t)nobs}, {V10m, 8 * (size_t)nobs}, {mr, 8 * (size_t)nch}};
  constexpr int kIn = sizeof(ins) / sizeof(ins[0]);
  const double* d[kIn];
  for (int k = 0; k < kIn; ++k) {
    if (int rc = c.stage[k].ensure(ins[k].bytes + 8)) return rc;
    CUDA_TRY(cudaMemcpyAsync(c.stage[k].p, ins[k].src, ins[k].bytes, cudaMemcpyHostToDevice, s));
    d[k] = (const double*)c.stage[k].p;
  }
  if (int rc = c.stage[kIn].ensure(24 * nx + 8 * nx + 8)) return rc;
  double* drad = (double*)c.stage[kIn].p;
  double* drefl = drad + nx;
  double* dbr = drefl + nx;
  int* dnf = (int*)(dbr + nx);
  int* dst = dnf + nx;
  LambertInputs in{km, nch, nobs, nMom, d[0], d[1], d[2], d[3], d[4], d[5], nullptr, d[6], d[7], d[8],
                   nullptr, nullptr, nullptr, nullptr, nullptr, MISSING};
  BrdfSurface sf;
  sf.kind = kind;
  sf.u10 = d[9];
  sf.v10 = d[10];
  sf.mr = d[11];
  if (int rc = dispatch_brdf(c, nstreams, brdf_options(plane_parallel), in, sf, drad, drefl, dbr, dnf, dst, s))
    return rc;
  CUDA_TRY(cudaMemcpyAsync(radiance_VL_SURF, drad, 8 * nx, cudaMemcpyDeviceToHost, s));
  CUDA_TRY(cudaMemcpyAsync(reflectance_VL_SURF, drefl, 8 * nx, cudaMemcpyDeviceToHost, s));
  CUDA_TRY(cudaMemcpyAsync(BRDF, dbr, 8 * nx, cudaMemcpyDeviceToHost, s));
  if (nfourier) CUDA_TRY(cudaMemcpyAsync(nfourier, dnf, 4 * nx, cudaMemcpyDeviceToHost, s));
  if (status) CUDA_TRY(cudaMemcpyAsync(status, dst, 4 * nx, cudaMemcpyDeviceToHost, s));
  CUDA_TRY(cudaStreamSynchronize(s));
  return AERORT_OK;
}

}  // namespace

#define AERORT_GLINT_ENTRIES(NAME, KIND)                                                                          \
  extern "C" int aerort_vlidort_scalar_##NAME##_batch_dev(                                                       \
      int km, int nch, int nobs, int nstreams, int plane_parallel, int nMom, const int* nlay, const double* ROT,  \
      const double* depol, const double* tau, const double* ssa, const double* pmom, const float* tau_f,          \
      const float* ssa_f, const float* pmom_f, const double* he, const double* U10m, const double* V10m,          \
      const double* mr, const double* solar_zenith, const double* relat_azymuth, const double* sensor_zenith,    \
      double MISSING, double* radiance_VL_SURF, double* reflectance_VL_SURF, double* BRDF, int* nfourier,         \
      int* status, void* stream) {                                                                                \
    return glint_batch_dev(KIND, km, nch, nobs, nstreams, plane_parallel, nMom, nlay, ROT, depol, tau, ssa, pmom, \
                           tau_f, ssa_f, pmom_f, he, U10m, V10m, mr, solar_zenith, relat_azymuth, sensor_zenith, \
                           MISSING, radiance_VL_SURF, reflectance_VL_SURF, BRDF, nfourier, status, stream);       \
  }                                                                                                               \
  extern "C" int aerort_vlidort_scalar_##NAME##_ex(                                                              \
      int km, int nch, int nobs, const double* channels, int nstreams, int plane_parallel, int nMom, int nPol,    \
      const double* ROT, const double* depol, const double* tau, const double* ssa, const double* g,              \
      const double* pmom, const double* pe, const double* he, const double* te, const double* U10m,              \
      const double* V10m, const double* mr, const double* solar_zenith, const double* relat_azymuth,             \
      const double* sensor_zenith, double MISSING, int verbose, double* radiance_VL_SURF,                         \
      double* reflectance_VL_SURF, double* BRDF, int* nfourier, int* status) {                                    \
    return glint_ex(KIND, km, nch, nobs, channels, nstreams, plane_parallel, nMom, nPol, ROT, depol, tau, ssa, g, \
                    pmom, pe, he, te, U10m, V10m, mr, solar_zenith, relat_azymuth, sensor_zenith, MISSING,       \
                    verbose, radiance_VL_SURF, reflectance_VL_SURF, BRDF, nfourier, status);                      \
  }                                                                                                               \
  extern "C" int aerort_vlidort_scalar_##NAME(                                                                   \
      int km, int nch, int nobs, const double* channels, int nstreams, int plane_parallel, int nMom, int nPol,    \
      const double* ROT, const double* depol, const double* tau, const double* ssa, const double* g,              \
      const double* pmom, const double* pe, const double* he, const double* te, const double* U10m,              \
      const double* V10m, const double* mr, const double* solar_zenith, const double* relat_azymuth,             \
      const double* sensor_zenith, double MISSING, int verbose, double* radiance_VL_SURF,                         \
      double* reflectance_VL_SURF, double* BRDF) {                                                                \
    return glint_ex(KIND, km, nch, nobs, channels, nstreams, plane_parallel, nMom, nPol, ROT, depol, tau, ssa, g, \
                    pmom, pe, he, te, U10m, V10m, mr, solar_zenith, relat_azymuth, sensor_zenith, MISSING,       \
                    verbose, radiance_VL_SURF, reflectance_VL_SURF, BRDF, nullptr, nullptr);                      \
  }

// VLIDORT_Scalar_CX (VLIDORT_BRDF_CX.F90:420-584) and VLIDORT_Scalar_GissCX
// (:1553-1716): the same wrapper over the Cox-Munk and the GISS Cox-Munk kernel
AERORT_GLINT_ENTRIES(cx, kBrdfCoxMunk)
AERORT_GLINT_ENTRIES(gisscx, kBrdfGissCoxMunk)
