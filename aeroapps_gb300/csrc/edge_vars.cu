// Edge pressure, height and temperature of model columns on the device: the
// reference's getEdgeVars (src/Shared/GMAO_Shared/Chem_Base/MieObs_py.F90:27-83),
// which turns layer air density and pressure thickness into the km+1 edge
// profiles that the Rayleigh calculator and the RT take.  Default REAL
// (FP32) throughout, as in the reference.
//
// pe and ze are sums, products and quotients evaluated in the reference's
// order with explicitly rounded FP32 intrinsics (no FMA contraction): they are
// bit-identical.  te also needs a logarithm and a real power; CUDA's logf/powf
// and a host libm may differ in the last bits, so te agrees to within a few
// units in the last place.
//
// Layout: one thread per column, one warp of 32 columns per block.  The 32
// columns of a block are contiguous in the (km, nobs) inputs and in the
// (km+1, nobs) outputs, so they move between HBM and shared memory as whole
// coalesced chunks, with several loads in flight per lane; each thread then
// walks its own column in shared memory (odd column stride, so the 32 lanes
// hit 32 banks).  Three column arrays per block: pe has its own; ze
// overwrites delp and te overwrites airdens as each layer's input is used
// for the last time (ze walks up from the surface, te down from the top), so
// a block takes 27 KB at 72 layers and eight blocks fit an SM.
#include "aerort_internal.cuh"

namespace aerort_internal {
namespace {

constexpr int kEdgeCols = 32;
constexpr int kBatch = 9;  // loads in flight per lane and input (72-layer chunk: 2304 words = 8 x 9 x 32)
constexpr float kGrav = 9.80616f;
constexpr float kRgas = 287.0f;
constexpr float kKappa = 2.0f / 7.0f;  // REAL parameter 2.0/7.0, a single-precision quotient

__host__ __device__ inline int odd_stride(int n) { return n | 1; }

size_t edge_smem_bytes(int km) { return sizeof(float) * (size_t)kEdgeCols * 3 * (size_t)odd_stride(km + 1); }

__global__ void __launch_bounds__(kEdgeCols) k_edge_vars(int km, int nobs, const float* __restrict__ airdens,
                                                         const float* __restrict__ delp, float ptop,
                                                         float* __restrict__ pe, float* __restrict__ ze,
                                                         float* __restrict__ te) {
  extern __shared__ float sm[];
  const int ks = odd_stride(km + 1), es = ks;  // km + 1 slots per column in every array
  float* s_rho = sm;                  // airdens, then te
  float* s_dp = s_rho + kEdgeCols * ks;  // delp, then ze
  float* s_pe = s_dp + kEdgeCols * ks;
  float* s_ze = s_dp;
  float* s_te = s_rho;
  const int lane = threadIdx.x;
  for (long c0 = (long)blockIdx.x * kEdgeCols; c0 < nobs; c0 += (long)gridDim.x * kEdgeCols) {
    const int nc = (int)min((long)kEdgeCols, (long)nobs - c0);
    // the block's nc columns are one contiguous chunk of nc*km words per input:
    // each lane issues kBatch loads of both inputs before it stores any
    const int nin = nc * km;
    const float* a = airdens + c0 * km;
    const float* d = delp + c0 * km;
    for (int base = lane; base < nin; base += kEdgeCols * kBatch) {
      float va[kBatch], vd[kBatch];
#pragma unroll
      for (int u = 0; u < kBatch; ++u) {
        const int i = base + u * kEdgeCols;
        if (i < nin) {
          va[u] = a[i];
          vd[u] = d[i];
        }
      }
#pragma unroll
      for (int u = 0; u < kBatch; ++u) {
        const int i = base + u * kEdgeCols;
        if (i < nin) {
          const int j = i / km, k = i - j * km;
          s_rho[j * ks + k] = va[u];
          s_dp[j * ks + k] = vd[u];
        }
      }
    }
    __syncwarp();
    if (lane < nc) {
      float* R = s_rho + lane * ks;  // airdens; te in place (T[k] after R[k]'s last use)
      float* D = s_dp + lane * ks;   // delp; ze in place (Z[k] after D[k]'s last use)
      float* P = s_pe + lane * es;
      float* Z = D;
      float* T = R;
      P[0] = ptop;
      for (int k = 0; k < km; ++k) P[k + 1] = __fadd_rn(P[k], D[k]);
      Z[km] = 0.0f;  // height above the surface
      for (int k = km - 1; k >= 0; --k) Z[k] = __fadd_rn(Z[k + 1], __fdiv_rn(D[k], __fmul_rn(R[k], kGrav)));
      // layer mid pressure and temperature, carried one layer behind
      float pm_prev = __fdiv_rn(__fadd_rn(P[0], P[1]), 2.0f);
      float tm_prev = __fdiv_rn(pm_prev, __fmul_rn(R[0], kRgas));
      T[0] = tm_prev;  // isothermal at the top edge
      for (int k = 1; k < km; ++k) {
        const float pm = __fdiv_rn(__fadd_rn(P[k], P[k + 1]), 2.0f);
        const float tm = __fdiv_rn(pm, __fmul_rn(R[k], kRgas));
        const float alpha = __fdiv_rn(logf(__fdiv_rn(P[k], pm_prev)), logf(__fdiv_rn(pm, pm_prev)));
        T[k] = __fadd_rn(tm_prev, __fmul_rn(alpha, __fsub_rn(tm, tm_prev)));
        pm_prev = pm;
        tm_prev = tm;
      }
      T[km] = __fmul_rn(tm_prev, powf(__fdiv_rn(P[km], pm_prev), kKappa));  // dry adiabatic at the surface
    }
    __syncwarp();
    // outputs: one contiguous chunk of nc*(km+1) words each
    const int ne = km + 1, nout = nc * ne;
    const long o = c0 * ne;
    for (int i = lane; i < nout; i += kEdgeCols) {
      const int j = i / ne, k = i - j * ne;
      pe[o + i] = s_pe[j * es + k];
      ze[o + i] = s_ze[j * es + k];
      te[o + i] = s_te[j * es + k];
    }
    __syncwarp();
  }
}

int edge_checks(int km, int nobs) {
  if (km <= 0 || nobs < 0) return set_error(AERORT_RC_ARG, "get_edge_vars: bad sizes");
  if (edge_smem_bytes(km) > 200 * 1024) return set_error(AERORT_RC_NLAYERS, "get_edge_vars: km too large");
  return 0;
}

int launch_edge(int km, int nobs, const float* airdens, const float* delp, float ptop, float* pe, float* ze,
                float* te, cudaStream_t s, int num_sms) {
  if (nobs == 0) return 0;
  const size_t smem = edge_smem_bytes(km);
  if (smem > 48 * 1024)
    CUDA_TRY(cudaFuncSetAttribute(k_edge_vars, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  long blocks = (nobs + kEdgeCols - 1) / kEdgeCols;
  const long per_sm = (long)((227 * 1024) / smem);
  const long cap = (long)num_sms * (per_sm > 0 ? per_sm : 1);  // one resident wave
  if (blocks > cap) blocks = cap;
  k_edge_vars<<<(unsigned)blocks, kEdgeCols, smem, s>>>(km, nobs, airdens, delp, ptop, pe, ze, te);
  CUDA_TRY(cudaGetLastError());
  count_launches(1);
  return 0;
}

}  // namespace
}  // namespace aerort_internal

using namespace aerort_internal;

extern "C" int aerort_get_edge_vars_dev(int km, int nobs, const float* airdens, const float* delp, float ptop,
                                        float* pe, float* ze, float* te, void* stream) {
  if (int rc = edge_checks(km, nobs)) return rc;
  if (!airdens || !delp || !pe || !ze || !te) return set_error(AERORT_RC_ARG, "get_edge_vars_dev: null array");
  Context& c = ctx();
  int num_sms = 0;
  {
    std::lock_guard<std::mutex> lk(c.mu);
    if (int rc = c.setup()) return rc;
    num_sms = c.num_sms;
  }
  return launch_edge(km, nobs, airdens, delp, ptop, pe, ze, te, (cudaStream_t)stream, num_sms);
}

extern "C" int aerort_get_edge_vars(int km, int nobs, const float* airdens, const float* delp, float ptop, float* pe,
                                    float* ze, float* te) {
  if (int rc = edge_checks(km, nobs)) return rc;
  if (!airdens || !delp || !pe || !ze || !te) return set_error(AERORT_RC_ARG, "get_edge_vars: null array");
  Context& c = ctx();
  std::lock_guard<std::mutex> lk(c.mu);
  if (int rc = c.setup()) return rc;
  cudaStream_t s = c.stream;
  const size_t nl = (size_t)km * nobs, ne = (size_t)(km + 1) * nobs;
  // staging buffers 21..22 are this entry point's
  if (int rc = c.stage[21].ensure(4 * 2 * nl + 16)) return rc;
  if (int rc = c.stage[22].ensure(4 * 3 * ne + 16)) return rc;
  float* drho = (float*)c.stage[21].p;
  float* ddp = drho + nl;
  float* dpe = (float*)c.stage[22].p;
  float* dze = dpe + ne;
  float* dte = dze + ne;
  if (nobs > 0) {
    CUDA_TRY(cudaMemcpyAsync(drho, airdens, 4 * nl, cudaMemcpyHostToDevice, s));
    CUDA_TRY(cudaMemcpyAsync(ddp, delp, 4 * nl, cudaMemcpyHostToDevice, s));
  }
  if (int rc = launch_edge(km, nobs, drho, ddp, ptop, dpe, dze, dte, s, c.num_sms)) return rc;
  if (nobs > 0) {
    CUDA_TRY(cudaMemcpyAsync(pe, dpe, 4 * ne, cudaMemcpyDeviceToHost, s));
    CUDA_TRY(cudaMemcpyAsync(ze, dze, 4 * ne, cudaMemcpyDeviceToHost, s));
    CUDA_TRY(cudaMemcpyAsync(te, dte, 4 * ne, cudaMemcpyDeviceToHost, s));
  }
  CUDA_TRY(cudaStreamSynchronize(s));
  return AERORT_OK;
}
