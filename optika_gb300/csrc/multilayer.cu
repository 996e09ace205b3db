// Standalone multilayer efficiency kernel (optika.materials.multilayer_efficiency).
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/optika_gb300.h"
#include "trace_device.cuh"

namespace otx {

struct MLArgs {
  int64_t count;
  const float* wl;
  int64_t s_wl;
  const float* cosv;
  int64_t s_cos;
  const float* n_re;
  const float* n_im;
  int64_t s_n;
  const int32_t* stack;
  float *rs, *rp, *ts, *tp;
};

__global__ void __launch_bounds__(256)
    k_multilayer(const __grid_constant__ otx_system sys, const __grid_constant__ MLArgs a) {
  const int64_t step = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < a.count; i += step) {
    const float wl = a.wl[i * a.s_wl];
    const float c0 = a.cosv[i * a.s_cos];
    const cf n0{a.n_re ? a.n_re[i * a.s_n] : 1.f, a.n_im ? a.n_im[i * a.s_n] : 0.f};
    int k = a.stack ? a.stack[i] : 0;
    k = (k < 0 || k >= OTX_MAX_STACKS) ? 0 : k;
    float Rs, Rp, Ts, Tp;
    multilayer(sys, sys.stacks[k], wl, c0, n0, Rs, Rp, Ts, Tp);
    if (a.rs) a.rs[i] = Rs;
    if (a.rp) a.rp[i] = Rp;
    if (a.ts) a.ts[i] = Ts;
    if (a.tp) a.tp[i] = Tp;
  }
}

}  // namespace otx

using namespace otx;

extern "C" otx_status otx_multilayer_efficiency(
    const otx_system* sys, int64_t count, const float* wavelength, int64_t stride_wavelength,
    const float* cos_incidence, int64_t stride_cos, const float* n_re, const float* n_im,
    int64_t stride_n, const int32_t* stack_index, float* r_s, float* r_p, float* t_s,
    float* t_p, void* stream) {
  if (!sys || sys->abi_version != OTX_ABI_VERSION) return OTX_ERR_INVALID;
  if (count < 0) return OTX_ERR_INVALID;
  if (count == 0) return OTX_OK;
  if (!wavelength || !cos_incidence) return OTX_ERR_INVALID;
  if (stride_wavelength < 0 || stride_cos < 0 || stride_n < 0) return OTX_ERR_INVALID;
  for (int k = 0; k < OTX_MAX_STACKS; ++k) {
    const otx_stack& K = sys->stacks[k];
    if (K.pre_count < 0 || K.per_count < 0 || K.post_count < 0 || K.num_periods < 0)
      return OTX_ERR_INVALID;
    if (K.pre_count && (K.pre_begin < 0 || K.pre_begin + K.pre_count > OTX_MAX_LAYERS))
      return OTX_ERR_INVALID;
    if (K.per_count && (K.per_begin < 0 || K.per_begin + K.per_count > OTX_MAX_LAYERS))
      return OTX_ERR_INVALID;
    if (K.post_count && (K.post_begin < 0 || K.post_begin + K.post_count > OTX_MAX_LAYERS))
      return OTX_ERR_INVALID;
    if (K.substrate >= OTX_MAX_LAYERS) return OTX_ERR_INVALID;
  }
  for (int k = 0; k < OTX_MAX_LAYERS; ++k) {
    const int t = sys->layers[k].table;
    if (t >= OTX_MAX_STACKS * 4) return OTX_ERR_INVALID;
    if (t >= 0 && (sys->tables[t].count < 1 || sys->table_data == 0)) return OTX_ERR_INVALID;
  }
  MLArgs a{count, wavelength, stride_wavelength, cos_incidence, stride_cos, n_re, n_im,
           stride_n, stack_index, r_s, r_p, t_s, t_p};
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (sms <= 0) sms = 132;
  int64_t need = (count + 255) / 256;
  const int64_t cap = (int64_t)sms * 16;
  const int grid = (int)(need < cap ? need : cap);
  k_multilayer<<<grid, 256, 0, reinterpret_cast<cudaStream_t>(stream)>>>(*sys, a);
  return cudaGetLastError() == cudaSuccess ? OTX_OK : OTX_ERR_CUDA;
}
