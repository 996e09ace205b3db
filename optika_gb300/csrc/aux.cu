// Standalone sensor binning and sag evaluation, sharing the device functions
// of the fused trace.
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/optika_gb300.h"
#include "trace_device.cuh"
#include "trace_kernel_decl.h"

namespace otx {

__device__ __forceinline__ int64_t collect_bin(const otx_sensor& S, float x, float y,
                                               float wl) {
  const float hx = S.lo_x + S.num_x * S.width_x;
  const float hy = S.lo_y + S.num_y * S.width_y;
  if (!(x >= S.lo_x && x <= hx && y >= S.lo_y && y <= hy)) return -1;
  int ix = (int)floorf((x - S.lo_x) * S.inv_width_x);
  int iy = (int)floorf((y - S.lo_y) * S.inv_width_y);
  ix = min(max(ix, 0), S.num_x - 1);
  iy = min(max(iy, 0), S.num_y - 1);
  int iw = 0;
  if (S.w_hi > S.w_lo) {
    if (!(wl >= S.w_lo && wl <= S.w_hi)) return -1;
    iw = (int)floorf((wl - S.w_lo) * S.inv_width_w);
    iw = min(max(iw, 0), S.num_w - 1);
  }
  return ((int64_t)iw * S.num_x + ix) * S.num_y + iy;
}

// optika/sensors/_sensors.py:92-169: histogram of position.xy (and
// wavelength) weighted by intensity * unvignetted, and of the same weight
// times the cosine of incidence dz (flat sensor, normal -z).
__global__ void k_collect(const otx_sensor S, const otx_rays r, const otx_image img) {
  const int64_t step = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < r.count; i += step) {
    if (r.unvignetted && reinterpret_cast<const uint8_t*>(r.unvignetted)[i] == 0) continue;
    const float x = reinterpret_cast<const float*>(r.px)[i];
    const float y = reinterpret_cast<const float*>(r.py)[i];
    const float wl = r.wavelength ? reinterpret_cast<const float*>(r.wavelength)[i] : 0.f;
    const int64_t b = collect_bin(S, x, y, wl);
    if (b < 0) continue;
    if (img.counts) atomicAdd(reinterpret_cast<unsigned int*>(img.counts) + b, 1u);
    const float w = r.intensity ? reinterpret_cast<const float*>(r.intensity)[i] : 1.f;
    if (img.flux) atomicAdd(reinterpret_cast<float*>(img.flux) + b, w);
    if (img.cos_moment) {
      const float dz = r.dz ? reinterpret_cast<const float*>(r.dz)[i] : 1.f;
      atomicAdd(reinterpret_cast<float*>(img.cos_moment) + b, w * dz);
    }
  }
}

// mode 0: sag z(x, y) -> out.pz ; 1: normal -> out.d* ; 2: intercept -> out.p*
__global__ void k_sag(const __grid_constant__ otx_system sys, const int mode,
                      const otx_rays in, const otx_rays out) {
  const otx_surface& s = sys.surfaces[0];
  const int64_t step = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < in.count; i += step) {
    const float x = reinterpret_cast<const float*>(in.px)[i];
    const float y = reinterpret_cast<const float*>(in.py)[i];
    if (mode == 0) {
      float gx, gy;
      float z = sag_eval(s.sag_type, s, x, y, gx, gy);
      reinterpret_cast<float*>(out.pz)[i] = z;
    } else if (mode == 1) {
      float nx, ny, nz, v[3];
      normal(s.sag_type, s, x, y, nx, ny, nz, v);
      reinterpret_cast<float*>(out.dx)[i] = nx;
      reinterpret_cast<float*>(out.dy)[i] = ny;
      reinterpret_cast<float*>(out.dz)[i] = nz;
    } else {
      const float z0 = reinterpret_cast<const float*>(in.pz)[i];
      const float ux = reinterpret_cast<const float*>(in.dx)[i];
      const float uy = reinterpret_cast<const float*>(in.dy)[i];
      const float uz = reinterpret_cast<const float*>(in.dz)[i];
      const float lo[3] = {0.f, 0.f, 0.f};
      float px, py, pz, tl;
      intercept(s.sag_type, s, sys.newton_iterations, x, y, z0, lo, ux, uy, uz, 0.f, 0.f, 0.f,
                px, py, pz, tl);
      reinterpret_cast<float*>(out.px)[i] = px;
      reinterpret_cast<float*>(out.py)[i] = py;
      reinterpret_cast<float*>(out.pz)[i] = pz;
    }
  }
}

// mode 0: groove efficiency -> eff ; 1: effective incident direction -> out.d*
__global__ void k_rulings(const __grid_constant__ otx_system sys, const int mode,
                          const otx_rays r, const otx_rays nrm, float* eff,
                          const otx_rays out) {
  const otx_surface& s = sys.surfaces[0];
  const int64_t step = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < r.count; i += step) {
    Ray q;
    q.px = reinterpret_cast<const float*>(r.px)[i];
    q.py = reinterpret_cast<const float*>(r.py)[i];
    q.pz = reinterpret_cast<const float*>(r.pz)[i];
    q.dx = reinterpret_cast<const float*>(r.dx)[i];
    q.dy = reinterpret_cast<const float*>(r.dy)[i];
    q.dz = reinterpret_cast<const float*>(r.dz)[i];
    q.wl = reinterpret_cast<const float*>(r.wavelength)[i];
    q.n = r.index_refraction ? reinterpret_cast<const float*>(r.index_refraction)[i] : 1.f;
    const float nx = reinterpret_cast<const float*>(nrm.dx)[i];
    const float ny = reinterpret_cast<const float*>(nrm.dy)[i];
    const float nz = reinterpret_cast<const float*>(nrm.dz)[i];
    if (mode == 0) {
      eff[i] = (s.rule_eff_type == OTX_RULE_EFF_IDEAL)
                   ? s.rule_efficiency
                   : ruling_efficiency_call(sys, s, s.rule_type, q.px, q.py, q.pz, q.dx, q.dy,
                                            q.dz, q.wl, nx, ny, nz);
    } else {
      incident_effective(s.rule_type, s, q, nx, ny, nz);
      reinterpret_cast<float*>(out.dx)[i] = q.dx;
      reinterpret_cast<float*>(out.dy)[i] = q.dy;
      reinterpret_cast<float*>(out.dz)[i] = q.dz;
    }
  }
}

// One block per group (grid-stride over groups): per-thread double
// partial sums, then a warp-shuffle and shared-memory tree.
__global__ void __launch_bounds__(256) k_pupil_reduce(const otx_rays r, int64_t groups,
                                                      int64_t per, double* sums) {
  __shared__ double part[6][8];
  const float* px = reinterpret_cast<const float*>(r.px);
  const float* py = reinterpret_cast<const float*>(r.py);
  const float* in = reinterpret_cast<const float*>(r.intensity);
  const uint8_t* uv = reinterpret_cast<const uint8_t*>(r.unvignetted);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int64_t g = blockIdx.x; g < groups; g += gridDim.x) {
    double a[6] = {0, 0, 0, 0, 0, 0};
    const int64_t base = g * per;
    for (int64_t k = threadIdx.x; k < per; k += blockDim.x) {
      const int64_t i = base + k;
      const double x = px[i], y = py[i];
      a[3] += x;
      a[4] += y;
      if (!uv || uv[i]) {
        a[0] += 1.0;
        a[1] += x;
        a[2] += y;
        a[5] += in ? (double)in[i] : 1.0;
      }
    }
#pragma unroll
    for (int j = 0; j < 6; ++j) {
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) a[j] += __shfl_down_sync(0xffffffffu, a[j], o);
    }
    if (lane == 0) {
#pragma unroll
      for (int j = 0; j < 6; ++j) part[j][warp] = a[j];
    }
    __syncthreads();
    if (threadIdx.x < 6) {
      double t = 0.0;
      for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += part[threadIdx.x][w];
      sums[g * 6 + threadIdx.x] = t;
    }
    __syncthreads();
  }
}

static int grid_for(int64_t n) {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (sms <= 0) sms = 132;
  int64_t need = (n + 255) / 256;
  const int64_t cap = (int64_t)sms * 16;
  return (int)(need < cap ? need : cap);
}

}  // namespace otx

using namespace otx;

extern "C" otx_status otx_collect(const otx_sensor* sensor, const otx_rays* rays,
                                  const otx_image* image, void* stream) {
  if (!sensor || !rays || !image || rays->count < 0) return OTX_ERR_INVALID;
  if (sensor->num_x < 1 || sensor->num_y < 1 || sensor->num_w < 1) return OTX_ERR_INVALID;
  if (!(sensor->width_x > 0.f) || !(sensor->width_y > 0.f)) return OTX_ERR_INVALID;
  if (rays->count == 0) return OTX_OK;
  if (!rays->px || !rays->py) return OTX_ERR_INVALID;
  if (sensor->w_hi > sensor->w_lo && !rays->wavelength) return OTX_ERR_INVALID;
  otx_sensor S = *sensor;
  S.inv_width_x = 1.f / S.width_x;
  S.inv_width_y = 1.f / S.width_y;
  S.inv_width_w = (S.w_hi > S.w_lo) ? (float)S.num_w / (S.w_hi - S.w_lo) : 0.f;
  k_collect<<<grid_for(rays->count), 256, 0, reinterpret_cast<cudaStream_t>(stream)>>>(
      S, *rays, *image);
  return cudaGetLastError() == cudaSuccess ? OTX_OK : OTX_ERR_CUDA;
}

extern "C" otx_status otx_sag_eval(const otx_system* sys, int32_t mode, const otx_rays* in,
                                   const otx_rays* out, void* stream) {
  if (!sys || sys->abi_version != OTX_ABI_VERSION || !in || !out) return OTX_ERR_INVALID;
  if (mode < 0 || mode > 2) return OTX_ERR_INVALID;
  const int st = sys->surfaces[0].sag_type;
  if (st < OTX_SAG_FLAT || st > OTX_SAG_CYLINDER) return OTX_ERR_UNSUPPORTED;
  if (in->count < 0) return OTX_ERR_INVALID;
  if (in->count == 0) return OTX_OK;
  if (!in->px || !in->py) return OTX_ERR_INVALID;
  if (mode == 0 && !out->pz) return OTX_ERR_INVALID;
  if (mode == 1 && (!out->dx || !out->dy || !out->dz)) return OTX_ERR_INVALID;
  if (mode == 2 && (!in->pz || !in->dx || !in->dy || !in->dz || !out->px || !out->py || !out->pz))
    return OTX_ERR_INVALID;
  k_sag<<<grid_for(in->count), 256, 0, reinterpret_cast<cudaStream_t>(stream)>>>(*sys, mode, *in,
                                                                               *out);
  return cudaGetLastError() == cudaSuccess ? OTX_OK : OTX_ERR_CUDA;
}

extern "C" otx_status otx_rulings_eval(const otx_system* sys, int32_t mode, const otx_rays* rays,
                                       const otx_rays* normal, float* efficiency,
                                       const otx_rays* out, void* stream) {
  if (!sys || !rays || !normal) return OTX_ERR_INVALID;
  if (mode < 0 || mode > 1) return OTX_ERR_INVALID;
  otx_system one = *sys;
  one.num_surfaces = 1;
  if (const otx_status vs = validate_system(&one)) return vs;
  if (sys->surfaces[0].rule_type == OTX_RULE_NONE) return OTX_ERR_INVALID;
  if (rays->count < 0) return OTX_ERR_INVALID;
  if (rays->count == 0) return OTX_OK;
  if (!rays->px || !rays->py || !rays->pz || !rays->dx || !rays->dy || !rays->dz ||
      !rays->wavelength || !normal->dx || !normal->dy || !normal->dz)
    return OTX_ERR_INVALID;
  if (mode == 0 && !efficiency) return OTX_ERR_INVALID;
  if (mode == 1 && (!out || !out->dx || !out->dy || !out->dz)) return OTX_ERR_INVALID;
  const otx_rays none{};
  k_rulings<<<grid_for(rays->count), 256, 0, reinterpret_cast<cudaStream_t>(stream)>>>(
      *sys, mode, *rays, *normal, efficiency, mode == 1 ? *out : none);
  return cudaGetLastError() == cudaSuccess ? OTX_OK : OTX_ERR_CUDA;
}

extern "C" otx_status otx_pupil_reduce(const otx_rays* rays, int64_t groups, int64_t per_group,
                                       double* sums, void* stream) {
  if (!rays || groups < 0 || per_group < 1) return OTX_ERR_INVALID;
  if (groups == 0) return OTX_OK;
  if (!rays->px || !rays->py || !sums) return OTX_ERR_INVALID;
  if (rays->count != groups * per_group) return OTX_ERR_INVALID;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (sms <= 0) sms = 132;
  const int64_t cap = (int64_t)sms * 8;
  const int grid = (int)(groups < cap ? groups : cap);
  k_pupil_reduce<<<grid, 256, 0, reinterpret_cast<cudaStream_t>(stream)>>>(*rays, groups,
                                                                           per_group, sums);
  return cudaGetLastError() == cudaSuccess ? OTX_OK : OTX_ERR_CUDA;
}
