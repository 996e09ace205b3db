// Learned surrogate of a batched trace's ray map: packing of the network
// inputs and training targets, the training loss, and image simulation
// with the trace as fallback in the same kernel.
//
// The network (a BF16 MLP run by the tensor-core GEMM) predicts, per ray,
// the residual of the image position over a per-configuration quadratic
// polynomial of the normalised ray inputs, and a vignetting logit.  The
// image kernel lands confidently classified rays of trusted configurations
// at the predicted position; every other ray is compacted in shared memory
// and traced through the configuration's surfaces by the same CTA, so the
// fallback costs no second launch, no host round trip and no idle lanes.
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include "../../include/optika_gb300.h"
#include "surrogate_common.cuh"

namespace otx {

struct PackArgs {
  otx_batch b;
  otx_surrogate sg;
  int64_t first, count;
  const int64_t* perm;
  const float* px;
  const float* py;
  const uint8_t* unvig;
  __nv_bfloat16* x;
  __nv_bfloat16* xt;
  int ldt;
  float4* aux;
  float4* u;  // 2 per row: u0..u3, then u4, config, 0, 0 (or null)
};

__global__ void __launch_bounds__(256) k_surrogate_pack(const __grid_constant__ PackArgs a) {
  const int64_t* offs = reinterpret_cast<const int64_t*>(a.b.ray_offset);
  const float* cin = reinterpret_cast<const float*>(a.sg.config_inputs);
  const float* coef = reinterpret_cast<const float*>(a.sg.baseline);
  const int64_t total = offs[a.b.num_configs];
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < a.count;
       r += (int64_t)gridDim.x * blockDim.x) {
    int64_t gid = a.perm ? a.perm[a.first + r] : a.first + r;
    gid = gid < 0 ? 0 : (gid >= total ? total - 1 : gid);  // bounded even for a bad perm
    const int cfg = config_of(offs, a.b.num_configs, gid);
    const BatchInputs v = batch_inputs(a.b, cfg, gid - offs[cfg]);
    float f[OTX_SURROGATE_LDX];
    ray_features(a.b, v, f);
#pragma unroll
    for (int j = 0; j < 4; ++j) f[5 + j] = cin[cfg * 4 + j];
#pragma unroll
    for (int j = OTX_SURROGATE_NIN; j < OTX_SURROGATE_LDX; ++j) f[j] = 0.f;
    uint32_t w[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      __nv_bfloat162 h = __floats2bfloat162_rn(f[2 * j], f[2 * j + 1]);
      w[j] = *reinterpret_cast<uint32_t*>(&h);
    }
    uint4* xr = reinterpret_cast<uint4*>(a.x + r * OTX_SURROGATE_LDX);
    xr[0] = make_uint4(w[0], w[1], w[2], w[3]);
    xr[1] = make_uint4(w[4], w[5], w[6], w[7]);
    if (a.xt) {
#pragma unroll
      for (int j = 0; j < OTX_SURROGATE_NIN; ++j)
        a.xt[(int64_t)j * a.ldt + r] = __float2bfloat16_rn(f[j]);
    }
    if (a.u) {
      a.u[2 * r] = make_float4(f[0], f[1], f[2], f[3]);
      a.u[2 * r + 1] = make_float4(f[4], (float)cfg, 0.f, 0.f);
    }
    float bx, by;
    baseline_xy(coef + (int64_t)cfg * 2 * OTX_SURROGATE_NBASE, f, bx, by);
    float4 o;
    if (a.px) {
      const float inv = 1.f / a.sg.out_scale;
      const bool lab = a.unvig[gid] != 0;
      o.x = lab ? (a.px[gid] - bx) * inv : 0.f;
      o.y = lab ? (a.py[gid] - by) * inv : 0.f;
      o.z = lab ? 1.f : 0.f;
      o.w = 0.f;
    } else {
      o = make_float4(bx, by, v.wl, (float)cfg);
    }
    a.aux[r] = o;
  }
}

// Loss and its gradient for one batch.  Position residuals: squared error
// on unvignetted rays; logit: binary cross-entropy with logits (Bernoulli
// likelihood of the unvignetted label), in its overflow-free form
// max(s, 0) - s t + log(1 + exp(-|s|)).
__global__ void __launch_bounds__(256)
    k_surrogate_loss(const float* __restrict__ y, int ldy, const float4* __restrict__ aux,
                     int64_t count, float w_pos, float w_cls, float norm,
                     __nv_bfloat16* __restrict__ dy, __nv_bfloat16* __restrict__ dyt, int ldt,
                     float* __restrict__ sums) {
  float s_pos = 0.f, s_bce = 0.f, s_lab = 0.f, s_ok = 0.f;
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < count;
       r += (int64_t)gridDim.x * blockDim.x) {
    const float4 t = aux[r];
    const float y0 = y[r * ldy], y1 = y[r * ldy + 1], s = y[r * ldy + 2];
    const float e0 = y0 - t.x, e1 = y1 - t.y;
    const float lab = t.z;
    const float sig = 1.f / (1.f + __expf(-s));
    const float g0 = 2.f * w_pos * norm * lab * e0;
    const float g1 = 2.f * w_pos * norm * lab * e1;
    const float g2 = w_cls * norm * (sig - lab);
    s_pos += lab * (e0 * e0 + e1 * e1);
    s_bce += fmaxf(s, 0.f) - s * lab + log1pf(__expf(-fabsf(s)));
    s_lab += lab;
    s_ok += ((s > 0.f) == (lab > 0.5f)) ? 1.f : 0.f;
    __nv_bfloat162 h01 = __floats2bfloat162_rn(g0, g1);
    __nv_bfloat162 h2z = __floats2bfloat162_rn(g2, 0.f);
    const uint4 row = make_uint4(*reinterpret_cast<uint32_t*>(&h01),
                                 *reinterpret_cast<uint32_t*>(&h2z), 0u, 0u);
    reinterpret_cast<uint4*>(dy)[r] = row;
    dyt[r] = __low2bfloat16(h01);
    dyt[(int64_t)ldt + r] = __high2bfloat16(h01);
    dyt[2 * (int64_t)ldt + r] = __low2bfloat16(h2z);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    s_pos += __shfl_xor_sync(0xffffffffu, s_pos, o);
    s_bce += __shfl_xor_sync(0xffffffffu, s_bce, o);
    s_lab += __shfl_xor_sync(0xffffffffu, s_lab, o);
    s_ok += __shfl_xor_sync(0xffffffffu, s_ok, o);
  }
  if ((threadIdx.x & 31) == 0) {
    atomicAdd(sums + 0, s_pos);
    atomicAdd(sums + 1, s_bce);
    atomicAdd(sums + 2, s_lab);
    atomicAdd(sums + 3, s_ok);
  }
}

constexpr int SG_IMAGE_BLOCK = 256;
constexpr int SG_IMAGE_RPT = 4;  // rays per thread: a CTA covers 1024 rays

struct ImageArgs {
  otx_batch b;
  otx_surrogate sg;
  int64_t first, count;
  const float* y;
  int ldy;
  const float4* aux;
  otx_image img;
  unsigned long long* stats;
};

template <class... Ks>
__global__ void __launch_bounds__(SG_IMAGE_BLOCK)
    k_surrogate_image(const __grid_constant__ otx_system sys, const __grid_constant__ ImageArgs a) {
  constexpr int PER_CTA = SG_IMAGE_BLOCK * SG_IMAGE_RPT;
  __shared__ otx_surface surf[OTX_MAX_SURFACES];
  __shared__ int list[PER_CTA];
  __shared__ int s_nfb, s_net;
  const int tid = threadIdx.x;
  const int64_t r0 = (int64_t)blockIdx.x * PER_CTA;
  if (r0 >= a.count) return;
  const int64_t r1 = min(a.count, r0 + PER_CTA);
  if (tid == 0) {
    s_nfb = 0;
    s_net = 0;
  }
  __syncthreads();
  const uint8_t* trusted = reinterpret_cast<const uint8_t*>(a.sg.trusted);
  const int64_t* offs = reinterpret_cast<const int64_t*>(a.b.ray_offset);
  int net = 0;
  for (int64_t r = r0 + tid; r < r1; r += SG_IMAGE_BLOCK) {
    const float4 x = a.aux[r];
    const int cfg = min(max((int)x.w, 0), a.b.num_configs - 1);
    const float s = a.y[r * a.ldy + 2];
    const bool ok_cfg = trusted ? trusted[cfg] != 0 : true;
    if (!ok_cfg || !(fabsf(s) >= a.sg.logit_band)) {  // NaN logits are traced too
      list[atomicAdd(&s_nfb, 1)] = (int)(r - r0);
    } else if (s > 0.f) {
      Ray ray;
      ray.px = fmaf(a.sg.out_scale, a.y[r * a.ldy], x.x);
      ray.py = fmaf(a.sg.out_scale, a.y[r * a.ldy + 1], x.y);
      ray.wl = x.z;
      ray.inten = 1.f;
      ray.ok = true;
      const otx_image img = config_image(a.img, a.b.image_stride, cfg);
      if (img.counts || img.flux) {
        if (sensor_bin(sys.sensor, ray) >= 0) ++net;
        bin_ray(sys.sensor, img, ray);
      }
    }
  }
  atomicAdd(&s_net, net);
  __syncthreads();
  const int nfb = s_nfb;
  int traced_binned = 0;
  if (nfb > 0) {
    // the base surfaces once; each configuration's overrides go on top
    const int words = sys.num_surfaces * (int)(sizeof(otx_surface) / 4);
    const int* src = reinterpret_cast<const int*>(sys.surfaces);
    int* dst = reinterpret_cast<int*>(surf);
    for (int w = tid; w < words; w += SG_IMAGE_BLOCK) dst[w] = src[w];
    __syncthreads();  // nfb is uniform: every thread reaches this barrier
  }
  if (nfb > 0) {
    const int c_lo = min(max((int)a.aux[r0].w, 0), a.b.num_configs - 1);
    const int c_hi = min(max((int)a.aux[r1 - 1].w, 0), a.b.num_configs - 1);
    const otx_surface* ov = reinterpret_cast<const otx_surface*>(a.b.overrides);
    for (int c = c_lo; c <= c_hi; ++c) {
      const int words = (int)(sizeof(otx_surface) / 4);
      for (int j = 0; j < a.b.num_overrides; ++j) {
        const int* src = reinterpret_cast<const int*>(ov + (int64_t)c * a.b.num_overrides + j);
        int* dst = reinterpret_cast<int*>(surf + a.b.override_index[j]);
        for (int w = tid; w < words; w += SG_IMAGE_BLOCK) dst[w] = src[w];
      }
      __syncthreads();
      const otx_image img = config_image(a.img, a.b.image_stride, c);
      for (int j = tid; j < nfb; j += SG_IMAGE_BLOCK) {
        const int64_t r = r0 + list[j];
        const int cfg = min(max((int)a.aux[r].w, 0), a.b.num_configs - 1);
        if (cfg != c) continue;
        const int64_t gid = a.first + r;
        Ray ray;
        batch_ray(a.b, c, gid - offs[c], ray);
        propagate_all<Ks...>(sys, surf, ray);
        if (img.counts || img.flux) {
          if (ray.ok && sensor_bin(sys.sensor, ray) >= 0) ++traced_binned;
          bin_ray(sys.sensor, img, ray);
        }
      }
      __syncthreads();  // surf is rewritten for the next configuration
    }
  }
  // per-CTA statistics
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) traced_binned += __shfl_xor_sync(0xffffffffu, traced_binned, o);
  if ((tid & 31) == 0 && traced_binned) atomicAdd(a.stats + 3, (unsigned long long)traced_binned);
  if (tid == 0) {
    atomicAdd(a.stats + 0, (unsigned long long)(r1 - r0));
    atomicAdd(a.stats + 1, (unsigned long long)nfb);
    atomicAdd(a.stats + 2, (unsigned long long)s_net);
  }
}

static int grid_for(int64_t n, int block) {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (sms <= 0) sms = 132;
  const int64_t need = (n + block - 1) / block;
  const int64_t cap = (int64_t)sms * 8;
  return (int)(need < cap ? (need > 0 ? need : 1) : cap);
}

static bool batch_ok(const otx_batch* b, const otx_surrogate* sg) {
  return b && sg && b->num_configs >= 1 && b->ray_offset && sg->num_configs == b->num_configs &&
         sg->config_inputs && sg->baseline && sg->out_scale > 0.f;
}

}  // namespace otx

using namespace otx;

extern "C" {

otx_status otx_surrogate_pack(const otx_batch* batch, const otx_surrogate* sg, int64_t first,
                              int64_t count, const int64_t* perm, const float* px,
                              const float* py, const uint8_t* unvignetted, void* x, void* x_t,
                              int32_t ldt, float* aux, float* u, void* stream) {
  if (!batch_ok(batch, sg) || first < 0 || count < 0 || !x || !aux) return OTX_ERR_INVALID;
  if (reinterpret_cast<uintptr_t>(u) & 15) return OTX_ERR_INVALID;
  if ((px || py || unvignetted) && !(px && py && unvignetted)) return OTX_ERR_INVALID;
  if (x_t && ldt < count) return OTX_ERR_INVALID;
  if ((reinterpret_cast<uintptr_t>(x) | reinterpret_cast<uintptr_t>(aux)) & 15)
    return OTX_ERR_INVALID;
  if (count == 0) return OTX_OK;
  PackArgs a;
  memset(&a, 0, sizeof(a));
  a.b = *batch;
  a.sg = *sg;
  a.first = first;
  a.count = count;
  a.perm = perm;
  a.px = px;
  a.py = py;
  a.unvig = unvignetted;
  a.x = reinterpret_cast<__nv_bfloat16*>(x);
  a.xt = reinterpret_cast<__nv_bfloat16*>(x_t);
  a.ldt = ldt;
  a.aux = reinterpret_cast<float4*>(aux);
  a.u = reinterpret_cast<float4*>(u);
  k_surrogate_pack<<<grid_for(count, 256), 256, 0, reinterpret_cast<cudaStream_t>(stream)>>>(a);
  return cudaGetLastError() == cudaSuccess ? OTX_OK : OTX_ERR_CUDA;
}

otx_status otx_surrogate_loss(const float* y, int32_t ldy, const float* aux, int64_t count,
                              float w_pos, float w_cls, float norm, void* dy, void* dy_t,
                              int32_t ldt, float* sums, void* stream) {
  if (count < 0 || !y || ldy < 3 || !aux || !dy || !dy_t || !sums || ldt < count)
    return OTX_ERR_INVALID;
  if ((reinterpret_cast<uintptr_t>(dy) | reinterpret_cast<uintptr_t>(aux)) & 15)
    return OTX_ERR_INVALID;
  if (count == 0) return OTX_OK;
  k_surrogate_loss<<<grid_for(count, 256), 256, 0, reinterpret_cast<cudaStream_t>(stream)>>>(
      y, ldy, reinterpret_cast<const float4*>(aux), count, w_pos, w_cls, norm,
      reinterpret_cast<__nv_bfloat16*>(dy), reinterpret_cast<__nv_bfloat16*>(dy_t), ldt, sums);
  return cudaGetLastError() == cudaSuccess ? OTX_OK : OTX_ERR_CUDA;
}

otx_status otx_surrogate_image(const otx_system* base, const otx_batch* batch,
                               const otx_surrogate* sg, int64_t first, int64_t count,
                               const float* y, int32_t ldy, const float* aux,
                               const otx_image* image, unsigned long long* stats, void* stream) {
  if (!base || !batch_ok(batch, sg) || first < 0 || count < 0 || !y || ldy < 3 || !aux || !stats)
    return OTX_ERR_INVALID;
  if (const otx_status vs = validate_system(base)) return vs;
  if (base->input_mode != OTX_INPUT_GRID_INFINITY) return OTX_ERR_INVALID;
  // predicted positions are in the output frame, binning in the sensor's
  if (!(base->flags & OTX_SYS_FLAG_FINAL_IDENTITY)) return OTX_ERR_UNSUPPORTED;
  const otx_batch& b = *batch;
  if (b.num_overrides < 0 || b.num_overrides > OTX_BATCH_MAX_OVERRIDES) return OTX_ERR_SIZE;
  for (int j = 0; j < b.num_overrides; ++j)
    if (b.override_index[j] < 0 || b.override_index[j] >= base->num_surfaces)
      return OTX_ERR_INVALID;
  if (b.num_overrides > 0 && !b.overrides) return OTX_ERR_INVALID;
  // the network predicts no direction: no cosine moment from this path
  if (image && image->cos_moment) return OTX_ERR_UNSUPPORTED;
  const bool bin = image && (image->counts || image->flux);
  if (bin && (base->sensor.num_x < 1 || base->sensor.num_y < 1 || base->sensor.num_w < 1 ||
              !(base->sensor.width_x > 0.f) || !(base->sensor.width_y > 0.f) ||
              b.image_stride < base->sensor.num_w * base->sensor.num_x * base->sensor.num_y))
    return OTX_ERR_INVALID;
  if (count == 0) return OTX_OK;
  otx_system sys = *base;
  otx_sensor& S = sys.sensor;
  S.inv_width_x = S.width_x > 0.f ? 1.f / S.width_x : 0.f;
  S.inv_width_y = S.width_y > 0.f ? 1.f / S.width_y : 0.f;
  S.inv_width_w = (S.w_hi > S.w_lo) ? (float)S.num_w / (S.w_hi - S.w_lo) : 0.f;
  ImageArgs a;
  memset(&a, 0, sizeof(a));
  a.b = b;
  a.sg = *sg;
  a.first = first;
  a.count = count;
  a.y = y;
  a.ldy = ldy;
  a.aux = reinterpret_cast<const float4*>(aux);
  if (bin) a.img = *image;
  a.stats = stats;
  constexpr int PER_CTA = SG_IMAGE_BLOCK * SG_IMAGE_RPT;
  const int64_t grid = (count + PER_CTA - 1) / PER_CTA;
  if (grid > 0x7fffffff) return OTX_ERR_SIZE;
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  if (shape_matches<BObject, BSphere, BGrating, BSensor>(sys))
    k_surrogate_image<BObject, BSphere, BGrating, BSensor>
        <<<(unsigned)grid, SG_IMAGE_BLOCK, 0, st>>>(sys, a);
  else
    k_surrogate_image<><<<(unsigned)grid, SG_IMAGE_BLOCK, 0, st>>>(sys, a);
  return cudaGetLastError() == cudaSuccess ? OTX_OK : OTX_ERR_CUDA;
}

}  // extern "C"
