// Batched trace: many configurations of one system shape in one persistent
// launch.
//
// Persistent CTAs take work items (a tile of up to tile_size rays of one
// configuration) from a device counter.  A CTA keeps the surface
// descriptors of its current configuration in shared memory (the base
// system's surfaces, with the configuration's overridden surfaces copied
// over them), generates its rays with Philox4x32-10 and traces them with the
// same device functions as the single-system kernels.  Configurations with
// uneven ray counts (1e3 .. 1e6) balance through the shared counter.
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>


#include "../../include/optika_gb300.h"
#include "batch_rays.cuh"

namespace otx {

struct BatchArgs {
  otx_batch b;
  otx_rays out;
  otx_image img;
};

template <int RPT, class... Ks>
__global__ void __launch_bounds__(256) k_trace_batch(const __grid_constant__ otx_system sys,
                                                     const __grid_constant__ BatchArgs a) {
  __shared__ otx_surface surf[OTX_MAX_SURFACES];
  __shared__ int s_item;
  const otx_batch& b = a.b;
  const int tid = threadIdx.x;
  const int ns = sys.num_surfaces;
  {
    const int words = ns * (int)(sizeof(otx_surface) / 4);
    const int* src = reinterpret_cast<const int*>(sys.surfaces);
    int* dst = reinterpret_cast<int*>(surf);
    for (int w = tid; w < words; w += blockDim.x) dst[w] = src[w];
  }
  const otx_surface* ov = reinterpret_cast<const otx_surface*>(b.overrides);
  const int64_t* offs = reinterpret_cast<const int64_t*>(b.ray_offset);
  const int32_t* tiles = reinterpret_cast<const int32_t*>(b.tiles);
  unsigned int* counter = reinterpret_cast<unsigned int*>(b.counter);
  const bool bin = image_any(a.img);
  int bin_skip = 0;
  int cur = -1;
  bool skip0 = false;
  for (;;) {
    __syncthreads();  // previous item done: s_item and surf may be rewritten
    if (tid == 0) s_item = (int)atomicAdd(counter, 1u);
    __syncthreads();
    const int item = s_item;
    if ((int64_t)item >= b.num_tiles) break;
    const int cfg = tiles[2 * item];
    const int64_t start = tiles[2 * item + 1];
    if (cfg < 0 || cfg >= b.num_configs) continue;
    if (cfg != cur) {
      const int words = (int)(sizeof(otx_surface) / 4);
      for (int j = 0; j < b.num_overrides; ++j) {
        const int* src = reinterpret_cast<const int*>(ov + (int64_t)cfg * b.num_overrides + j);
        int* dst = reinterpret_cast<int*>(surf + b.override_index[j]);
        for (int w = tid; w < words; w += blockDim.x) dst[w] = src[w];
      }
      __syncthreads();
      cur = cfg;
      skip0 = batch_first_is_noop(surf[0]);
    }
    const int64_t base = offs[cfg];
    const int64_t n_c = offs[cfg + 1] - base;
    const int64_t end = start + b.tile_size < n_c ? start + b.tile_size : n_c;
    for (int64_t i0 = start + tid; i0 < end; i0 += (int64_t)blockDim.x * RPT) {
      Ray r[RPT];
#pragma unroll
      for (int k = 0; k < RPT; ++k) {
        const int64_t i = i0 + (int64_t)k * blockDim.x;
        if (i < end) {
          batch_ray(b, cfg, i, r[k]);
          propagate_all<Ks...>(sys, surf, r[k], skip0);
        }
      }
#pragma unroll
      for (int k = 0; k < RPT; ++k) {
        const int64_t i = i0 + (int64_t)k * blockDim.x;
        if (i < end) {
          if (bin) {
            otx_image img = a.img;
            const int64_t off = (int64_t)cfg * b.image_stride;
            if (img.counts) img.counts += off * 4;
            if (img.flux) img.flux += off * 4;
            if (img.cos_moment) img.cos_moment += off * 4;
            bin_ray_warp(sys.sensor, img, r[k], bin_skip);
          }
          store_ray<true>(a.out, base + i, sys.final_to_output, r[k]);
        }
      }
    }
  }
}

template <class... Ks>
static void launch_batch(int rpt, int grid, int block, const otx_system& sys, const BatchArgs& a,
                         cudaStream_t st) {
  if (rpt == 2)
    k_trace_batch<2, Ks...><<<grid, block, 0, st>>>(sys, a);
  else
    k_trace_batch<1, Ks...><<<grid, block, 0, st>>>(sys, a);
}

}  // namespace otx

using namespace otx;

extern "C" otx_status otx_trace_batch(const otx_system* base, const otx_batch* batch,
                                      const otx_rays* out, const otx_image* image,
                                      const otx_launch* launch, void* stream) {
  if (!base || !batch || !out) return OTX_ERR_INVALID;
  if (const otx_status vs = validate_system(base)) return vs;
  if (base->input_mode != OTX_INPUT_GRID_INFINITY) return OTX_ERR_INVALID;
  // rays are stored in the last surface's frame: it must be the output frame
  if (!(base->flags & OTX_SYS_FLAG_FINAL_IDENTITY)) return OTX_ERR_UNSUPPORTED;
  const otx_batch& b = *batch;
  if (b.num_configs < 0 || b.num_tiles < 0 || b.tile_size < 1) return OTX_ERR_INVALID;
  if (b.num_overrides < 0 || b.num_overrides > OTX_BATCH_MAX_OVERRIDES) return OTX_ERR_SIZE;
  for (int j = 0; j < b.num_overrides; ++j)
    if (b.override_index[j] < 0 || b.override_index[j] >= base->num_surfaces)
      return OTX_ERR_INVALID;
  if (b.num_tiles == 0) return OTX_OK;
  if (!b.ray_offset || !b.tiles || !b.counter || (b.num_overrides > 0 && !b.overrides))
    return OTX_ERR_INVALID;
  const bool bin = image && (image->counts || image->flux);
  if (bin && (base->sensor.num_x < 1 || base->sensor.num_y < 1 || base->sensor.num_w < 1 ||
              !(base->sensor.width_x > 0.f) || !(base->sensor.width_y > 0.f) ||
              (int64_t)b.image_stride < (int64_t)base->sensor.num_w * base->sensor.num_x *
                                            base->sensor.num_y))
    return OTX_ERR_INVALID;
  int rpt = (launch && launch->rays_per_thread > 0) ? launch->rays_per_thread : 1;
  if (rpt != 1 && rpt != 2) return OTX_ERR_INVALID;
  int block = (launch && launch->block_size > 0) ? launch->block_size : 256;
  if (block > 256 || block % 32 != 0) return OTX_ERR_INVALID;

  otx_system sys = *base;
  otx_sensor& S = sys.sensor;
  S.inv_width_x = S.width_x > 0.f ? 1.f / S.width_x : 0.f;
  S.inv_width_y = S.width_y > 0.f ? 1.f / S.width_y : 0.f;
  S.inv_width_w = (S.w_hi > S.w_lo) ? (float)S.num_w / (S.w_hi - S.w_lo) : 0.f;
  BatchArgs a;
  memset(&a, 0, sizeof(a));
  a.b = b;
  a.out = *out;
  if (bin) a.img = *image;

  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  if (cudaMemsetAsync(reinterpret_cast<void*>(b.counter), 0, sizeof(unsigned int), st) !=
      cudaSuccess)
    return OTX_ERR_CUDA;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (sms <= 0) sms = 132;
  const int per_sm = 2048 / block;  // resident CTAs the scheduler can hold
  int64_t grid = (int64_t)sms * (per_sm < 8 ? per_sm : 8);
  if (grid > b.num_tiles) grid = b.num_tiles;

  // the spectrograph shape (object, spherical mirror, toroidal VLS grating,
  // sensor) runs its specialised kernel; anything else the generic one.
  // Overridden surfaces keep the kinds of the base surfaces they replace
  // (the host API checks this); the device functions bound every index
  // they read from a descriptor, so a descriptor breaking it is wrong but
  // never out of bounds.
  const bool fixed =
      !(launch && launch->generic_only) && shape_matches<BObject, BSphere, BGrating, BSensor>(sys);
  if (fixed)
    launch_batch<BObject, BSphere, BGrating, BSensor>(rpt, (int)grid, block, sys, a, st);
  else
    launch_batch<>(rpt, (int)grid, block, sys, a, st);
  return cudaGetLastError() == cudaSuccess ? OTX_OK : OTX_ERR_CUDA;
}

// ---------------------------------------------------------------- no allocation

// Scratch of otx_trace_batch_noalloc: word 0 is the work counter, words
// 64.. hold the tile list (config, first ray) of up to OTX_NOALLOC_MAX_TILES
// work items.  It is a file-scope device array, so the entry point needs no
// allocation; every GPU that loads the library holds its 1 MiB until exit,
// and every call shares it.
#define OTX_NOALLOC_HEADER_WORDS 64
static __device__ __align__(256) int32_t g_noalloc_scratch[OTX_NOALLOC_HEADER_WORDS +
                                                           2 * OTX_NOALLOC_MAX_TILES];

namespace otx {

// Tile list of a batch, built on the device from the ray-count prefix sums:
// one CTA, each thread owning a contiguous run of configurations, a block
// scan of their tile counts, then every thread writing its tiles.  Writes
// are bounded by num_tiles (the scratch array's capacity); entries past the
// batch's own tiles carry config -1, which the trace kernel skips.  A work
// item holds its first ray as int32, so a configuration of more than
// 2^31 - 1 rays gets no tiles (the host API rejects such counts).
__global__ void __launch_bounds__(1024) k_make_tiles(const int64_t* __restrict__ offs,
                                                    int num_configs, int tile_size,
                                                    int64_t num_tiles, int32_t* __restrict__ tiles) {
  __shared__ int64_t sums[1024];
  const int tid = threadIdx.x, nt = blockDim.x;
  const int per = (num_configs + nt - 1) / nt;
  const int c0 = tid * per, c1 = min(num_configs, c0 + per);
  int64_t mine = 0;
  for (int c = c0; c < c1; ++c) {
    const int64_t n = offs[c + 1] - offs[c];
    if (n > 0 && n <= INT32_MAX) mine += (n + tile_size - 1) / tile_size;
  }
  sums[tid] = mine;
  __syncthreads();
  for (int d = 1; d < nt; d <<= 1) {  // inclusive Hillis-Steele scan
    const int64_t v = tid >= d ? sums[tid - d] : 0;
    __syncthreads();
    sums[tid] += v;
    __syncthreads();
  }
  int64_t t = sums[tid] - mine;  // exclusive prefix
  for (int c = c0; c < c1; ++c) {
    const int64_t n = offs[c + 1] - offs[c];
    if (n > INT32_MAX) continue;
    for (int64_t start = 0; start < n && t < num_tiles; start += tile_size, ++t) {
      tiles[2 * t] = c;
      tiles[2 * t + 1] = (int32_t)start;
    }
  }
  const int64_t total = sums[nt - 1];
  for (int64_t k = total + tid; k < num_tiles; k += nt) {
    tiles[2 * k] = -1;
    tiles[2 * k + 1] = 0;
  }
}

// Device address of the scratch array on the current device.  The host
// name g_noalloc_scratch is only a stand-in for the array; its address in
// the current context comes from cudaGetSymbolAddress (which allocates
// nothing), looked up on every call so that a context recreated since the
// last call (after cudaDeviceReset, say) is never given a stale pointer.
static int32_t* noalloc_scratch() {
  void* p = nullptr;
  if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess) return nullptr;
  return static_cast<int32_t*>(p);
}

}  // namespace otx

extern "C" otx_status otx_trace_batch_noalloc(const otx_system* base, const otx_batch* batch,
                                              const otx_rays* out, const otx_image* image,
                                              const otx_launch* launch, void* stream) {
  if (!base || !batch || !out) return OTX_ERR_INVALID;
  if (const otx_status vs = validate_system(base)) return vs;
  if (base->input_mode != OTX_INPUT_GRID_INFINITY) return OTX_ERR_INVALID;
  // rays are stored in the last surface's frame: it must be the output frame
  if (!(base->flags & OTX_SYS_FLAG_FINAL_IDENTITY)) return OTX_ERR_UNSUPPORTED;
  const otx_batch& b = *batch;
  if (b.num_configs < 0 || b.num_tiles < 0 || b.tile_size < 1) return OTX_ERR_INVALID;
  if (b.num_tiles > OTX_NOALLOC_MAX_TILES) return OTX_ERR_SIZE;
  if (b.num_overrides < 0 || b.num_overrides > OTX_BATCH_MAX_OVERRIDES) return OTX_ERR_SIZE;
  for (int j = 0; j < b.num_overrides; ++j)
    if (b.override_index[j] < 0 || b.override_index[j] >= base->num_surfaces)
      return OTX_ERR_INVALID;
  if (b.num_tiles == 0) return OTX_OK;
  if (b.num_configs < 1 || !b.ray_offset || (b.num_overrides > 0 && !b.overrides))
    return OTX_ERR_INVALID;
  const bool bin = image && (image->counts || image->flux);
  if (bin && (base->sensor.num_x < 1 || base->sensor.num_y < 1 || base->sensor.num_w < 1 ||
              !(base->sensor.width_x > 0.f) || !(base->sensor.width_y > 0.f) ||
              (int64_t)b.image_stride < (int64_t)base->sensor.num_w * base->sensor.num_x *
                                            base->sensor.num_y))
    return OTX_ERR_INVALID;
  int rpt = (launch && launch->rays_per_thread > 0) ? launch->rays_per_thread : 1;
  if (rpt != 1 && rpt != 2) return OTX_ERR_INVALID;
  int block = (launch && launch->block_size > 0) ? launch->block_size : 256;
  if (block > 256 || block % 32 != 0) return OTX_ERR_INVALID;

  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return OTX_ERR_CUDA;
  int32_t* scratch = noalloc_scratch();
  if (!scratch) return OTX_ERR_CUDA;
  int32_t* counter = scratch;
  int32_t* tiles = scratch + OTX_NOALLOC_HEADER_WORDS;

  otx_system sys = *base;
  otx_sensor& S = sys.sensor;
  S.inv_width_x = S.width_x > 0.f ? 1.f / S.width_x : 0.f;
  S.inv_width_y = S.width_y > 0.f ? 1.f / S.width_y : 0.f;
  S.inv_width_w = (S.w_hi > S.w_lo) ? (float)S.num_w / (S.w_hi - S.w_lo) : 0.f;
  // The tile list is built on the device from the ray offsets and padded
  // to the array's capacity, and the trace takes work items up to that
  // capacity (padding items are skipped): the caller's num_tiles, which
  // the host cannot check against device-resident offsets, is used only
  // for the size check above.
  BatchArgs a;
  memset(&a, 0, sizeof(a));
  a.b = b;
  a.b.tiles = reinterpret_cast<uint64_t>(tiles);
  a.b.counter = reinterpret_cast<uint64_t>(counter);
  a.b.num_tiles = OTX_NOALLOC_MAX_TILES;
  a.out = *out;
  if (bin) a.img = *image;

  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  // the array keeps the previous call's contents: clear the counter
  if (cudaMemsetAsync(counter, 0, OTX_NOALLOC_HEADER_WORDS * sizeof(int32_t), st) != cudaSuccess)
    return OTX_ERR_CUDA;
  k_make_tiles<<<1, 1024, 0, st>>>(reinterpret_cast<const int64_t*>(b.ray_offset), b.num_configs,
                                   b.tile_size, (int64_t)OTX_NOALLOC_MAX_TILES, tiles);
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (sms <= 0) sms = 132;
  const int per_sm = 2048 / block;
  const int64_t grid = (int64_t)sms * (per_sm < 8 ? per_sm : 8);
  const bool fixed =
      !(launch && launch->generic_only) && shape_matches<BObject, BSphere, BGrating, BSensor>(sys);
  if (fixed)
    launch_batch<BObject, BSphere, BGrating, BSensor>(rpt, (int)grid, block, sys, a, st);
  else
    launch_batch<>(rpt, (int)grid, block, sys, a, st);
  return cudaGetLastError() == cudaSuccess ? OTX_OK : OTX_ERR_CUDA;
}
