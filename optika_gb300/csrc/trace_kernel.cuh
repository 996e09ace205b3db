// Fused trace kernel template, instantiated per input mode in
// trace_rays.cu, trace_grid_inf.cu and trace_grid_fin.cu so that the modes
// compile in parallel.
#pragma once
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "../../include/optika_gb300.h"
#include "cells.cuh"
#include "trace_device.cuh"
#include "trace_kernel_decl.h"

namespace otx {


// sin a as a float-float pair and cos a - 1, for |a| <= 1/16 rad, from
// their Taylor series (truncation below 1e-12 of the result there):
//   sin a     = a + a p,  p = a^2 (-1/6 + a^2 (1/120 - a^2 / 5040))
//   cos a - 1 = a^2 (-1/2 + a^2 (1/24 - a^2 (1/720 - a^2 / 40320)))
// The high part of sin a is a + a p rounded once; its low part is the
// rounding error, recovered exactly by an FMA (a - s is exact by Sterbenz).
__device__ __forceinline__ void sin_cosm1_small(float a, float& s_hi, float& s_lo, float& cm1) {
  const float a2 = a * a;
  const float p = a2 * fmaf(a2, fmaf(a2, -1.f / 5040.f, 1.f / 120.f), -1.f / 6.f);
  s_hi = fmaf(a, p, a);
  s_lo = fmaf(a, p, a - s_hi);
  cm1 = a2 * fmaf(a2, fmaf(a2, fmaf(a2, 1.f / 40320.f, -1.f / 720.f), 1.f / 24.f), -0.5f);
}

// Direction cosines from (azimuth, elevation), optika/_util.py:69-73:
// (-cos ay sin ax, -sin ay, cos ay cos ax), as a float-float vector unit to
// ~1e-12.  Angles up to 1/16 rad (every field of the telescopes and
// spectrographs here) take the series above, with cos written as 1 + (cos - 1)
// so that the direction's dominant component keeps its low part; larger
// angles take sincosf and unit_ff.
__device__ __forceinline__ void direction_from_angles(float ax, float ay, float& dx, float& dy,
                                                      float& dz, float& lx, float& ly,
                                                      float& lz) {
  if (fmaxf(fabsf(ax), fabsf(ay)) <= 0.0625f) {
    float sxh, sxl, cmx, syh, syl, cmy;
    sin_cosm1_small(ax, sxh, sxl, cmx);
    sin_cosm1_small(ay, syh, syl, cmy);
    // -cos ay sin ax = -(sx + (cos ay - 1) sx)
    const float xh = fmaf(cmy, sxh, sxh);
    const float xl = fmaf(cmy, sxh, sxh - xh) + fmaf(cmy, sxl, sxl);
    dx = -xh;
    lx = -xl;
    dy = -syh;
    ly = -syl;
    // cos ay cos ax = 1 + s, s = (cos ax - 1) + (cos ay - 1) + (cos ax - 1)(cos ay - 1)
    const float sz = fmaf(cmx, cmy, cmx + cmy);
    dz = 1.f + sz;
    lz = sz - (dz - 1.f);
    return;
  }
  float sx, cx, sy, cy;
  sincosf(ax, &sx, &cx);
  sincosf(ay, &sy, &cy);
  dx = -cy * sx;
  dy = -sy;
  dz = cy * cx;
  lx = ly = lz = 0.f;
  unit_ff(dx, dy, dz, lx, ly, lz);
}

template <int MODE>
__device__ __forceinline__ void load_ray(const TraceArgs& a, int64_t i, Ray& r) {
  if (MODE == OTX_INPUT_RAYS) {
    const otx_rays& in = a.in;
    r.px = reinterpret_cast<const float*>(in.px)[i];
    r.py = reinterpret_cast<const float*>(in.py)[i];
    r.pz = reinterpret_cast<const float*>(in.pz)[i];
    r.dx = reinterpret_cast<const float*>(in.dx)[i];
    r.dy = reinterpret_cast<const float*>(in.dy)[i];
    r.dz = reinterpret_cast<const float*>(in.dz)[i];
    r.lx = r.ly = r.lz = 0.f;
    unit_ff(r.dx, r.dy, r.dz, r.lx, r.ly, r.lz);
    r.wl = in.wavelength ? reinterpret_cast<const float*>(in.wavelength)[i] : 0.f;
    r.inten = in.intensity ? reinterpret_cast<const float*>(in.intensity)[i] : 1.f;
    r.att = in.attenuation ? reinterpret_cast<const float*>(in.attenuation)[i] : 0.f;
    r.n = in.index_refraction ? reinterpret_cast<const float*>(in.index_refraction)[i] : 1.f;
    r.ok = in.unvignetted ? (reinterpret_cast<const uint8_t*>(in.unvignetted)[i] != 0) : true;
    const double o = in.opl ? reinterpret_cast<const double*>(in.opl)[i] : 0.0;
    r.opl_hi = (float)o;
    r.opl_lo = (float)(o - (double)r.opl_hi);
  } else {
    float wl, fx, fy, qx, qy;
    float inten = 1.f;
    if constexpr (MODE == OTX_MODE_CELLS_INFINITY || MODE == OTX_MODE_CELLS_FINITE) {
      // the cell's ray, generated in place of reading a grid
      if (a.cells_idx32)
        cell_ray<uint32_t>(a.cells, a.first + i, wl, fx, fy, qx, qy, inten);
      else
        cell_ray<uint64_t>(a.cells, a.first + i, wl, fx, fy, qx, qy, inten);
    } else {
      const otx_grid& g = a.grid;
      wl = reinterpret_cast<const float*>(g.wavelength)[i * g.stride_wavelength];
      fx = reinterpret_cast<const float*>(g.field_x)[i * g.stride_field];
      fy = reinterpret_cast<const float*>(g.field_y)[i * g.stride_field];
      qx = reinterpret_cast<const float*>(g.pupil_x)[i * g.stride_pupil];
      qy = reinterpret_cast<const float*>(g.pupil_y)[i * g.stride_pupil];
      if (g.intensity) inten = reinterpret_cast<const float*>(g.intensity)[i * g.stride_intensity];
    }
    if (MODE == OTX_INPUT_GRID_INFINITY || MODE == OTX_MODE_CELLS_INFINITY) {
      r.px = qx;
      r.py = qy;
      direction_from_angles(fx, fy, r.dx, r.dy, r.dz, r.lx, r.ly, r.lz);
    } else {
      r.px = fx;
      r.py = fy;
      direction_from_angles(qx, qy, r.dx, r.dy, r.dz, r.lx, r.ly, r.lz);
    }
    r.pz = 0.f;
    r.wl = wl;
    r.inten = inten;
    r.att = 0.f;
    r.n = 1.f;
    r.ok = true;
    r.opl_hi = 0.f;
    r.opl_lo = 0.f;
  }
}

template <bool IDENTITY>
__device__ __forceinline__ void store_ray(const otx_rays& o, int64_t i,
                                          const otx_affine& f, const Ray& r) {
  float x = r.px, y = r.py, z = r.pz;
  float dx = r.dx + r.lx, dy = r.dy + r.ly, dz = r.dz + r.lz;
  if (!IDENTITY) {
    affine_point_folded(f, x, y, z);
    rotate(f, dx, dy, dz);
  }
  if (o.px) reinterpret_cast<float*>(o.px)[i] = x;
  if (o.py) reinterpret_cast<float*>(o.py)[i] = y;
  if (o.pz) reinterpret_cast<float*>(o.pz)[i] = z;
  if (o.dx) reinterpret_cast<float*>(o.dx)[i] = dx;
  if (o.dy) reinterpret_cast<float*>(o.dy)[i] = dy;
  if (o.dz) reinterpret_cast<float*>(o.dz)[i] = dz;
  if (o.wavelength) reinterpret_cast<float*>(o.wavelength)[i] = r.wl;
  if (o.intensity) reinterpret_cast<float*>(o.intensity)[i] = r.inten;
  if (o.attenuation) reinterpret_cast<float*>(o.attenuation)[i] = r.att;
  if (o.index_refraction) reinterpret_cast<float*>(o.index_refraction)[i] = r.n;
  if (o.unvignetted) reinterpret_cast<uint8_t*>(o.unvignetted)[i] = r.ok ? 1 : 0;
  if (o.opl) reinterpret_cast<double*>(o.opl)[i] = (double)r.opl_hi + (double)r.opl_lo;
}

// Histogram bin of a ray in the sensor frame, numpy.histogramdd edges:
// [e_j, e_j+1) with the last edge inclusive; outside and NaN are dropped
// (optika/sensors/_sensors.py:141-155).  Every operation is explicitly
// rounded (no contraction), so a float32 restatement of this formula
// reproduces each ray's bin exactly: upper edge lo + num w as one fused
// multiply-add, bin floor((p - lo) * (1 / w)).
__device__ __forceinline__ int64_t sensor_bin(const otx_sensor& S, const Ray& r) {
  const float hx = __fmaf_rn((float)S.num_x, S.width_x, S.lo_x);
  const float hy = __fmaf_rn((float)S.num_y, S.width_y, S.lo_y);
  if (!(r.px >= S.lo_x && r.px <= hx && r.py >= S.lo_y && r.py <= hy)) return -1;
  int ix = (int)floorf(__fmul_rn(__fsub_rn(r.px, S.lo_x), S.inv_width_x));
  int iy = (int)floorf(__fmul_rn(__fsub_rn(r.py, S.lo_y), S.inv_width_y));
  ix = min(max(ix, 0), S.num_x - 1);
  iy = min(max(iy, 0), S.num_y - 1);
  int iw = 0;
  if (S.w_hi > S.w_lo) {
    if (!(r.wl >= S.w_lo && r.wl <= S.w_hi)) return -1;
    iw = (int)floorf(__fmul_rn(__fsub_rn(r.wl, S.w_lo), S.inv_width_w));
    iw = min(max(iw, 0), S.num_w - 1);
  }
  return ((int64_t)iw * S.num_x + ix) * S.num_y + iy;
}

__device__ __forceinline__ void bin_ray(const otx_sensor& S, const otx_image& img,
                                        const Ray& r) {
  if (!r.ok) return;
  const int64_t b = sensor_bin(S, r);
  if (b < 0) return;
  if (img.counts) atomicAdd(reinterpret_cast<unsigned int*>(img.counts) + b, 1u);
  if (img.flux) atomicAdd(reinterpret_cast<float*>(img.flux) + b, r.inten);
  // cosine of incidence on the flat sensor (normal -z in its frame): dz
  if (img.cos_moment) atomicAdd(reinterpret_cast<float*>(img.cos_moment) + b, r.inten * r.dz);
}

// Sensor binning of the trace kernels with warp aggregation.  A warp first
// counts its lanes whose pixel equals their left neighbour's (one shuffle and
// one ballot).  Rays spread over the sensor (the precision workload's random
// fields) rarely share a pixel: those warps add with plain atomics, and skip
// the test for their next 7 rays (`skip`, a per-thread counter the kernel
// keeps across its loop; a warp's lanes update it alike), since whether a
// warp's rays repeat pixels follows from the ray order and persists.  When
// several lanes repeat a pixel (a warp of rays from one field point of a
// telescope lands in a handful of pixels), the active lanes of each pixel
// form one group (__match_any_sync on the bin index), sum their
// intensities (and cosine moments) by shared-memory atomics into the group
// leader's slot, and the leader adds the group's count and sums to the
// images with one global atomic each, so the atomics on those contended
// addresses fall by up to 32x.  Counts are exact integers however the lanes
// group; the float sums are order-dependent within FP32 rounding, as any
// atomic sum is.  Blocks of up to OTX_BIN_MAX_THREADS threads (the trace
// kernels' limit; larger blocks bin with plain atomics); image indices fit
// int32 (the host checks the image size).
#define OTX_BIN_MAX_THREADS 256
__device__ __forceinline__ void bin_ray_warp(const otx_sensor& S, const otx_image& img,
                                             const Ray& r, int& skip) {
  __shared__ float s_flux[OTX_BIN_MAX_THREADS], s_mom[OTX_BIN_MAX_THREADS];
  if (skip > 0 || blockDim.x > OTX_BIN_MAX_THREADS) {
    --skip;
    bin_ray(S, img, r);
    return;
  }
  const unsigned mask = __activemask();
  const int b = r.ok ? (int)sensor_bin(S, r) : -1;
  const int lane = threadIdx.x & 31;
  const int prev = __shfl_up_sync(mask, b, 1);
  const bool repeat = b >= 0 && lane > 0 && ((mask >> (lane - 1)) & 1u) && prev == b;
  if (__popc(__ballot_sync(mask, repeat)) < 4) {
    skip = 7;
    bin_ray(S, img, r);
    return;
  }
  const unsigned peers = __match_any_sync(mask, b);
  const int leader = __ffs(peers) - 1;
  const int slot = (threadIdx.x & ~31) + leader;
  const bool lead = lane == leader;
  const bool mom = img.cos_moment != 0;
  if (lead) {
    s_flux[threadIdx.x] = 0.f;
    if (mom) s_mom[threadIdx.x] = 0.f;
  }
  __syncwarp(mask);
  if (b >= 0) {
    atomicAdd(&s_flux[slot], r.inten);
    // cosine of incidence on the flat sensor (normal -z in its frame): dz
    if (mom) atomicAdd(&s_mom[slot], r.inten * r.dz);
  }
  __syncwarp(mask);
  if (lead && b >= 0) {
    if (img.counts) atomicAdd(reinterpret_cast<unsigned int*>(img.counts) + b, (unsigned)__popc(peers));
    if (img.flux) atomicAdd(reinterpret_cast<float*>(img.flux) + b, s_flux[threadIdx.x]);
    if (mom) atomicAdd(reinterpret_cast<float*>(img.cos_moment) + b, s_mom[threadIdx.x]);
  }
}

// Minimum resident CTAs per SM requested from the register allocator (256
// threads each): 4 for the one-ray kernels without the layered multilayer
// evaluator (64 registers, no spills: 3.41 ms per 5e7 rays of the precision
// workload against 3.96 ms at their natural 79 registers and 3 CTAs, 3.65 ms
// at 5 CTAs with spills); 2 for the one-ray kernels with it (128 registers,
// a few spilled bytes: 1.56 ms against 2.20 ms per 4e6 rays onto a 40-bilayer
// mirror at their natural ~160 registers and 1 CTA); the two-ray kernels at
// their natural register counts.
template <int RPT, bool ML>
constexpr int trace_min_blocks() {
  return RPT != 1 ? 1 : (ML ? 2 : 4);
}

template <int RPT, int MODE, bool ACC, bool ML>
__global__ void __launch_bounds__(256, trace_min_blocks<RPT, ML>())
    k_trace(const __grid_constant__ otx_system sys,
            const __grid_constant__ TraceArgs a) {
  const int64_t n = a.count;
  const int64_t step = (int64_t)gridDim.x * blockDim.x * RPT;
  const int ns = sys.num_surfaces;
  const bool bin = image_any(a.img);
  const bool final_identity = (sys.flags & OTX_SYS_FLAG_FINAL_IDENTITY) != 0;
  int bin_skip = 0;
  for (int64_t base = (int64_t)blockIdx.x * blockDim.x * RPT + threadIdx.x; base < n;
       base += step) {
    Ray r[RPT];
#pragma unroll
    for (int k = 0; k < RPT; ++k) {
      const int64_t i = base + (int64_t)k * blockDim.x;
      if (i < n) load_ray<MODE>(a, i, r[k]);
    }
    for (int s = 0; s < ns; ++s) {
      const otx_surface& S = sys.surfaces[s];
#pragma unroll
      for (int k = 0; k < RPT; ++k) {
        const int64_t i = base + (int64_t)k * blockDim.x;
        if (i < n) {
          propagate_surface<AnyKind, ML>(sys, S, r[k]);
          if (ACC) store_ray<false>(a.out, (int64_t)s * a.out.surface_stride + i, S.to_output, r[k]);
        }
      }
    }
#pragma unroll
    for (int k = 0; k < RPT; ++k) {
      const int64_t i = base + (int64_t)k * blockDim.x;
      if (i < n) {
        if (bin) bin_ray_warp(sys.sensor, a.img, r[k], bin_skip);
        if (!ACC) {
          if (final_identity)
            store_ray<true>(a.out, i, sys.final_to_output, r[k]);
          else
            store_ray<false>(a.out, i, sys.final_to_output, r[k]);
        }
      }
    }
  }
}

// ---------------------------------------------------------------- fixed shapes

// The whole surface sequence as compile-time kinds: sys.surfaces[I] is read
// at compile-time offsets (constant-bank operands, no indexed loads) and
// every type switch folds away.
template <int I, class K, class... Rest>
__device__ __forceinline__ void propagate_fixed(const otx_system& sys, Ray& r) {
  propagate_surface<K, false>(sys, sys.surfaces[I], r);
  if constexpr (sizeof...(Rest) > 0) propagate_fixed<I + 1, Rest...>(sys, r);
}

// Whether surface 0 leaves the rays of a grid input unchanged: a flat
// vacuum surface without aperture or rulings whose frame is the input frame.
// Grid rays start on its plane (z = 0) in vacuum (n = 1, no attenuation), so
// its intercept is at t = 0, the Snell step between equal indices keeps the
// (unit) direction and nothing clips: the step is an exact no-op.
template <int MODE, class K>
__device__ __forceinline__ bool first_is_noop(const otx_system& sys) {
  // (every mode but OTX_INPUT_RAYS starts its rays on the z = 0 plane)
  if constexpr (MODE != OTX_INPUT_RAYS && K::sag == OTX_SAG_FLAT && K::mat == OTX_MAT_VACUUM &&
                K::aper == OTX_APER_NONE && K::rule == OTX_RULE_NONE) {
    const otx_affine& f = sys.surfaces[0].to_local;
    return (f.flags & OTX_AFFINE_ROT_IDENTITY) && f.t_hi[0] == 0.f && f.t_hi[1] == 0.f &&
           f.t_hi[2] == 0.f && f.t_lo[0] == 0.f && f.t_lo[1] == 0.f && f.t_lo[2] == 0.f;
  } else {
    return false;
  }
}

// The shape-specialised kernels keep 6 CTAs of 256 threads resident per SM
// (at most 40 registers per thread, no spills for the Newtonian shapes):
// they are bound by instruction issue and latency, and measured on the
// precision workload 6 CTAs per SM run 4 % faster than 4 (64 registers),
// which run 9 % faster than 3; at 7 the registers spill.
template <int MODE, class K0, class... Ks>
__global__ void __launch_bounds__(256, 6)
    k_trace_fixed(const __grid_constant__ otx_system sys,
                  const __grid_constant__ TraceArgs a) {
  const int64_t n = a.count;
  const int64_t step = (int64_t)gridDim.x * blockDim.x;
  const bool bin = image_any(a.img);
  const bool final_identity = (sys.flags & OTX_SYS_FLAG_FINAL_IDENTITY) != 0;
  const bool skip0 = first_is_noop<MODE, K0>(sys);
  int bin_skip = 0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += step) {
    Ray r;
    load_ray<MODE>(a, i, r);
    if (!skip0) propagate_surface<K0, false>(sys, sys.surfaces[0], r);
    if constexpr (sizeof...(Ks) > 0) propagate_fixed<1, Ks...>(sys, r);
    if (bin) bin_ray_warp(sys.sensor, a.img, r, bin_skip);
    if (final_identity)
      store_ray<true>(a.out, i, sys.final_to_output, r);
    else
      store_ray<false>(a.out, i, sys.final_to_output, r);
  }
}

// Kind of surface i as the fixed kernels see it (a multilayer mirror on a
// bare substrate is the Fresnel mirror kind).
inline int effective_mat(const otx_system& sys, const otx_surface& s) {
  if (s.mat_type == OTX_MAT_MULTILAYER_MIRROR) {
    const otx_stack& K = sys.stacks[s.mat_stack];
    if (!stack_needs_product(sys, K))
      return OTX_MAT_FRESNEL_MIRROR;
  }
  return s.mat_type;
}

template <class... Ks>
bool shape_matches(const otx_system& sys) {
  constexpr int n = sizeof...(Ks);
  if (sys.num_surfaces != n) return false;
  const int sig[n][4] = {{Ks::sag, Ks::mat, Ks::aper, Ks::rule}...};
  for (int i = 0; i < n; ++i) {
    const otx_surface& s = sys.surfaces[i];
    if (s.sag_type != sig[i][0] || effective_mat(sys, s) != sig[i][1] ||
        s.aper_type != sig[i][2] || s.rule_type != sig[i][3])
      return false;
  }
  return true;
}

template <int MODE, class... Ks>
bool try_fixed(int grid, int block, const otx_system& sys, const TraceArgs& a,
               cudaStream_t st) {
  if (!shape_matches<Ks...>(sys)) return false;
  k_trace_fixed<MODE, Ks...><<<grid, block, 0, st>>>(sys, a);
  return true;
}

template <int MODE, bool ML>
void launch_ml(int rpt, bool acc, int grid, int block, const otx_system& sys,
               const TraceArgs& a, cudaStream_t st) {
  if (acc) {
    if (rpt == 2)
      k_trace<2, MODE, true, ML><<<grid, block, 0, st>>>(sys, a);
    else
      k_trace<1, MODE, true, ML><<<grid, block, 0, st>>>(sys, a);
  } else {
    if (rpt == 2)
      k_trace<2, MODE, false, ML><<<grid, block, 0, st>>>(sys, a);
    else
      k_trace<1, MODE, false, ML><<<grid, block, 0, st>>>(sys, a);
  }
}

// Launch of one input mode; rays_per_thread is 1 or 2; `ml` selects the
// variant able to evaluate layered multilayer stacks.
template <int MODE>
void launch_mode(int rpt, bool acc, bool ml, int grid, int block, const otx_system& sys,
                 const TraceArgs& a, cudaStream_t st) {
  if (ml)
    launch_ml<MODE, true>(rpt, acc, grid, block, sys, a, st);
  else
    launch_ml<MODE, false>(rpt, acc, grid, block, sys, a, st);
}

}  // namespace otx
