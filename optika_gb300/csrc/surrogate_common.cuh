// Device helpers shared by the surrogate's kernels: the configuration of a
// batch ray, the network's normalised ray inputs, the quadratic baseline
// of the image position, and a configuration's image.
#pragma once

#include "../../include/optika_gb300.h"
#include "batch_rays.cuh"

namespace otx {

// Configuration of global batch ray gid: the last c with offs[c] <= gid.
__device__ __forceinline__ int config_of(const int64_t* offs, int num_configs, int64_t gid) {
  int lo = 0, hi = num_configs - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (offs[mid] <= gid)
      lo = mid;
    else
      hi = mid - 1;
  }
  return lo;
}

// Normalised ray inputs: field and pupil by their half ranges, wavelength
// about the band centre.
__device__ __forceinline__ void ray_features(const otx_batch& b, const BatchInputs& v, float u[5]) {
  const float wl_mid = 0.5f * (b.wl_lo + b.wl_hi), wl_half = 0.5f * (b.wl_hi - b.wl_lo);
  u[0] = b.field_x_half > 0.f ? v.fx / b.field_x_half : 0.f;
  u[1] = b.field_y_half > 0.f ? v.fy / b.field_y_half : 0.f;
  u[2] = b.pupil_half > 0.f ? v.qx / b.pupil_half : 0.f;
  u[3] = b.pupil_half > 0.f ? v.qy / b.pupil_half : 0.f;
  u[4] = wl_half > 0.f ? (v.wl - wl_mid) / wl_half : 0.f;
}

// Quadratic baseline: terms 1, u0..u4, then u_i u_j for i <= j in
// lexicographic order (21 terms), coefficients c[0..20] for x, c[21..41]
// for y.
__device__ __forceinline__ void baseline_xy(const float* __restrict__ c, const float u[5],
                                            float& x, float& y) {
  float t[OTX_SURROGATE_NBASE];
  t[0] = 1.f;
#pragma unroll
  for (int i = 0; i < 5; ++i) t[1 + i] = u[i];
  int k = 6;
#pragma unroll
  for (int i = 0; i < 5; ++i)
#pragma unroll
    for (int j = i; j < 5; ++j) t[k++] = u[i] * u[j];
  float sx = 0.f, sy = 0.f;
#pragma unroll
  for (int i = OTX_SURROGATE_NBASE - 1; i >= 0; --i) {
    sx = fmaf(c[i], t[i], sx);
    sy = fmaf(c[OTX_SURROGATE_NBASE + i], t[i], sy);
  }
  x = sx;
  y = sy;
}

__device__ __forceinline__ otx_image config_image(const otx_image& img, int64_t stride, int cfg) {
  otx_image o = img;
  const int64_t off = (int64_t)cfg * stride * 4;
  if (o.counts) o.counts += off;
  if (o.flux) o.flux += off;
  if (o.cos_moment) o.cos_moment += off;
  return o;
}

}  // namespace otx
