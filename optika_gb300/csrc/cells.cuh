// One input ray of a scene cell (SequentialSystem.image): shared by the
// standalone cell-ray kernel (otx_cell_rays) and the trace kernels that
// generate their rays in place (otx_trace_cells).
#pragma once

#include <stdint.h>

#include "../../include/optika_gb300.h"
#include "philox.cuh"

namespace otx {

// Linear interpolation of the vertex table row `v` (stride `n + 1`) at
// vertex index k with weight u, then across the two wavelength vertices.
__device__ __forceinline__ float cell_lerp(const float* t, int n, int iw, int k, float uw,
                                           float u) {
  const float* a = t + (int64_t)iw * (n + 1) + k;
  const float* b = a + (n + 1);
  const float lo = fmaf(a[1] - a[0], u, a[0]);
  const float hi = fmaf(b[1] - b[0], u, b[0]);
  return fmaf(hi - lo, uw, lo);
}

// The ray of cell i (index ((((iw nfx + ifx) nfy + ify) npx + ipx) npy +
// ipy)): a uniformly drawn point of the cell (or its centre), the
// wavelength interpolated with the same weight as the field and pupil
// vertices, and the cell's flux as intensity
// (optika/systems/_sequential.py:1002-1086).  IDX is the type of the index
// arithmetic: 32-bit when every index of the scene fits.
template <typename IDX>
__device__ __forceinline__ void cell_ray(const otx_cells& c, int64_t i, float& wl, float& fx,
                                         float& fy, float& px, float& py, float& inten) {
  const uint32_t k0 = (uint32_t)c.seed, k1 = (uint32_t)(c.seed >> 32);
  IDX q = (IDX)i;
  const int ipy = (int)(q % (IDX)c.npy);
  q /= (IDX)c.npy;
  const int ipx = (int)(q % (IDX)c.npx);
  q /= (IDX)c.npx;
  const int ify = (int)(q % (IDX)c.nfy);
  q /= (IDX)c.nfy;
  const int ifx = (int)(q % (IDX)c.nfx);
  const int iw = (int)(q / (IDX)c.nfx);
  float uw = 0.5f, ufx = 0.5f, ufy = 0.5f, upx = 0.5f, upy = 0.5f;
  if (c.random) {
    // one Philox call, counter (ray index, stream 0x1ce115, 0), key =
    // seed: four uniforms from the top 24 bits of its words and a fifth
    // from the low bytes of the first three
    const u32x4 a = philox4x32_10(
        u32x4{(uint32_t)i, (uint32_t)((uint64_t)i >> 32), 0x1ce115u, 0u}, k0, k1);
    uw = u01(a.x);
    ufx = u01(a.y);
    ufy = u01(a.z);
    upx = u01(a.w);
    upy = u01(((a.x & 0xffu) << 24) | ((a.y & 0xffu) << 16) | ((a.z & 0xffu) << 8));
  }
  const float* wv = reinterpret_cast<const float*>(c.wavelength);
  wl = fmaf(wv[iw + 1] - wv[iw], uw, wv[iw]);
  fx = cell_lerp(reinterpret_cast<const float*>(c.field_x), c.nfx, iw, ifx, uw, ufx);
  fy = cell_lerp(reinterpret_cast<const float*>(c.field_y), c.nfy, iw, ify, uw, ufy);
  px = cell_lerp(reinterpret_cast<const float*>(c.pupil_x), c.npx, iw, ipx, uw, upx);
  py = cell_lerp(reinterpret_cast<const float*>(c.pupil_y), c.npy, iw, ipy, uw, upy);
  const float w =
      reinterpret_cast<const float*>(c.weight)[((int64_t)iw * c.nfx + ifx) * c.nfy + ify];
  const float wp =
      reinterpret_cast<const float*>(c.weight_pupil)[((int64_t)iw * c.npx + ipx) * c.npy + ipy];
  inten = w * wp;
}

// Checks of a cell table shared by its entry points (OTX_OK when usable).
__host__ __forceinline__ otx_status validate_cells(const otx_cells* cells, int64_t first,
                                                   int64_t count) {
  if (!cells || first < 0 || count < 0) return OTX_ERR_INVALID;
  const otx_cells& c = *cells;
  if (c.nw < 1 || c.nfx < 1 || c.nfy < 1 || c.npx < 1 || c.npy < 1) return OTX_ERR_INVALID;
  const int64_t total = (int64_t)c.nw * c.nfx * c.nfy * c.npx * c.npy;
  if (first + count > total) return OTX_ERR_SIZE;
  if (count > 0 && (!c.wavelength || !c.field_x || !c.field_y || !c.pupil_x || !c.pupil_y ||
                    !c.weight || !c.weight_pupil))
    return OTX_ERR_INVALID;
  return OTX_OK;
}

}  // namespace otx
