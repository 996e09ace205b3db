// The forward model's device steps around the fused trace: input rays of
// scene cells (stratified random sampling) and the exposure of an ideal
// sensor (shot and read noise).
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "../../include/optika_gb300.h"
#include "cells.cuh"
#include "philox.cuh"

namespace otx {

// IDX is the type of the cell-index arithmetic: 32-bit when every index
// of the scene fits (the divisions are then a fraction of the 64-bit ones).
template <typename IDX>
__global__ void __launch_bounds__(256) k_cell_rays(const otx_cells c, int64_t first,
                                                   int64_t count, otx_grid out) {
  const int64_t step = (int64_t)gridDim.x * blockDim.x;
  for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < count; j += step) {
    float wl, fx, fy, px, py, inten;
    cell_ray<IDX>(c, first + j, wl, fx, fy, px, py, inten);
    reinterpret_cast<float*>(out.wavelength)[j] = wl;
    reinterpret_cast<float*>(out.field_x)[j] = fx;
    reinterpret_cast<float*>(out.field_y)[j] = fy;
    reinterpret_cast<float*>(out.pupil_x)[j] = px;
    reinterpret_cast<float*>(out.pupil_y)[j] = py;
    reinterpret_cast<float*>(out.intensity)[j] = inten;
  }
}

// Uniforms of one pixel's Philox stream, four per generator call.
struct PixelStream {
  uint32_t c0, c1, k0, k1, n;
  u32x4 buf;
  int used;
  __device__ float next() {
    if (used == 4) {
      buf = philox4x32_10(u32x4{c0, c1, 0xe7905eu, n++}, k0, k1);
      used = 0;
    }
    const uint32_t x = used == 0 ? buf.x : used == 1 ? buf.y : used == 2 ? buf.z : buf.w;
    ++used;
    return u01(x);
  }
};

// Poisson variate of mean lam.  lam >= 10: transformed rejection with
// squeeze (Hormann, "The transformed rejection method for generating
// Poisson random variables", 1993), the acceptance test in double
// precision; below: the multiplication method (count uniforms until their
// product falls under exp(-lam)).  Both loops are bounded; the bounds are
// far beyond the expected iteration counts (about 1.1 and lam + 1).
__device__ double poisson(PixelStream& s, double lam) {
  if (!(lam > 0.0)) return lam == 0.0 ? 0.0 : NAN;
  if (lam >= 10.0) {
    const double slam = sqrt(lam), loglam = log(lam);
    const double b = 0.931 + 2.53 * slam;
    const double a = -0.059 + 0.02483 * b;
    const double invalpha = 1.1239 + 1.1328 / (b - 3.4);
    const double vr = 0.9277 - 3.6224 / (b - 2.0);
    for (int it = 0; it < 256; ++it) {
      const double U = (double)s.next() - 0.5;
      const double V = (double)s.next();
      const double us = 0.5 - fabs(U);
      const double k = floor((2.0 * a / us + b) * U + lam + 0.43);
      if (us >= 0.07 && V <= vr) return k;
      if (k < 0.0 || (us < 0.013 && V > us)) continue;
      if (log(V) + log(invalpha) - log(a / (us * us) + b) <= -lam + k * loglam - lgamma(k + 1.0))
        return k;
    }
    return floor(lam + 0.5);  // not reached in practice (each try accepts with p > 0.8)
  }
  const float enlam = expf(-(float)lam);
  float prod = 1.f;
  for (int k = 0; k < 512; ++k) {
    prod *= s.next();
    if (prod <= enlam) return (double)k;
  }
  return 512.0;
}

__global__ void __launch_bounds__(256) k_expose(const float* photons, float* electrons,
                                                int64_t count, float scale, float read_noise,
                                                int noise, uint64_t seed) {
  const int64_t step = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += step) {
    const float mean = scale * photons[i];
    if (!noise) {
      electrons[i] = mean;
      continue;
    }
    PixelStream s{(uint32_t)i, (uint32_t)((uint64_t)i >> 32), (uint32_t)seed,
                  (uint32_t)(seed >> 32), 0u, u32x4{0, 0, 0, 0}, 4};
    float e = (float)poisson(s, (double)mean);
    if (read_noise != 0.f) {
      // Box-Muller; 1 - u lies in (0, 1]
      const float u1 = 1.f - s.next(), u2 = s.next();
      e = fmaf(read_noise, sqrtf(-2.f * logf(u1)) * cospif(2.f * u2), e);
    }
    electrons[i] = e;
  }
}

static int grid_for(int64_t n) {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (sms <= 0) sms = 132;
  const int64_t need = (n + 255) / 256;
  const int64_t cap = (int64_t)sms * 16;
  return (int)(need < cap ? need : cap);
}

}  // namespace otx

using namespace otx;

extern "C" otx_status otx_cell_rays(const otx_cells* cells, int64_t first, int64_t count,
                                    const otx_grid* out, void* stream) {
  if (!out) return OTX_ERR_INVALID;
  if (const otx_status vs = validate_cells(cells, first, count)) return vs;
  const otx_cells& c = *cells;
  const int64_t total = (int64_t)c.nw * c.nfx * c.nfy * c.npx * c.npy;
  if (count == 0) return OTX_OK;
  if (!out->wavelength || !out->field_x || !out->field_y || !out->pupil_x || !out->pupil_y ||
      !out->intensity)
    return OTX_ERR_INVALID;
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  if (total <= (int64_t)UINT32_MAX)
    k_cell_rays<uint32_t><<<grid_for(count), 256, 0, st>>>(c, first, count, *out);
  else
    k_cell_rays<uint64_t><<<grid_for(count), 256, 0, st>>>(c, first, count, *out);
  return cudaGetLastError() == cudaSuccess ? OTX_OK : OTX_ERR_CUDA;
}

extern "C" otx_status otx_expose(const float* photons, float* electrons, int64_t count,
                                 float scale, float read_noise, int32_t noise, uint64_t seed,
                                 void* stream) {
  if (count < 0) return OTX_ERR_INVALID;
  if (count == 0) return OTX_OK;
  if (!photons || !electrons) return OTX_ERR_INVALID;
  k_expose<<<grid_for(count), 256, 0, reinterpret_cast<cudaStream_t>(stream)>>>(
      photons, electrons, count, scale, read_noise, noise, seed);
  return cudaGetLastError() == cudaSuccess ? OTX_OK : OTX_ERR_CUDA;
}
