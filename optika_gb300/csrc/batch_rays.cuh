// Rays of a batched trace, generated on the device, and the surface
// sequence they run through: shared by the batched trace and the
// surrogate's packing and fallback kernels.
#pragma once

#include "philox.cuh"
#include "trace_kernel.cuh"

namespace otx {

// Rays of the batch: wavelength, field angles and pupil position from one
// Philox block (counter: ray index, config, 0): four uniforms from the top
// 24 bits of its words and a fifth from the low bytes of the first three,
// each value formed with explicitly rounded FP32 operations so that the
// host restatement reproduces it exactly.
struct BatchInputs {
  float wl, fx, fy, qx, qy;
};

__device__ __forceinline__ BatchInputs batch_inputs(const otx_batch& b, int cfg, int64_t i) {
  const uint32_t k0 = (uint32_t)b.seed, k1 = (uint32_t)(b.seed >> 32);
  const u32x4 c0 = philox4x32_10(u32x4{(uint32_t)i, (uint32_t)(i >> 32), (uint32_t)cfg, 0u}, k0, k1);
  const uint32_t low = ((c0.x & 0xffu) << 24) | ((c0.y & 0xffu) << 16) | ((c0.z & 0xffu) << 8);
  BatchInputs v;
  v.wl = __fadd_rn(b.wl_lo, __fmul_rn(u01(c0.x), __fsub_rn(b.wl_hi, b.wl_lo)));
  v.fx = __fmul_rn(b.field_x_half, __fsub_rn(__fmul_rn(2.f, u01(c0.y)), 1.f));
  v.fy = __fmul_rn(b.field_y_half, __fsub_rn(__fmul_rn(2.f, u01(c0.z)), 1.f));
  v.qx = __fmul_rn(b.pupil_half, __fsub_rn(__fmul_rn(2.f, u01(c0.w)), 1.f));
  v.qy = __fmul_rn(b.pupil_half, __fsub_rn(__fmul_rn(2.f, u01(low)), 1.f));
  return v;
}

__device__ __forceinline__ void batch_ray(const otx_batch& b, int cfg, int64_t i, Ray& r) {
  const BatchInputs v = batch_inputs(b, cfg, i);
  const float wl = v.wl, fx = v.fx, fy = v.fy, qx = v.qx, qy = v.qy;
  r.px = qx;
  r.py = qy;
  r.pz = 0.f;
  direction_from_angles(fx, fy, r.dx, r.dy, r.dz, r.lx, r.ly, r.lz);
  r.wl = wl;
  r.inten = 1.f;
  r.att = 0.f;
  r.n = 1.f;
  r.ok = true;
  r.opl_hi = 0.f;
  r.opl_lo = 0.f;
}

template <int I, class K, class... Rest>
__device__ __forceinline__ void propagate_smem(const otx_system& sys, const otx_surface* s,
                                               Ray& r) {
  propagate_surface<K, false>(sys, s[I], r);
  if constexpr (sizeof...(Rest) > 0) propagate_smem<I + 1, Rest...>(sys, s, r);
}

// Whether the first surface leaves a batch ray unchanged: batch rays start
// on the z = 0 plane of the input frame in vacuum (n = 1, no attenuation),
// so a flat vacuum surface without aperture or rulings in that frame has its
// intercept at t = 0 and keeps the direction (the condition of
// first_is_noop, read from the staged descriptor).
__device__ __forceinline__ bool batch_first_is_noop(const otx_surface& s) {
  const otx_affine& f = s.to_local;
  return s.sag_type == OTX_SAG_FLAT && s.mat_type == OTX_MAT_VACUUM &&
         s.aper_type == OTX_APER_NONE && s.rule_type == OTX_RULE_NONE &&
         (f.flags & OTX_AFFINE_ROT_IDENTITY) && f.t_hi[0] == 0.f && f.t_hi[1] == 0.f &&
         f.t_hi[2] == 0.f && f.t_lo[0] == 0.f && f.t_lo[1] == 0.f && f.t_lo[2] == 0.f;
}

template <class K0, class... Rest>
__device__ __forceinline__ void propagate_smem_skip(const otx_system& sys, const otx_surface* s,
                                                    Ray& r, bool skip0) {
  if (!skip0) propagate_surface<K0, false>(sys, s[0], r);
  if constexpr (sizeof...(Rest) > 0) propagate_smem<1, Rest...>(sys, s, r);
}

// All surfaces of the staged sequence; skip0 (batch_first_is_noop of the
// first) leaves out the first step.
template <class... Ks>
__device__ __forceinline__ void propagate_all(const otx_system& sys, const otx_surface* s,
                                              Ray& r, bool skip0 = false) {
  if constexpr (sizeof...(Ks) > 0) {
    propagate_smem_skip<Ks...>(sys, s, r, skip0);
  } else {
    for (int k = skip0 ? 1 : 0; k < sys.num_surfaces; ++k)
      propagate_surface<AnyKind, true>(sys, s[k], r);
  }
}

// The spectrograph shape (object, spherical mirror, toroidal VLS grating,
// sensor): its batches run kernels specialised to these kinds.
using BObject = Kind<OTX_SAG_FLAT, OTX_MAT_VACUUM, OTX_APER_NONE, OTX_RULE_NONE>;
using BSphere = Kind<OTX_SAG_SPHERE, OTX_MAT_MIRROR, OTX_APER_CIRCULAR, OTX_RULE_NONE>;
using BGrating = Kind<OTX_SAG_TOROID, OTX_MAT_MIRROR, OTX_APER_NONE, OTX_RULE_POLY1D>;
using BSensor = Kind<OTX_SAG_FLAT, OTX_MAT_VACUUM, OTX_APER_RECTANGULAR, OTX_RULE_NONE>;

}  // namespace otx
