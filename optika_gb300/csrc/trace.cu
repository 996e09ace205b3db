// C-ABI entry points of the fused sequential raytrace: descriptor
// validation, launch geometry, and dispatch to the per-mode kernels.
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include "../../include/optika_gb300.h"
#include "trace_kernel_decl.h"

namespace otx {

// ---------------------------------------------------------------- host side

static int g_num_sms = 0;

static int num_sms() {
  if (g_num_sms == 0) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&g_num_sms, cudaDevAttrMultiProcessorCount, dev);
    if (g_num_sms <= 0) g_num_sms = 132;
  }
  return g_num_sms;
}

static otx_status validate_system(const otx_system* sys) {
  if (!sys) return OTX_ERR_INVALID;
  if (sys->abi_version != OTX_ABI_VERSION) return OTX_ERR_INVALID;
  if (sys->num_surfaces < 1 || sys->num_surfaces > OTX_MAX_SURFACES) return OTX_ERR_SIZE;
  for (int i = 0; i < sys->num_surfaces; ++i) {
    const otx_surface& s = sys->surfaces[i];
    if (s.sag_type < OTX_SAG_FLAT || s.sag_type > OTX_SAG_TOROID) return OTX_ERR_UNSUPPORTED;
    if (s.mat_type < OTX_MAT_VACUUM || s.mat_type > OTX_MAT_MULTILAYER_FILM)
      return OTX_ERR_UNSUPPORTED;
    if (s.aper_type < OTX_APER_NONE || s.aper_type > OTX_APER_POLYGON) return OTX_ERR_UNSUPPORTED;
    if (s.rule_type < OTX_RULE_NONE || s.rule_type > OTX_RULE_HOLOGRAPHIC)
      return OTX_ERR_UNSUPPORTED;
    if (s.mat_type == OTX_MAT_MULTILAYER_MIRROR || s.mat_type == OTX_MAT_MULTILAYER_FILM) {
      if (s.mat_stack < 0 || s.mat_stack >= OTX_MAX_STACKS) return OTX_ERR_INVALID;
    }
    if (s.aper_type == OTX_APER_POLYGON) {
      if (s.aper_vertex_begin < 0 || s.aper_vertex_count < 3 ||
          s.aper_vertex_begin + s.aper_vertex_count > OTX_MAX_VERTICES)
        return OTX_ERR_INVALID;
    }
    if (s.rule_type == OTX_RULE_POLY1D &&
        (s.rule_num_terms < 0 || s.rule_num_terms > OTX_MAX_POLY_TERMS))
      return OTX_ERR_SIZE;
  }
  for (int k = 0; k < OTX_MAX_STACKS; ++k) {
    const otx_stack& K = sys->stacks[k];
    const int32_t b[3] = {K.pre_begin, K.per_begin, K.post_begin};
    const int32_t c[3] = {K.pre_count, K.per_count, K.post_count};
    for (int j = 0; j < 3; ++j) {
      if (c[j] < 0 || (c[j] > 0 && (b[j] < 0 || b[j] + c[j] > OTX_MAX_LAYERS))) return OTX_ERR_INVALID;
    }
    if (K.substrate >= OTX_MAX_LAYERS) return OTX_ERR_INVALID;
    if (K.num_periods < 0) return OTX_ERR_INVALID;
  }
  for (int k = 0; k < OTX_MAX_LAYERS; ++k) {
    const int t = sys->layers[k].table;
    if (t >= OTX_MAX_STACKS * 4) return OTX_ERR_INVALID;
    if (t >= 0 && (sys->tables[t].count < 1 || sys->table_data == 0)) return OTX_ERR_INVALID;
  }
  return OTX_OK;
}

static otx_status validate_image(const otx_system* sys, const otx_image* img) {
  if (!img || (!img->counts && !img->flux)) return OTX_OK;
  const otx_sensor& S = sys->sensor;
  if (S.num_x < 1 || S.num_y < 1 || S.num_w < 1) return OTX_ERR_INVALID;
  if (!(S.width_x > 0.f) || !(S.width_y > 0.f)) return OTX_ERR_INVALID;
  return OTX_OK;
}

// Derived sensor fields (inverse pitches) are computed here, on the host
// copy that becomes the kernel parameter; callers need not set them.
static void fill_sensor(otx_sensor& S) {
  S.inv_width_x = S.width_x > 0.f ? 1.f / S.width_x : 0.f;
  S.inv_width_y = S.width_y > 0.f ? 1.f / S.width_y : 0.f;
  S.inv_width_w = (S.w_hi > S.w_lo) ? (float)S.num_w / (S.w_hi - S.w_lo) : 0.f;
}

static otx_status launch_trace(const otx_system* sys_in, int mode, const TraceArgs& a,
                               const otx_launch* launch, void* stream) {
  otx_system local = *sys_in;
  fill_sensor(local.sensor);
  const otx_system* sys = &local;
  int rpt = (launch && launch->rays_per_thread > 0) ? launch->rays_per_thread : 1;
  if (rpt != 1 && rpt != 2) return OTX_ERR_INVALID;
  int block = (launch && launch->block_size > 0) ? launch->block_size : 256;
  if (block > 256 || block % 32 != 0) return OTX_ERR_INVALID;
  const bool acc = launch && launch->accumulate;
  if (a.count == 0) return OTX_OK;
  const int64_t per_cta = (int64_t)block * rpt;
  int64_t need = (a.count + per_cta - 1) / per_cta;
  const int64_t cap = (int64_t)num_sms() * 16;
  const int grid = (int)(need < cap ? need : cap);
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  // the heavy multilayer variant only when a surface uses a layered stack
  bool ml = false;
  for (int i = 0; i < sys->num_surfaces; ++i) {
    const otx_surface& s = sys->surfaces[i];
    if (s.mat_type == OTX_MAT_MULTILAYER_MIRROR || s.mat_type == OTX_MAT_MULTILAYER_FILM) {
      const otx_stack& K = sys->stacks[s.mat_stack];
      if (K.pre_count > 0 || (K.per_count > 0 && K.num_periods > 0) || K.post_count > 0)
        ml = true;
    }
  }
  if (!(launch && launch->generic_only) && launch_fixed(mode, acc, rpt, grid, block, *sys, a, st))
    return cudaGetLastError() == cudaSuccess ? OTX_OK : OTX_ERR_CUDA;
  switch (mode) {
    case OTX_INPUT_RAYS:
      launch_mode<OTX_INPUT_RAYS>(rpt, acc, ml, grid, block, *sys, a, st);
      break;
    case OTX_INPUT_GRID_INFINITY:
      launch_mode<OTX_INPUT_GRID_INFINITY>(rpt, acc, ml, grid, block, *sys, a, st);
      break;
    case OTX_INPUT_GRID_FINITE:
      launch_mode<OTX_INPUT_GRID_FINITE>(rpt, acc, ml, grid, block, *sys, a, st);
      break;
    default:
      return OTX_ERR_INVALID;
  }
  return cudaGetLastError() == cudaSuccess ? OTX_OK : OTX_ERR_CUDA;
}

}  // namespace otx

using namespace otx;

extern "C" {

int64_t otx_sizeof(int32_t which) {
  switch (which) {
    case 0: return sizeof(otx_system);
    case 1: return sizeof(otx_surface);
    case 2: return sizeof(otx_rays);
    case 3: return sizeof(otx_grid);
    case 4: return sizeof(otx_image);
    case 5: return sizeof(otx_launch);
    case 6: return sizeof(otx_affine);
    case 7: return sizeof(otx_sensor);
    case 8: return sizeof(otx_layer);
    case 9: return sizeof(otx_stack);
    case 10: return sizeof(otx_periodic_stack);
    case 11: return sizeof(otx_batch);
    case 12: return sizeof(otx_surrogate);
    default: return -1;
  }
}

int32_t otx_abi_version(void) { return OTX_ABI_VERSION; }

const char* otx_status_string(otx_status s) {
  switch (s) {
    case OTX_OK: return "ok";
    case OTX_ERR_INVALID: return "invalid descriptor or argument";
    case OTX_ERR_UNSUPPORTED: return "unsupported type tag";
    case OTX_ERR_CUDA: return "CUDA runtime error";
    case OTX_ERR_SIZE: return "size exceeds a documented maximum";
    case OTX_ERR_TIMEOUT: return "bounded device wait gave up";
    default: return "unknown status";
  }
}

otx_status otx_trace_rays(const otx_system* sys, const otx_rays* in, const otx_rays* out,
                          const otx_image* image, const otx_launch* launch, void* stream) {
  otx_status st = validate_system(sys);
  if (st != OTX_OK) return st;
  if (!in || !out || in->count < 0) return OTX_ERR_INVALID;
  if (in->count > 0 && (!in->px || !in->py || !in->pz || !in->dx || !in->dy || !in->dz))
    return OTX_ERR_INVALID;
  st = validate_image(sys, image);
  if (st != OTX_OK) return st;
  if (launch && launch->accumulate && out->surface_stride < in->count) return OTX_ERR_INVALID;
  TraceArgs a;
  memset(&a, 0, sizeof(a));
  a.in = *in;
  a.out = *out;
  if (image) a.img = *image;
  a.count = in->count;
  return launch_trace(sys, OTX_INPUT_RAYS, a, launch, stream);
}

otx_status otx_trace_grid(const otx_system* sys, const otx_grid* in, const otx_rays* out,
                          const otx_image* image, const otx_launch* launch, void* stream) {
  otx_status st = validate_system(sys);
  if (st != OTX_OK) return st;
  if (!in || !out || in->count < 0) return OTX_ERR_INVALID;
  if (sys->input_mode != OTX_INPUT_GRID_INFINITY && sys->input_mode != OTX_INPUT_GRID_FINITE)
    return OTX_ERR_INVALID;
  if (in->count > 0 && (!in->wavelength || !in->field_x || !in->field_y || !in->pupil_x ||
                        !in->pupil_y))
    return OTX_ERR_INVALID;
  if (in->stride_wavelength < 0 || in->stride_field < 0 || in->stride_pupil < 0 ||
      in->stride_intensity < 0)
    return OTX_ERR_INVALID;
  st = validate_image(sys, image);
  if (st != OTX_OK) return st;
  if (launch && launch->accumulate && out->surface_stride < in->count) return OTX_ERR_INVALID;
  TraceArgs a;
  memset(&a, 0, sizeof(a));
  a.grid = *in;
  a.out = *out;
  if (image) a.img = *image;
  a.count = in->count;
  return launch_trace(sys, sys->input_mode, a, launch, stream);
}

}  // extern "C"
