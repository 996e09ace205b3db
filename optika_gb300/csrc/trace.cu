// C-ABI entry points of the fused sequential raytrace: descriptor
// validation, launch geometry, and dispatch to the per-mode kernels.
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include <mutex>

#include "../../include/optika_gb300.h"
#include "cells.cuh"
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

otx_status validate_system(const otx_system* sys) {
  if (!sys) return OTX_ERR_INVALID;
  if (sys->abi_version != OTX_ABI_VERSION) return OTX_ERR_INVALID;
  if (sys->num_surfaces < 1 || sys->num_surfaces > OTX_MAX_SURFACES) return OTX_ERR_SIZE;
  for (int i = 0; i < sys->num_surfaces; ++i) {
    const otx_surface& s = sys->surfaces[i];
    if (s.sag_type < OTX_SAG_FLAT || s.sag_type > OTX_SAG_CYLINDER) return OTX_ERR_UNSUPPORTED;
    if (s.mat_type < OTX_MAT_VACUUM || s.mat_type > OTX_MAT_MEASURED_MIRROR)
      return OTX_ERR_UNSUPPORTED;
    if (s.mat_type == OTX_MAT_MEASURED_MIRROR &&
        (s.mat_table < 0 || s.mat_table >= OTX_MAX_STACKS * 4 ||
         sys->tables[s.mat_table].count < 1 || sys->table_data == 0))
      return OTX_ERR_INVALID;
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
    if (s.rule_type != OTX_RULE_NONE) {
      if (s.rule_eff_type < OTX_RULE_EFF_IDEAL || s.rule_eff_type > OTX_RULE_EFF_RECTANGULAR)
        return OTX_ERR_UNSUPPORTED;
      if (s.rule_eff_type == OTX_RULE_EFF_MEASURED &&
          (s.rule_table < 0 || s.rule_table >= OTX_MAX_STACKS * 4 ||
           sys->tables[s.rule_table].count < 1 || sys->table_data == 0))
        return OTX_ERR_INVALID;
    }
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
  if (!img || !image_any(*img)) return OTX_OK;
  const otx_sensor& S = sys->sensor;
  if (S.num_x < 1 || S.num_y < 1 || S.num_w < 1) return OTX_ERR_INVALID;
  // pixel indices are int32 in the binning
  if ((int64_t)S.num_w * S.num_x * S.num_y > INT32_MAX) return OTX_ERR_SIZE;
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
  const int rpt_req = launch ? launch->rays_per_thread : 0;  // 0: the library's choice
  int rpt = rpt_req > 0 ? rpt_req : 1;
  if (rpt != 1 && rpt != 2) return OTX_ERR_INVALID;
  int block = (launch && launch->block_size > 0) ? launch->block_size : 256;
  if (block > 256 || block % 32 != 0) return OTX_ERR_INVALID;
  const bool acc = launch && launch->accumulate;
  if (a.count == 0) return OTX_OK;
  const int64_t per_cta = (int64_t)block * rpt;
  int64_t need = (a.count + per_cta - 1) / per_cta;
  // about one ray per thread: measured on the precision workload (1e8 rays,
  // 6 CTAs resident per SM), 4.28 ms at 64 or more CTAs per SM of grid
  // against 4.36 ms at 32, 4.44 ms at 16 and 4.63 ms at one wave (6); the
  // cap only bounds the grid of very large calls, which then stride
  const int64_t cap = (int64_t)num_sms() * 4096;
  const int grid = (int)(need < cap ? need : cap);
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  // the heavy multilayer variant only when a surface uses a layered stack
  bool ml = false;
  for (int i = 0; i < sys->num_surfaces; ++i) {
    const otx_surface& s = sys->surfaces[i];
    if (s.mat_type == OTX_MAT_MULTILAYER_MIRROR || s.mat_type == OTX_MAT_MULTILAYER_FILM) {
      if (stack_needs_product(*sys, sys->stacks[s.mat_stack])) ml = true;
    }
  }
  if (!(launch && launch->generic_only) &&
      launch_fixed(mode, acc, rpt_req > 0 ? rpt_req : 0, grid, block, *sys, a, st))
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
    case OTX_MODE_CELLS_INFINITY:
      launch_mode<OTX_MODE_CELLS_INFINITY>(rpt, acc, ml, grid, block, *sys, a, st);
      break;
    case OTX_MODE_CELLS_FINITE:
      launch_mode<OTX_MODE_CELLS_FINITE>(rpt, acc, ml, grid, block, *sys, a, st);
      break;
    default:
      return OTX_ERR_INVALID;
  }
  return cudaGetLastError() == cudaSuccess ? OTX_OK : OTX_ERR_CUDA;
}

// ---------------------------------------------------------------- host staging

// Two ways for host arrays.  Page-locked arrays that the GPU addresses at
// their host address (every pinned allocation under unified addressing,
// as on GB300 where the GPU reaches Grace memory over NVLink-C2C) are read
// and written by the trace kernel itself: one launch, no staging, the
// loads and stores crossing C2C at the link's rate.  Other (pageable)
// arrays are staged through the GPU in chunks: slot s of the workspace
// holds one chunk's strided inputs and its outputs; chunk i's
// host->device copy runs on the copy-in stream, its trace on the caller's
// stream and its device->host copy on the copy-out stream, so with three
// slots the copy in of chunk i + 1, the trace of chunk i and the copy out
// of chunk i - 1 overlap.
constexpr int HOST_SLOTS = 3;
constexpr int HOST_MAX_DEVICES = 64;
constexpr int64_t HOST_ALIGN = 256;
constexpr int64_t HOST_HEAD = 256;  // broadcast scalars of the grid
constexpr int HOST_TARGET_CHUNKS = 16;
constexpr int64_t HOST_MIN_CHUNK = 1 << 20;

struct HostPipe {
  bool ready = false;
  cudaStream_t in = nullptr, out = nullptr;
  cudaEvent_t start = nullptr, end = nullptr;
  cudaEvent_t copied[HOST_SLOTS], traced[HOST_SLOTS], drained[HOST_SLOTS];
};

static HostPipe g_pipes[HOST_MAX_DEVICES];
static std::mutex g_pipe_mu;

static otx_status host_pipe(HostPipe** out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= HOST_MAX_DEVICES)
    return OTX_ERR_CUDA;
  HostPipe& p = g_pipes[dev];
  if (!p.ready) {
    const unsigned f = cudaEventDisableTiming;
    if (cudaStreamCreateWithFlags(&p.in, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithFlags(&p.out, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&p.start, f) != cudaSuccess ||
        cudaEventCreateWithFlags(&p.end, f) != cudaSuccess)
      return OTX_ERR_CUDA;
    for (int s = 0; s < HOST_SLOTS; ++s) {
      if (cudaEventCreateWithFlags(&p.copied[s], f) != cudaSuccess ||
          cudaEventCreateWithFlags(&p.traced[s], f) != cudaSuccess ||
          cudaEventCreateWithFlags(&p.drained[s], f) != cudaSuccess)
        return OTX_ERR_CUDA;
    }
    p.ready = true;
  }
  *out = &p;
  return OTX_OK;
}

static int64_t align_up(int64_t x) { return (x + HOST_ALIGN - 1) / HOST_ALIGN * HOST_ALIGN; }

// The output fields of otx_rays in declaration order with their element sizes.
static void out_fields(const otx_rays* r, uint64_t* ptrs[12], int sizes[12]) {
  otx_rays* m = const_cast<otx_rays*>(r);
  uint64_t* p[12] = {&m->px, &m->py, &m->pz, &m->dx, &m->dy, &m->dz, &m->wavelength,
                     &m->intensity, &m->attenuation, &m->index_refraction, &m->unvignetted,
                     &m->opl};
  for (int i = 0; i < 12; ++i) {
    ptrs[i] = p[i];
    sizes[i] = i == 10 ? 1 : (i == 11 ? 8 : 4);
  }
}

struct HostPlan {
  int64_t chunk = 0;     // rays per chunk
  int64_t slot = 0;      // bytes per slot
  int64_t needed = 0;    // workspace bytes for this plan
  int surfaces = 1;      // output planes (accumulate: one per surface)
};

// Inputs: the five grid arrays and the intensity, each strided (stride 1,
// staged per chunk) or broadcast (stride 0, staged once in the head).
static void grid_fields(const otx_grid* g, uint64_t ptrs[6], int64_t strides[6]) {
  const uint64_t p[6] = {g->wavelength, g->field_x, g->field_y, g->pupil_x, g->pupil_y,
                         g->intensity};
  const int64_t s[6] = {g->stride_wavelength, g->stride_field, g->stride_field,
                        g->stride_pupil, g->stride_pupil, g->stride_intensity};
  for (int i = 0; i < 6; ++i) {
    ptrs[i] = p[i];
    strides[i] = s[i];
  }
}

static int64_t slot_bytes(const otx_grid* g, const otx_rays* o, int surfaces, int64_t chunk) {
  uint64_t gp[6];
  int64_t gs[6];
  grid_fields(g, gp, gs);
  int64_t b = 0;
  for (int i = 0; i < 6; ++i)
    if (gp[i] && gs[i] != 0) b += align_up(chunk * 4);
  uint64_t* op[12];
  int sz[12];
  out_fields(o, op, sz);
  for (int i = 0; i < 12; ++i)
    if (*op[i]) b += align_up(chunk * sz[i] * (int64_t)surfaces);
  return b;
}

// True when the GPU addresses [p, p + bytes) at p: page-locked host memory
// mapped at the same address (checked at both ends of the range).
static bool mapped_same(uint64_t p, int64_t bytes) {
  if (!p || bytes <= 0) return true;
  const uint64_t ends[2] = {p, p + (uint64_t)bytes - 1};
  for (uint64_t q : ends) {
    cudaPointerAttributes at;
    memset(&at, 0, sizeof(at));
    if (cudaPointerGetAttributes(&at, reinterpret_cast<void*>(q)) != cudaSuccess) {
      cudaGetLastError();  // clear the sticky-free error of an unknown pointer
      return false;
    }
    if (at.type != cudaMemoryTypeHost || reinterpret_cast<uint64_t>(at.devicePointer) != q)
      return false;
  }
  return true;
}

// Every strided input and every output of the call is mapped (see above).
static bool all_mapped(const otx_grid* g, const otx_rays* o, int surfaces) {
  uint64_t gp[6];
  int64_t gs[6];
  grid_fields(g, gp, gs);
  for (int i = 0; i < 6; ++i)
    if (gp[i] && gs[i] != 0 && !mapped_same(gp[i], g->count * 4)) return false;
  uint64_t* op[12];
  int sz[12];
  out_fields(o, op, sz);
  const int64_t planes = surfaces > 1 ? (int64_t)(surfaces - 1) * o->surface_stride + g->count
                                      : g->count;
  for (int i = 0; i < 12; ++i)
    if (*op[i] && !mapped_same(*op[i], planes * sz[i])) return false;
  return true;
}

static HostPlan plan_host(const otx_grid* g, const otx_rays* o, int surfaces, int64_t workspace) {
  HostPlan p;
  p.surfaces = surfaces;
  const int64_t n = g->count;
  int64_t chunk = (n + HOST_TARGET_CHUNKS - 1) / HOST_TARGET_CHUNKS;
  chunk = (chunk + HOST_MIN_CHUNK - 1) / HOST_MIN_CHUNK * HOST_MIN_CHUNK;
  if (chunk > n) chunk = n > 0 ? n : 1;
  if (workspace >= 0) {
    // shrink to what the given workspace holds
    while (chunk > 1 && HOST_HEAD + HOST_SLOTS * slot_bytes(g, o, surfaces, chunk) > workspace)
      chunk = chunk > 4096 ? chunk / 2 : chunk - 1;
  }
  p.chunk = chunk;
  p.slot = slot_bytes(g, o, surfaces, chunk);
  p.needed = HOST_HEAD + HOST_SLOTS * p.slot;
  return p;
}

}  // namespace otx

using namespace otx;

extern "C" {

int64_t otx_trace_grid_host_workspace(const otx_grid* in, const otx_rays* out, int32_t surfaces) {
  if (!in || !out || in->count < 0 || surfaces < 1) return -1;
  if (in->count > 0 && all_mapped(in, out, surfaces)) return HOST_HEAD;
  return plan_host(in, out, surfaces, -1).needed;
}

otx_status otx_trace_grid_host(const otx_system* sys, const otx_grid* in, const otx_rays* out,
                               const otx_image* image, const otx_launch* launch, void* workspace,
                               int64_t workspace_bytes, void* stream) {
  otx_status st = validate_system(sys);
  if (st != OTX_OK) return st;
  if (!in || !out || in->count < 0) return OTX_ERR_INVALID;
  if (sys->input_mode != OTX_INPUT_GRID_INFINITY && sys->input_mode != OTX_INPUT_GRID_FINITE)
    return OTX_ERR_INVALID;
  if (in->count > 0 && (!in->wavelength || !in->field_x || !in->field_y || !in->pupil_x ||
                        !in->pupil_y))
    return OTX_ERR_INVALID;
  uint64_t gp[6];
  int64_t gs[6];
  grid_fields(in, gp, gs);
  for (int i = 0; i < 6; ++i)
    if (gs[i] != 0 && gs[i] != 1) return OTX_ERR_INVALID;  // host arrays: contiguous or scalar
  st = validate_image(sys, image);
  if (st != OTX_OK) return st;
  const bool acc = launch && launch->accumulate;
  const int surfaces = acc ? sys->num_surfaces : 1;
  if (acc && out->surface_stride < in->count) return OTX_ERR_INVALID;
  const int64_t n = in->count;
  if (n == 0) return OTX_OK;
  if (!workspace || (reinterpret_cast<uintptr_t>(workspace) % HOST_ALIGN) != 0)
    return OTX_ERR_INVALID;
  if (launch && ((launch->rays_per_thread != 0 && launch->rays_per_thread != 1 &&
                  launch->rays_per_thread != 2) ||
                 launch->block_size < 0 || launch->block_size > 256 ||
                 launch->block_size % 32 != 0))
    return OTX_ERR_INVALID;
  if (workspace_bytes < HOST_HEAD) return OTX_ERR_SIZE;
  cudaStream_t cs = reinterpret_cast<cudaStream_t>(stream);
  char* ws = reinterpret_cast<char*>(workspace);
  float* head = reinterpret_cast<float*>(ws);
#define OTX_CK(x) \
  if ((x) != cudaSuccess) return OTX_ERR_CUDA
  if (all_mapped(in, out, surfaces)) {
    // the kernel reads and writes the host arrays in place; broadcast
    // scalars go to the head so that no thread reads host memory for them
    otx_grid g = *in;
    uint64_t* gdst[6] = {&g.wavelength, &g.field_x, &g.field_y, &g.pupil_x, &g.pupil_y,
                         &g.intensity};
    for (int i = 0; i < 6; ++i) {
      if (!gp[i] || gs[i] != 0) continue;
      OTX_CK(cudaMemcpyAsync(head + i, reinterpret_cast<const void*>(gp[i]), 4,
                             cudaMemcpyHostToDevice, cs));
      *gdst[i] = reinterpret_cast<uint64_t>(head + i);
    }
    TraceArgs a;
    memset(&a, 0, sizeof(a));
    a.grid = g;
    a.out = *out;
    if (image) a.img = *image;
    a.count = n;
    return launch_trace(sys, sys->input_mode, a, launch, stream);
  }
  const HostPlan plan = plan_host(in, out, surfaces, workspace_bytes);
  if (plan.needed > workspace_bytes || plan.chunk < 1) return OTX_ERR_SIZE;

  std::lock_guard<std::mutex> lock(g_pipe_mu);
  HostPipe* pp = nullptr;
  st = host_pipe(&pp);
  if (st != OTX_OK) return st;
  HostPipe& P = *pp;
  // the copies start after the caller's earlier work on its stream
  OTX_CK(cudaEventRecord(P.start, cs));
  OTX_CK(cudaStreamWaitEvent(P.in, P.start, 0));
  OTX_CK(cudaStreamWaitEvent(P.out, P.start, 0));
  // broadcast scalars into the head
  for (int i = 0; i < 6; ++i)
    if (gp[i] && gs[i] == 0)
      OTX_CK(cudaMemcpyAsync(head + i, reinterpret_cast<const void*>(gp[i]), 4,
                             cudaMemcpyHostToDevice, P.in));
  uint64_t* op[12];
  int osz[12];
  out_fields(out, op, osz);
  const int64_t nchunks = (n + plan.chunk - 1) / plan.chunk;
  for (int64_t c = 0; c < nchunks; ++c) {
    const int s = (int)(c % HOST_SLOTS);
    const int64_t first = c * plan.chunk;
    const int64_t cn = first + plan.chunk <= n ? plan.chunk : n - first;
    char* slot = ws + HOST_HEAD + s * plan.slot;
    // inputs: wait until the trace that last read this slot is done
    if (c >= HOST_SLOTS) OTX_CK(cudaStreamWaitEvent(P.in, P.traced[s], 0));
    otx_grid g = *in;
    uint64_t* gdst[6] = {&g.wavelength, &g.field_x, &g.field_y, &g.pupil_x, &g.pupil_y,
                         &g.intensity};
    char* cur = slot;
    for (int i = 0; i < 6; ++i) {
      if (!gp[i]) continue;
      if (gs[i] == 0) {
        *gdst[i] = reinterpret_cast<uint64_t>(head + i);
        continue;
      }
      OTX_CK(cudaMemcpyAsync(cur, reinterpret_cast<const float*>(gp[i]) + first, cn * 4,
                             cudaMemcpyHostToDevice, P.in));
      *gdst[i] = reinterpret_cast<uint64_t>(cur);
      cur += align_up(plan.chunk * 4);
    }
    g.count = cn;
    OTX_CK(cudaEventRecord(P.copied[s], P.in));
    // outputs of this slot: the previous copy out of the slot must be done
    otx_rays o = *out;
    uint64_t* odst[12];
    int dummy[12];
    out_fields(&o, odst, dummy);
    char* obase[12];
    for (int i = 0; i < 12; ++i) {
      obase[i] = nullptr;
      if (!*op[i]) continue;
      obase[i] = cur;
      *odst[i] = reinterpret_cast<uint64_t>(cur);
      cur += align_up(plan.chunk * osz[i] * (int64_t)surfaces);
    }
    o.count = cn;
    o.surface_stride = acc ? plan.chunk : 0;
    OTX_CK(cudaStreamWaitEvent(cs, P.copied[s], 0));
    if (c >= HOST_SLOTS) OTX_CK(cudaStreamWaitEvent(cs, P.drained[s], 0));
    TraceArgs a;
    memset(&a, 0, sizeof(a));
    a.grid = g;
    a.out = o;
    if (image) a.img = *image;
    a.count = cn;
    st = launch_trace(sys, sys->input_mode, a, launch, stream);
    if (st != OTX_OK) return st;
    OTX_CK(cudaEventRecord(P.traced[s], cs));
    // copy out: one copy per field and surface plane (1-D copies: a 2-D
    // copy into pageable memory was seen to land nothing on GB300)
    OTX_CK(cudaStreamWaitEvent(P.out, P.traced[s], 0));
    for (int i = 0; i < 12; ++i) {
      if (!obase[i]) continue;
      const size_t e = (size_t)osz[i];
      for (int j = 0; j < surfaces; ++j) {
        char* dst = reinterpret_cast<char*>(*op[i]) +
                    ((size_t)j * (size_t)(acc ? out->surface_stride : 0) + (size_t)first) * e;
        const char* src = obase[i] + (size_t)j * (size_t)plan.chunk * e;
        OTX_CK(cudaMemcpyAsync(dst, src, (size_t)cn * e, cudaMemcpyDeviceToHost, P.out));
      }
    }
    OTX_CK(cudaEventRecord(P.drained[s], P.out));
  }
  // the caller's stream continues once every copy has landed
  OTX_CK(cudaEventRecord(P.end, P.out));
  OTX_CK(cudaStreamWaitEvent(cs, P.end, 0));
#undef OTX_CK
  return OTX_OK;
}

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
    case 13: return sizeof(otx_mlp);
    case 14: return sizeof(otx_cells);
    case 15: return sizeof(otx_stop_solve);
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

otx_status otx_trace_cells(const otx_system* sys, const otx_cells* cells, int64_t first,
                           int64_t count, const otx_image* image, const otx_launch* launch,
                           void* stream) {
  otx_status st = validate_system(sys);
  if (st != OTX_OK) return st;
  if (sys->input_mode != OTX_INPUT_GRID_INFINITY && sys->input_mode != OTX_INPUT_GRID_FINITE)
    return OTX_ERR_INVALID;
  st = validate_cells(cells, first, count);
  if (st != OTX_OK) return st;
  if (!image || !image_any(*image)) return OTX_ERR_INVALID;  // the image is the output
  st = validate_image(sys, image);
  if (st != OTX_OK) return st;
  if (launch && launch->accumulate) return OTX_ERR_INVALID;
  const otx_cells& c = *cells;
  const int64_t total = (int64_t)c.nw * c.nfx * c.nfy * c.npx * c.npy;
  TraceArgs a;
  memset(&a, 0, sizeof(a));
  a.img = *image;
  a.count = count;
  a.cells = c;
  a.first = first;
  a.cells_idx32 = total <= (int64_t)UINT32_MAX ? 1 : 0;
  const int mode = sys->input_mode == OTX_INPUT_GRID_INFINITY ? OTX_MODE_CELLS_INFINITY
                                                              : OTX_MODE_CELLS_FINITE;
  return launch_trace(sys, mode, a, launch, stream);
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
