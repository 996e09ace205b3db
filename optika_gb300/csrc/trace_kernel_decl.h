// Declarations of the per-mode launchers (defined in trace_kernel.cuh and
// explicitly instantiated in trace_rays.cu / trace_grid_inf.cu /
// trace_grid_fin.cu).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/optika_gb300.h"

namespace otx {

// Whether any sensor image of the call is produced.
__host__ __device__ __forceinline__ bool image_any(const otx_image& img) {
  return img.counts != 0 || img.flux != 0 || img.cos_moment != 0;
}

// Whether a multilayer stack needs the transfer-matrix product: layers, or
// a rough substrate.  A smooth bare substrate takes the Fresnel form, which
// has no interface profile and keeps the shape-specialised kernels small.
__host__ __device__ __forceinline__ bool stack_needs_product(const otx_system& sys,
                                                             const otx_stack& K) {
  return K.pre_count > 0 || (K.per_count > 0 && K.num_periods > 0) || K.post_count > 0 ||
         (K.substrate >= 0 && K.substrate < OTX_MAX_LAYERS &&
          sys.layers[K.substrate].interface_type != OTX_PROFILE_NONE);
}

// Checks of a system descriptor shared by every entry point that traces
// through it: type tags, pool indices and sizes (OTX_OK when usable).
otx_status validate_system(const otx_system* sys);

// Input modes of the trace kernels beyond the OTX_INPUT_* of a system:
// scene cells whose rays the kernel generates itself (otx_trace_cells),
// with the object at infinity or at a finite distance.
#define OTX_MODE_CELLS_INFINITY 101
#define OTX_MODE_CELLS_FINITE 102

struct TraceArgs {
  otx_rays in;
  otx_grid grid;
  otx_rays out;
  otx_image img;
  int64_t count;
  otx_cells cells;     // cell modes: the scene's tables
  int64_t first;       // cell modes: cell index of ray 0
  int32_t cells_idx32; // cell modes: every cell index fits 32 bits
};

template <int MODE>
void launch_mode(int rpt, bool acc, bool ml, int grid, int block, const otx_system& sys,
                 const TraceArgs& a, cudaStream_t st);

extern template void launch_mode<OTX_INPUT_RAYS>(int, bool, bool, int, int, const otx_system&,
                                                 const TraceArgs&, cudaStream_t);
extern template void launch_mode<OTX_INPUT_GRID_INFINITY>(int, bool, bool, int, int,
                                                          const otx_system&,
                                                          const TraceArgs&, cudaStream_t);
extern template void launch_mode<OTX_INPUT_GRID_FINITE>(int, bool, bool, int, int,
                                                        const otx_system&,
                                                        const TraceArgs&, cudaStream_t);
extern template void launch_mode<OTX_MODE_CELLS_INFINITY>(int, bool, bool, int, int,
                                                          const otx_system&,
                                                          const TraceArgs&, cudaStream_t);
extern template void launch_mode<OTX_MODE_CELLS_FINITE>(int, bool, bool, int, int,
                                                        const otx_system&,
                                                        const TraceArgs&, cudaStream_t);

// Launch a kernel specialised for the system's shape if one exists
// (trace_fixed.cu); false when the generic kernel must run.
bool launch_fixed(int mode, bool acc, int rpt, int grid, int block, const otx_system& sys,
                  const TraceArgs& a, cudaStream_t st);

}  // namespace otx
