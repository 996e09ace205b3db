// Trace kernels specialised for fixed system shapes.
//
// A system whose surface kinds match one of the shapes below runs a kernel
// with the surface sequence compiled in; every other system runs the
// generic kernel (trace_kernel.cuh), which reads the kinds at run time.
#include "trace_kernel.cuh"
#include "trace_pair.cuh"

namespace otx {

using Object = Kind<OTX_SAG_FLAT, OTX_MAT_VACUUM, OTX_APER_NONE, OTX_RULE_NONE>;
using Stop = Kind<OTX_SAG_FLAT, OTX_MAT_VACUUM, OTX_APER_CIRCULAR, OTX_RULE_NONE>;
using ConicMirror = Kind<OTX_SAG_CONIC, OTX_MAT_MIRROR, OTX_APER_CIRCULAR, OTX_RULE_NONE>;
using FlatMirror = Kind<OTX_SAG_FLAT, OTX_MAT_MIRROR, OTX_APER_CIRCULAR, OTX_RULE_NONE>;
using ConicCoated = Kind<OTX_SAG_CONIC, OTX_MAT_FRESNEL_MIRROR, OTX_APER_CIRCULAR, OTX_RULE_NONE>;
using FlatCoated = Kind<OTX_SAG_FLAT, OTX_MAT_FRESNEL_MIRROR, OTX_APER_CIRCULAR, OTX_RULE_NONE>;
using Detector = Kind<OTX_SAG_FLAT, OTX_MAT_VACUUM, OTX_APER_RECTANGULAR, OTX_RULE_NONE>;

template <class... Ks>
bool try_pair(int grid, int block, const otx_system& sys, const TraceArgs& a, cudaStream_t st) {
  if (!shape_matches<Ks...>(sys)) return false;
  k_trace_pair<Ks...><<<(grid + 1) / 2, block, 0, st>>>(sys, a);
  return true;
}

// Grid input with the object at infinity, final rays only.  rays_per_thread
// 2 runs the packed two-rays-per-thread kernels (trace_pair.cuh); 0 (unset)
// and 1 the one-ray kernels, which measured faster.
bool launch_fixed(int mode, bool acc, int rpt, int grid, int block, const otx_system& sys,
                  const TraceArgs& a, cudaStream_t st) {
  if (acc) return false;
  if (mode == OTX_MODE_CELLS_INFINITY && rpt != 2) {
    // the forward model's cells, their rays generated in the kernel
    constexpr int C = OTX_MODE_CELLS_INFINITY;
    if (try_fixed<C, Object, Stop, ConicMirror, FlatMirror, Detector>(grid, block, sys, a, st))
      return true;
    if (try_fixed<C, Object, Stop, ConicCoated, FlatCoated, Detector>(grid, block, sys, a, st))
      return true;
    return false;
  }
  if (mode != OTX_INPUT_GRID_INFINITY) return false;
  if (rpt == 2) {
    if (try_pair<Object, Stop, ConicMirror, FlatMirror, Detector>(grid, block, sys, a, st))
      return true;
    if (try_pair<Object, Stop, ConicCoated, FlatCoated, Detector>(grid, block, sys, a, st))
      return true;
  }
  if (rpt == 2) return false;
  constexpr int M = OTX_INPUT_GRID_INFINITY;
  // Newtonian telescope: object, obscuration, primary, fold, sensor
  if (try_fixed<M, Object, Stop, ConicMirror, FlatMirror, Detector>(grid, block, sys, a, st))
    return true;
  if (try_fixed<M, Object, Stop, ConicCoated, FlatCoated, Detector>(grid, block, sys, a, st))
    return true;
  return false;
}

}  // namespace otx
