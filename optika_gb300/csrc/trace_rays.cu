// Instantiation of the fused trace kernel for input mode OTX_INPUT_RAYS.
#include "trace_kernel.cuh"

namespace otx {
template void launch_mode<OTX_INPUT_RAYS>(int, bool, bool, int, int, const otx_system&, const TraceArgs&,
                                  cudaStream_t);
}  // namespace otx
