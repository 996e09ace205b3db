// Instantiation of the fused trace kernel for the cell input modes (rays of
// scene cells generated in the kernel, otx_trace_cells).
#include "trace_kernel.cuh"

namespace otx {
template void launch_mode<OTX_MODE_CELLS_INFINITY>(int, bool, bool, int, int, const otx_system&,
                                                   const TraceArgs&, cudaStream_t);
template void launch_mode<OTX_MODE_CELLS_FINITE>(int, bool, bool, int, int, const otx_system&,
                                                 const TraceArgs&, cudaStream_t);
}  // namespace otx
