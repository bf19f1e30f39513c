// Traversal launchers for ORIGIN_TABLE: rays from a per-ray origin table (OnDn).
#include "trace_launch.cuh"

namespace rmg {

template cudaError_t launch_trace<ORIGIN_TABLE>(const TraceParams&, int, unsigned, unsigned, cudaStream_t);
template cudaError_t launch_trace_refill<ORIGIN_TABLE>(const TraceParams&, int, unsigned, unsigned long long*, uint32_t,
                                           uint32_t, cudaStream_t);

}  // namespace rmg
