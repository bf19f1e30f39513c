// Traversal launchers for ORIGIN_SINGLE: rays from one sensor-frame origin (O1Dn).
#include "trace_launch.cuh"

namespace rmg {

template cudaError_t launch_trace<ORIGIN_SINGLE>(const TraceParams&, int, unsigned, unsigned, cudaStream_t);
template cudaError_t launch_trace_refill<ORIGIN_SINGLE>(const TraceParams&, int, unsigned, unsigned long long*, uint32_t,
                                           uint32_t, cudaStream_t);

}  // namespace rmg
