// Traversal launchers for ORIGIN_POSE: rays from the sensor origin at the pose (spherical, pinhole).
#include "trace_launch.cuh"

namespace rmg {

template cudaError_t launch_trace<ORIGIN_POSE>(const TraceParams&, int, unsigned, unsigned, cudaStream_t);
template cudaError_t launch_trace_refill<ORIGIN_POSE>(const TraceParams&, int, unsigned, unsigned long long*, uint32_t,
                                           uint32_t, cudaStream_t);

}  // namespace rmg
