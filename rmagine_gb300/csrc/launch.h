// Kernel launchers shared between translation units.
#pragma once

#include <cuda_runtime.h>

#include "common.cuh"

namespace rmg {

struct TraceParams;

// Traversal launchers for one OriginKind (trace_launch.cuh; instantiated in
// trace_pose.cu, trace_single.cu and trace_table.cu).
template <int OK>
cudaError_t launch_trace(const TraceParams& P, int stack_depth, unsigned grid, unsigned block, cudaStream_t st);
template <int OK>
cudaError_t launch_trace_refill(const TraceParams& P, int stack_depth, unsigned block, unsigned long long* counter,
                                uint32_t chunk, uint32_t refill, cudaStream_t st);

inline bool valid_stack_depth(uint32_t s) { return s == 0 || s == 8 || s == 16; }

}  // namespace rmg
