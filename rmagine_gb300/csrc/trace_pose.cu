// Instantiates the traversal kernel for ORIGIN_POSE rays (see trace.cuh).
#include "trace.cuh"
#include "launch.h"

namespace rmg {

namespace {
template <int SS>
cudaError_t by_trail(const TraceParams& P, unsigned grid, unsigned block, cudaStream_t st) {
  switch (P.trail_bits) {
    case 32: k_trace<ORIGIN_POSE, SS, 32><<<grid, block, 0, st>>>(P); break;
    case 64: k_trace<ORIGIN_POSE, SS, 64><<<grid, block, 0, st>>>(P); break;
    default: k_trace<ORIGIN_POSE, SS, 128><<<grid, block, 0, st>>>(P); break;
  }
  return cudaGetLastError();
}
}  // namespace

cudaError_t launch_trace_pose(const TraceParams& P, int stack_depth, unsigned grid, unsigned block,
                               cudaStream_t st) {
  switch (stack_depth) {
    case 0: return by_trail<0>(P, grid, block, st);
    case 8: return by_trail<8>(P, grid, block, st);
    case 16: return by_trail<16>(P, grid, block, st);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace rmg
