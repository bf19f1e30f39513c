// Instantiates the traversal kernel for ORIGIN_TABLE rays (see trace.cuh).
#include "trace.cuh"
#include "launch.h"

namespace rmg {

cudaError_t launch_trace_table(const TraceParams& P, int stack_depth, unsigned grid, unsigned block,
                               cudaStream_t st) {
  switch (stack_depth) {
    case 0: k_trace<ORIGIN_TABLE, 0><<<grid, block, 0, st>>>(P); break;
    case 4: k_trace<ORIGIN_TABLE, 4><<<grid, block, 0, st>>>(P); break;
    case 8: k_trace<ORIGIN_TABLE, 8><<<grid, block, 0, st>>>(P); break;
    case 16: k_trace<ORIGIN_TABLE, 16><<<grid, block, 0, st>>>(P); break;
    case 32: k_trace<ORIGIN_TABLE, 32><<<grid, block, 0, st>>>(P); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

}  // namespace rmg
