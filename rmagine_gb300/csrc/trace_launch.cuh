// Launchers of the traversal kernels for one origin kind (see trace.cuh): the
// walk is picked from the launch configuration and the tree (wide, packet,
// full stack, trail width and short-stack size).  Each trace_<kind>.cu unit
// instantiates them for one OriginKind, so the three compile in parallel.
#pragma once

#include <algorithm>

#include "internal.h"
#include "launch.h"
#include "trace.cuh"

namespace rmg {
namespace trace_detail {

template <int OK, int SS>
cudaError_t by_trail(const TraceParams& P, unsigned grid, unsigned block, cudaStream_t st) {
  if (P.wide8) {  // the 8-wide quantized tree: same results
    k_trace<OK, 0, kWide8TB><<<grid, block, 0, st>>>(P);
    return cudaGetLastError();
  }
  if (P.wide) {  // the 4-wide tree: same results, fewer and wider visits
    k_trace<OK, 0, kWideTB><<<grid, block, 0, st>>>(P);
    return cudaGetLastError();
  }
  if (P.packet) {  // the warp walks together: same results
    k_trace<OK, 0, kPacketTB><<<grid, block, 0, st>>>(P);
    return cudaGetLastError();
  }
  if (SS > 0 && P.full_stack) {  // same visits and results, without trail bookkeeping
    k_trace<OK, kFullStack, 0><<<grid, block, 0, st>>>(P);
    return cudaGetLastError();
  }
  switch (P.trail_bits) {
    case 32: k_trace<OK, SS, 32><<<grid, block, 0, st>>>(P); break;
    case 64: k_trace<OK, SS, 64><<<grid, block, 0, st>>>(P); break;
    default: k_trace<OK, SS, 128><<<grid, block, 0, st>>>(P); break;
  }
  return cudaGetLastError();
}

template <int OK, int SS, int TB>
cudaError_t refill_one(const TraceParams& P, unsigned block, unsigned long long* counter, uint32_t chunk,
                       uint32_t refill, cudaStream_t st) {
  int per_sm = 0;
  cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_trace_refill<OK, SS, TB>,
                                                                (int)block, 0);
  if (e != cudaSuccess) return e;
  const unsigned grid = (unsigned)(std::max(per_sm, 1) * device_sm_count());
  k_trace_refill<OK, SS, TB><<<grid, block, 0, st>>>(P, counter, chunk, refill);
  return cudaGetLastError();
}

template <int OK, int SS>
cudaError_t refill_by_trail(const TraceParams& P, unsigned block, unsigned long long* counter, uint32_t chunk,
                            uint32_t refill, cudaStream_t st) {
  switch (P.trail_bits) {
    case 32: return refill_one<OK, SS, 32>(P, block, counter, chunk, refill, st);
    case 64: return refill_one<OK, SS, 64>(P, block, counter, chunk, refill, st);
    default: return refill_one<OK, SS, 128>(P, block, counter, chunk, refill, st);
  }
}

}  // namespace trace_detail

template <int OK>
cudaError_t launch_trace(const TraceParams& P, int stack_depth, unsigned grid, unsigned block, cudaStream_t st) {
  using namespace trace_detail;
  switch (stack_depth) {
    case 0: return by_trail<OK, 0>(P, grid, block, st);
    case 8: return by_trail<OK, 8>(P, grid, block, st);
    case 16: return by_trail<OK, 16>(P, grid, block, st);
    default: return cudaErrorInvalidValue;
  }
}

template <int OK>
cudaError_t launch_trace_refill(const TraceParams& P, int stack_depth, unsigned block, unsigned long long* counter,
                                uint32_t chunk, uint32_t refill, cudaStream_t st) {
  using namespace trace_detail;
  switch (stack_depth) {
    case 8: return refill_by_trail<OK, 8>(P, block, counter, chunk, refill, st);
    case 16: return refill_by_trail<OK, 16>(P, block, counter, chunk, refill, st);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace rmg
