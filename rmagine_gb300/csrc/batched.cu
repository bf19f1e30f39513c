// Batched simulation of many heterogeneous sensors in ONE persistent kernel,
// replayed from a CUDA graph, with an autotuner for its launch options.
//
// No counterpart in the reference: rmagine simulates one sensor per call
// (SphereSimulatorOptix.cpp:64-81 launches one optixLaunch per simulate), and a
// user with many sensors runs many simulators.  Here a plan (rmg_batch) holds a
// device table of jobs -- one per (sensor, Tsb, Tbm, n_poses, outputs) -- and
// the concatenated index space of all their ray tiles.  Persistent warps take
// `grab` tiles at a time from a global counter, find the job by binary search
// over the tiles' prefix sums, and run exactly the per-ray code of rmg_simulate
// (same ray setup, traversal and epilogue), so every output is bit-identical to
// one plain rmg_simulate per job.  The counter is reset by a memset node at the
// start of the captured graph.
#include <algorithm>
#include <chrono>
#include <cstring>
#include <new>
#include <vector>

#include "internal.h"
#include "launch.h"
#include "trace.cuh"

namespace rmg {

struct JobDev {
  SensorDev sen;
  Tf Tsb;
  const rmg_transform* Tbm;
  uint32_t n_poses;
  rmg_outputs out;
  uint32_t tile_w_log2, tile_h, tiles_x, tiles_per_pose;
  uint64_t tile_begin;
};

namespace {

constexpr int kMaxJobsShared = 512;

struct BatchParams {
  DeviceMap map;
  const JobDev* jobs;
  uint32_t n_jobs;
  uint64_t total_tiles;
  unsigned long long* counter;
  uint32_t grab;
  unsigned budget;
  int trail_bits;
  int full_stack;
};

template <int OK, int SS, int TB>
__device__ __forceinline__ void batched_ray(const BatchParams& B, const JobDev& J, uint64_t tile_in_job,
                                            uint32_t lane) {
  const uint32_t pose = (uint32_t)(tile_in_job / J.tiles_per_pose);
  const uint32_t r = (uint32_t)(tile_in_job - (uint64_t)pose * J.tiles_per_pose);
  const uint32_t ty = r / J.tiles_x, tx = r - ty * J.tiles_x;
  const uint32_t tile_w = 1u << J.tile_w_log2;
  const uint32_t vid = ty * J.tile_h + (lane >> J.tile_w_log2);
  const uint32_t hid = tx * tile_w + (lane & (tile_w - 1));
  const uint32_t W = J.sen.width, H = J.sen.height;
  if (vid >= H || hid >= W) return;
  const uint32_t loc = visit_loc(J.sen, vid * W + hid);
  const uint64_t gid = (uint64_t)pose * W * H + loc;
  const Tf Tsm = tmul(load_tf(J.Tbm[pose]), J.Tsb);
  V dir_s, orig_s, o, d;
  setup_ray<OK>(J.sen, Tsm, loc, dir_s, orig_s, o, d);
  Hit h;
  bool over = false;
  trace_ray<SS, TB>(B.map, o, d, J.sen.range_max, B.budget, h, over);
  if (over) atomicExch(B.map.status, (unsigned)RMG_ERR_TRAVERSAL_BUDGET);
  TraceParams P;  // the epilogue reads only map, sensor range and outputs
  P.map = B.map;
  P.sen = J.sen;
  P.out = J.out;
  write_attributes<OK>(P, gid, h, dir_s, orig_s, Tsm);
}

#ifndef RMG_BATCHED_MIN_BLOCKS
#define RMG_BATCHED_MIN_BLOCKS 5
#endif

template <int SS, int TB>
__global__ void __launch_bounds__(256, RMG_BATCHED_MIN_BLOCKS) k_trace_batched(const BatchParams B) {
  __shared__ unsigned long long s_begin[kMaxJobsShared + 1];
  const bool in_smem = B.n_jobs <= kMaxJobsShared;
  if (in_smem) {
    for (uint32_t j = threadIdx.x; j < B.n_jobs; j += blockDim.x) s_begin[j] = B.jobs[j].tile_begin;
    if (threadIdx.x == 0) s_begin[B.n_jobs] = B.total_tiles;
  }
  __syncthreads();
  const uint32_t lane = threadIdx.x & 31;
  for (;;) {
    unsigned long long base = 0;
    if (lane == 0) base = atomicAdd(B.counter, (unsigned long long)B.grab);
    base = __shfl_sync(0xffffffffu, base, 0);
    if (base >= B.total_tiles) break;
    for (uint32_t k = 0; k < B.grab; ++k) {
      const uint64_t tile = base + k;
      if (tile >= B.total_tiles) break;
      // job = last j with begin[j] <= tile
      uint32_t lo = 0, hi = B.n_jobs;
      while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        const unsigned long long b = in_smem ? s_begin[mid] : B.jobs[mid].tile_begin;
        if (b <= tile) lo = mid; else hi = mid;
      }
      const JobDev& J = B.jobs[lo];
      const uint64_t t = tile - J.tile_begin;
      switch (J.sen.kind) {
        case RMG_MODEL_SPHERICAL:
        case RMG_MODEL_PINHOLE: batched_ray<ORIGIN_POSE, SS, TB>(B, J, t, lane); break;
        case RMG_MODEL_O1DN: batched_ray<ORIGIN_SINGLE, SS, TB>(B, J, t, lane); break;
        default: batched_ray<ORIGIN_TABLE, SS, TB>(B, J, t, lane); break;
      }
    }
  }
}

template <int SS>
cudaError_t launch_batched_tb(const BatchParams& B, unsigned grid, unsigned block, cudaStream_t st) {
  if (SS > 0 && B.full_stack) {
    k_trace_batched<kFullStack, 0><<<grid, block, 0, st>>>(B);
    return cudaGetLastError();
  }
  switch (B.trail_bits) {
    case 32: k_trace_batched<SS, 32><<<grid, block, 0, st>>>(B); break;
    case 64: k_trace_batched<SS, 64><<<grid, block, 0, st>>>(B); break;
    default: k_trace_batched<SS, 128><<<grid, block, 0, st>>>(B); break;
  }
  return cudaGetLastError();
}

cudaError_t launch_batched(const BatchParams& B, int ss, unsigned grid, unsigned block, cudaStream_t st) {
  switch (ss) {
    case 0: return launch_batched_tb<0>(B, grid, block, st);
    case 8: return launch_batched_tb<8>(B, grid, block, st);
    case 16: return launch_batched_tb<16>(B, grid, block, st);
    default: return cudaErrorInvalidValue;
  }
}

template <int SS>
const void* batched_fn(int tb) {
  if (tb == 0) return reinterpret_cast<const void*>(k_trace_batched<kFullStack, 0>);
  return tb == 32 ? reinterpret_cast<const void*>(k_trace_batched<SS, 32>)
                  : tb == 64 ? reinterpret_cast<const void*>(k_trace_batched<SS, 64>)
                             : reinterpret_cast<const void*>(k_trace_batched<SS, 128>);
}

const void* kernel_ptr(int ss, int tb) {
  switch (ss) {
    case 0: return batched_fn<0>(tb);
    case 8: return batched_fn<8>(tb);
    default: return batched_fn<16>(tb);
  }
}

bool batch_stack_ok(uint32_t s) { return s == 0 || s == 8 || s == 16; }

}  // namespace
}  // namespace rmg

struct rmg_batch {
  int device;
  const rmg_map* map;
  std::vector<rmg_batch_entry> entries;
  std::vector<rmg::JobDev> jobs_h;
  rmg::JobDev* jobs = nullptr;
  unsigned long long* counter = nullptr;
  uint64_t total_tiles = 0;
  uint64_t total_rays = 0;
  rmg_batch_config cfg;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  cudaStream_t capture_stream = nullptr;
};

namespace rmg {

void fit_tile(uint32_t W, uint32_t H, uint32_t& tw, uint32_t& th);

namespace {

void drop_graph(rmg_batch* b) {
  if (b->exec) cudaGraphExecDestroy(b->exec);
  if (b->graph) cudaGraphDestroy(b->graph);
  b->exec = nullptr;
  b->graph = nullptr;
}

int check_batch_config(const rmg_batch_config& c) {
  if (!batch_stack_ok(c.stack_depth)) return fail(RMG_ERR_UNSUPPORTED, "batch config: stack_depth must be 0, 8 or 16");
  if (c.block_warps < 1 || c.block_warps > 8) return fail(RMG_ERR_UNSUPPORTED, "batch config: block_warps 1..8");
  if (c.tile_w == 0 || (c.tile_w & (c.tile_w - 1)) || c.tile_w > 32 || c.tile_w * c.tile_h != 32)
    return fail(RMG_ERR_UNSUPPORTED, "batch config: tile_w power of two, tile_w*tile_h == 32");
  if (c.grab < 1 || c.grab > 64) return fail(RMG_ERR_UNSUPPORTED, "batch config: grab 1..64");
  return RMG_OK;
}

// (Re)builds the device job table for the plan's tile shape.
int build_jobs(rmg_batch* b) {
  b->jobs_h.clear();
  uint64_t begin = 0, rays = 0;
  for (const rmg_batch_entry& e : b->entries) {
    JobDev J;
    std::memset(&J, 0, sizeof(J));
    J.sen = device_view(e.sensor);
    J.Tsb = Tf{Q{e.Tsb.R.x, e.Tsb.R.y, e.Tsb.R.z, e.Tsb.R.w}, V{e.Tsb.t.x, e.Tsb.t.y, e.Tsb.t.z}};
    J.Tbm = e.Tbm;
    J.n_poses = e.n_poses;
    J.out = e.out;
    uint32_t tw = b->cfg.tile_w, th = b->cfg.tile_h;
    fit_tile(e.sensor->width, e.sensor->height, tw, th);
    uint32_t l = 0;
    while ((1u << l) < tw) ++l;
    J.tile_w_log2 = l;
    J.tile_h = th;
    J.tiles_x = (e.sensor->width + tw - 1) / tw;
    J.tiles_per_pose = J.tiles_x * ((e.sensor->height + th - 1) / th);
    J.tile_begin = begin;
    begin += (uint64_t)J.tiles_per_pose * e.n_poses;
    rays += (uint64_t)e.sensor->width * e.sensor->height * e.n_poses;
    b->jobs_h.push_back(J);
  }
  b->total_tiles = begin;
  b->total_rays = rays;
  if (!b->jobs) {
    int s = dev_alloc(&b->jobs, std::max<size_t>(1, b->jobs_h.size()), "batch jobs");
    if (s != RMG_OK) return s;
  }
  RMG_CUDA_TRY(cudaMemcpy(b->jobs, b->jobs_h.data(), sizeof(JobDev) * b->jobs_h.size(), cudaMemcpyHostToDevice));
  return RMG_OK;
}

int persistent_grid(const rmg_batch_config& c, int trail_bits, unsigned& grid) {
  int per_sm = 0;
  RMG_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel_ptr((int)c.stack_depth, trail_bits),
                                                             32 * (int)c.block_warps, 0));
  per_sm = std::max(per_sm, 1);
  if (c.ctas_per_sm > 0) per_sm = std::min<int>(per_sm, (int)c.ctas_per_sm);
  grid = (unsigned)(per_sm * device_sm_count());
  return RMG_OK;
}

BatchParams params(const rmg_batch* b) {
  BatchParams B;
  B.map = device_view(b->map);
  B.jobs = b->jobs;
  B.n_jobs = (uint32_t)b->jobs_h.size();
  B.total_tiles = b->total_tiles;
  B.counter = b->counter;
  B.grab = b->cfg.grab;
  B.budget = 2u * b->map->n_nodes + 64u;
  B.trail_bits = trail_bits_for_depth(b->map->depth);
  B.full_stack = b->map->depth <= (unsigned)kFullStack ? 1 : 0;
  return B;
}

// One launch on `st` without a graph: counter reset + persistent kernel.
int launch_direct(rmg_batch* b, cudaStream_t st) {
  if (b->total_tiles == 0) return RMG_OK;
  unsigned grid = 0;
  const bool full = b->cfg.stack_depth > 0 && b->map->depth <= (unsigned)kFullStack;
  int s = persistent_grid(b->cfg, full ? 0 : trail_bits_for_depth(b->map->depth), grid);
  if (s != RMG_OK) return s;
  RMG_CUDA_TRY(cudaMemsetAsync(b->counter, 0, sizeof(unsigned long long), st));
  return cuda_status(launch_batched(params(b), (int)b->cfg.stack_depth, grid, 32u * b->cfg.block_warps, st),
                     "k_trace_batched");
}

int capture(rmg_batch* b) {
  drop_graph(b);
  if (!b->capture_stream) RMG_CUDA_TRY(cudaStreamCreateWithFlags(&b->capture_stream, cudaStreamNonBlocking));
  RMG_CUDA_TRY(cudaStreamBeginCapture(b->capture_stream, cudaStreamCaptureModeThreadLocal));
  const int s = launch_direct(b, b->capture_stream);
  cudaGraph_t g = nullptr;
  const cudaError_t e = cudaStreamEndCapture(b->capture_stream, &g);
  if (s != RMG_OK) { if (g) cudaGraphDestroy(g); return s; }
  RMG_CUDA_TRY(e);
  b->graph = g;
  RMG_CUDA_TRY(cudaGraphInstantiate(&b->exec, g, 0));
  return RMG_OK;
}

}  // namespace
}  // namespace rmg

using namespace rmg;

extern "C" int rmg_batch_default_config(rmg_batch_config* cfg) {
  return guarded("rmg_batch_default_config", [&]() -> int {
    if (!cfg) return fail(RMG_ERR_INVALID_ARG, "rmg_batch_default_config: NULL");
    cfg->stack_depth = 8;
    cfg->block_warps = 4;
    cfg->tile_w = 8;
    cfg->tile_h = 4;
    cfg->grab = 2;
    cfg->ctas_per_sm = 0;
    cfg->use_graph = 1;
    return RMG_OK;
  });
}

extern "C" int rmg_batch_create(const rmg_map* map, const rmg_batch_entry* entries, uint32_t n_entries,
                                rmg_batch** out) {
  return guarded("rmg_batch_create", [&]() -> int {
    if (!map || !out || (n_entries && !entries)) return fail(RMG_ERR_INVALID_ARG, "rmg_batch_create: NULL argument");
    *out = nullptr;
    for (uint32_t i = 0; i < n_entries; ++i) {
      const rmg_batch_entry& e = entries[i];
      if (!e.sensor) return fail(RMG_ERR_INVALID_ARG, "rmg_batch_create: entry without sensor");
      if (e.n_poses && !e.Tbm) return fail(RMG_ERR_INVALID_ARG, "rmg_batch_create: entry without poses");
    }
    rmg_batch* b = new (std::nothrow) rmg_batch;
    if (!b) return fail(RMG_ERR_OOM, "rmg_batch_create: host allocation");
    cudaGetDevice(&b->device);
    b->map = map;
    b->entries.assign(entries, entries + n_entries);
    rmg_batch_default_config(&b->cfg);
    int s = dev_alloc(&b->counter, 1, "batch counter");
    if (s == RMG_OK) s = build_jobs(b);
    if (s != RMG_OK) { cudaFree(b->jobs); cudaFree(b->counter); delete b; return s; }
    *out = b;
    return RMG_OK;
  });
}

extern "C" int rmg_batch_set_config(rmg_batch* b, const rmg_batch_config* cfg) {
  return guarded("rmg_batch_set_config", [&]() -> int {
    if (!b || !cfg) return fail(RMG_ERR_INVALID_ARG, "rmg_batch_set_config: NULL argument");
    int s = check_batch_config(*cfg);
    if (s != RMG_OK) return s;
    b->cfg = *cfg;
    drop_graph(b);
    return build_jobs(b);
  });
}

extern "C" int rmg_batch_get_config(const rmg_batch* b, rmg_batch_config* cfg) {
  return guarded("rmg_batch_get_config", [&]() -> int {
    if (!b || !cfg) return fail(RMG_ERR_INVALID_ARG, "rmg_batch_get_config: NULL argument");
    *cfg = b->cfg;
    return RMG_OK;
  });
}

extern "C" int rmg_batch_info(const rmg_batch* b, uint64_t* total_rays, uint64_t* total_tiles) {
  return guarded("rmg_batch_info", [&]() -> int {
    if (!b) return fail(RMG_ERR_INVALID_ARG, "rmg_batch_info: NULL batch");
    if (total_rays) *total_rays = b->total_rays;
    if (total_tiles) *total_tiles = b->total_tiles;
    return RMG_OK;
  });
}

extern "C" int rmg_batch_launch(rmg_batch* b, void* stream) {
  return guarded("rmg_batch_launch", [&]() -> int {
    if (!b) return fail(RMG_ERR_INVALID_ARG, "rmg_batch_launch: NULL batch");
    cudaStream_t st = as_stream(stream);
    if (!b->cfg.use_graph) return launch_direct(b, st);
    if (!b->exec) {
      const int s = capture(b);
      if (s != RMG_OK) return s;
    }
    if (b->total_tiles == 0) return RMG_OK;
    RMG_CUDA_TRY(cudaGraphLaunch(b->exec, st));
    return RMG_OK;
  });
}

// Times candidate launch options on the plan itself (direct launches, CUDA
// events, median of `reps` after one warm-up) and keeps the fastest; the
// graph is re-captured for it.  Candidates: stack depth {0, 8, 16} x warps
// per CTA {2, 4, 8} x tile {8x4, 4x8, 16x2} x grab {1, 4}, searched one
// coordinate at a time from the default.
extern "C" int rmg_batch_autotune(rmg_batch* b, void* stream, uint32_t reps, rmg_batch_config* best_out) {
  return guarded("rmg_batch_autotune", [&]() -> int {
    if (!b) return fail(RMG_ERR_INVALID_ARG, "rmg_batch_autotune: NULL batch");
    cudaStream_t st = as_stream(stream);
    reps = std::max<uint32_t>(reps, 1);
    cudaEvent_t e0, e1;
    RMG_CUDA_TRY(cudaEventCreate(&e0));
    RMG_CUDA_TRY(cudaEventCreate(&e1));
    auto time_cfg = [&](const rmg_batch_config& c, float& ms) -> int {
      b->cfg = c;
      int s = build_jobs(b);
      if (s != RMG_OK) return s;
      s = launch_direct(b, st);  // warm-up
      if (s != RMG_OK) return s;
      std::vector<float> t;
      for (uint32_t r = 0; r < reps; ++r) {
        RMG_CUDA_TRY(cudaEventRecord(e0, st));
        s = launch_direct(b, st);
        if (s != RMG_OK) return s;
        RMG_CUDA_TRY(cudaEventRecord(e1, st));
        RMG_CUDA_TRY(cudaEventSynchronize(e1));
        float x = 0;
        RMG_CUDA_TRY(cudaEventElapsedTime(&x, e0, e1));
        t.push_back(x);
      }
      std::sort(t.begin(), t.end());
      ms = t[t.size() / 2];
      return RMG_OK;
    };
    rmg_batch_config best = b->cfg;
    best.use_graph = b->cfg.use_graph;
    float best_ms = 0;
    int s = time_cfg(best, best_ms);
    const uint32_t stacks[] = {0, 8, 16};
    const uint32_t warps[] = {2, 4, 8};
    const uint32_t tiles[][2] = {{8, 4}, {4, 8}, {16, 2}};
    const uint32_t grabs[] = {1, 4};
    for (int coord = 0; coord < 4 && s == RMG_OK; ++coord) {
      const int n = coord == 0 ? 3 : coord == 1 ? 3 : coord == 2 ? 3 : 2;
      rmg_batch_config round_best = best;
      for (int i = 0; i < n && s == RMG_OK; ++i) {
        rmg_batch_config c = best;
        if (coord == 0) c.stack_depth = stacks[i];
        if (coord == 1) c.block_warps = warps[i];
        if (coord == 2) { c.tile_w = tiles[i][0]; c.tile_h = tiles[i][1]; }
        if (coord == 3) c.grab = grabs[i];
        if (std::memcmp(&c, &best, sizeof(c)) == 0) continue;
        float ms = 0;
        s = time_cfg(c, ms);
        if (s == RMG_OK && ms < best_ms) { best_ms = ms; round_best = c; }
      }
      best = round_best;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    b->cfg = best;
    drop_graph(b);
    int s2 = build_jobs(b);
    if (s == RMG_OK) s = s2;
    if (s == RMG_OK && best_out) *best_out = best;
    return s;
  });
}

extern "C" int rmg_batch_destroy(rmg_batch* b) {
  return guarded("rmg_batch_destroy", [&]() -> int {
    if (!b) return RMG_OK;
    drop_graph(b);
    if (b->capture_stream) cudaStreamDestroy(b->capture_stream);
    cudaFree(b->jobs);
    cudaFree(b->counter);
    delete b;
    return RMG_OK;
  });
}
