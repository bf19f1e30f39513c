// rmg_simulate: the C entry point of the plain (one sensor, many poses) path.
#include <algorithm>
#include <string>
#include <vector>

#include "internal.h"
#include "launch.h"
#include "trace.cuh"

// Walk the 4-wide tree when the launch config leaves the choice open.  Off:
// on the 1M-triangle terrain the binary walk is faster (spherical 6,296 vs
// 5,736 Mrays/s, pinhole 9,200 vs 8,035); the 4-wide walk wins on small maps
// (2,412-triangle room: 3,563 vs 3,281) and is chosen there with bvh_width = 4.
#ifndef RMG_DEFAULT_WIDE
#define RMG_DEFAULT_WIDE 0
#endif

// 8-wide quantized walk when the launch config leaves the width open.
#ifndef RMG_DEFAULT_WIDE8
#define RMG_DEFAULT_WIDE8 0
#endif

// Warp-synchronous packet walk when the launch config leaves the choice open.
#ifndef RMG_DEFAULT_PACKET
#define RMG_DEFAULT_PACKET 0
#endif

namespace rmg {

// Defaults from a sweep on the 1M-triangle terrain (spherical 128x1024): short
// stack 16, 4 warps per CTA, 8 x 4 ray tiles, one tile per warp.
int default_config(const rmg_sensor* s, rmg_launch_config* cfg) {
  cfg->stack_depth = 16;
  cfg->block_warps = 4;
  cfg->refill = 0;
  cfg->chunk = 4;
  cfg->bvh_width = 0;
  cfg->packet = 2;
  if (s && s->width >= 8 && s->height >= 4) { cfg->tile_w = 8; cfg->tile_h = 4; }
  else if (s && s->height < 4 && s->height > 1) { cfg->tile_w = 16; cfg->tile_h = 2; }
  else { cfg->tile_w = 32; cfg->tile_h = 1; }
  return RMG_OK;
}

int check_config(const rmg_launch_config& c) {
  if (!valid_stack_depth(c.stack_depth))
    return fail(RMG_ERR_UNSUPPORTED, "launch config: stack_depth must be 0, 8 or 16");
  if (c.block_warps < 1 || c.block_warps > 8)
    return fail(RMG_ERR_UNSUPPORTED, "launch config: block_warps must be 1..8");
  if (c.tile_w == 0 || (c.tile_w & (c.tile_w - 1)) != 0 || c.tile_w > 32 || c.tile_w * c.tile_h != 32)
    return fail(RMG_ERR_UNSUPPORTED, "launch config: tile_w must be a power of two with tile_w*tile_h == 32");
  if (c.refill > 32) return fail(RMG_ERR_UNSUPPORTED, "launch config: refill must be 0..32");
  if (c.refill && c.stack_depth == 0)
    return fail(RMG_ERR_UNSUPPORTED, "launch config: refill mode needs stack_depth 8 or 16");
  if (c.refill && (c.chunk < 1 || c.chunk > 1024)) return fail(RMG_ERR_UNSUPPORTED, "launch config: chunk 1..1024");
  if (c.bvh_width != 0 && c.bvh_width != 2 && c.bvh_width != 4 && c.bvh_width != 8)
    return fail(RMG_ERR_UNSUPPORTED, "launch config: bvh_width must be 0, 2, 4 or 8");
  if (c.packet > 2) return fail(RMG_ERR_UNSUPPORTED, "launch config: packet must be 0, 1 or 2");
  return RMG_OK;
}

int log2u(uint32_t v) {
  int l = 0;
  while ((1u << l) < v) ++l;
  return l;
}

// Tile shape for a sensor: a configured tile taller (wider) than the sensor is
// halved in height (width) and doubled in the other direction while the
// smaller size still covers the sensor, so a 1-row O1Dn table walks 32 x 1
// tiles instead of leaving three rows of an 8 x 4 tile idle.  Results do not
// depend on the tile shape.
void fit_tile(uint32_t W, uint32_t H, uint32_t& tw, uint32_t& th) {
  while (th > 1 && th / 2 >= H) { th /= 2; tw *= 2; }
  while (tw > 1 && tw / 2 >= W) { tw /= 2; th *= 2; }
}

// Fills the parameter block of one sensor's launch; returns the tile count.
int make_trace_params(const rmg_map* map, const rmg_sensor* sensor, const rmg_transform* Tsb,
                      const rmg_transform* Tbm, uint32_t n_poses, const rmg_outputs* out,
                      const rmg_launch_config& cfg, TraceParams& P) {
  P.map = device_view(map);
  P.sen = device_view(sensor);
  const rmg_transform Tsb_ = *Tsb;
  P.Tsb = Tf{Q{Tsb_.R.x, Tsb_.R.y, Tsb_.R.z, Tsb_.R.w}, V{Tsb_.t.x, Tsb_.t.y, Tsb_.t.z}};
  P.Tbm = Tbm;
  P.n_poses = n_poses;
  P.out = *out;
  uint32_t tw = cfg.tile_w, th = cfg.tile_h;
  fit_tile(sensor->width, sensor->height, tw, th);
  P.tile_w_log2 = (uint32_t)log2u(tw);
  P.tile_h = th;
  P.tiles_x = (sensor->width + tw - 1) / tw;
  const uint32_t tiles_y = (sensor->height + th - 1) / th;
  P.tiles_per_pose = P.tiles_x * tiles_y;
  P.n_tiles = (uint64_t)P.tiles_per_pose * n_poses;
  P.budget = 2u * map->n_nodes + 64u;
  P.trail_bits = trail_bits_for_depth(map->depth);
  P.full_stack = map->depth <= (unsigned)kFullStack ? 1 : 0;
  // 4-wide walk: 3 pushes per level at most, so 21 levels fit its 64-entry stack
  P.wide = (cfg.bvh_width != 2 && cfg.refill == 0 && map->d_nodes4 && 3 * map->depth4 <= (unsigned)kStack4 &&
            RMG_DEFAULT_WIDE) ? 1 : 0;
  if (cfg.bvh_width == 4 && cfg.refill == 0 && map->d_nodes4 && 3 * map->depth4 <= (unsigned)kStack4) P.wide = 1;
  // 8-wide quantized walk: a pending-children stack of kStack8 entries holds trees of kStack8 + 1 levels
  const bool have8 = map->d_nodes8 && map->depth8 <= (unsigned)kStack8 + 1u;
  P.wide8 = (have8 && cfg.refill == 0 && (cfg.bvh_width == 8 || (cfg.bvh_width == 0 && RMG_DEFAULT_WIDE8))) ? 1 : 0;
  if (P.wide8) {
    P.wide = 0;
    P.map.tris = map->d_tris8;  // h.tri of this walk indexes the 8-wide triangle copy
  }
  // warp-synchronous packet walk: binary tree, full stack
  const bool want_packet = cfg.packet == 1 || (cfg.packet == 2 && RMG_DEFAULT_PACKET);
  P.packet = (want_packet && !P.wide && !P.wide8 && cfg.refill == 0 && P.full_stack) ? 1 : 0;
  return RMG_OK;
}

int launch_refill(const TraceParams& P, const rmg_sensor* sensor, const rmg_launch_config& cfg, cudaStream_t st) {
  unsigned long long* counter = nullptr;
  RMG_CUDA_TRY(cudaMallocAsync(reinterpret_cast<void**>(&counter), sizeof(unsigned long long), st));
  cudaError_t e = cudaMemsetAsync(counter, 0, sizeof(unsigned long long), st);
  const unsigned block = 32u * cfg.block_warps;
  if (e == cudaSuccess) {
    switch (sensor->model.kind) {
      case RMG_MODEL_SPHERICAL:
      case RMG_MODEL_PINHOLE:
        e = launch_trace_refill<ORIGIN_POSE>(P, (int)cfg.stack_depth, block, counter, cfg.chunk, cfg.refill, st);
        break;
      case RMG_MODEL_O1DN:
        e = launch_trace_refill<ORIGIN_SINGLE>(P, (int)cfg.stack_depth, block, counter, cfg.chunk, cfg.refill, st);
        break;
      default: e = launch_trace_refill<ORIGIN_TABLE>(P, (int)cfg.stack_depth, block, counter, cfg.chunk, cfg.refill, st); break;
    }
  }
  const int s = cuda_status(e, "trace refill launch");
  cudaFreeAsync(counter, st);
  return s;
}

int launch_plain(const TraceParams& P, const rmg_sensor* sensor, const rmg_launch_config& cfg,
                 cudaStream_t st) {
  if (cfg.refill) return launch_refill(P, sensor, cfg, st);
  const uint64_t blocks = (P.n_tiles + cfg.block_warps - 1) / cfg.block_warps;
  if (blocks > 0x7fffffffull) return fail(RMG_ERR_INVALID_ARG, "rmg_simulate: too many rays for one launch");
  const unsigned block = 32u * cfg.block_warps;
  cudaError_t e;
  switch (sensor->model.kind) {
    case RMG_MODEL_SPHERICAL:
    case RMG_MODEL_PINHOLE: e = launch_trace<ORIGIN_POSE>(P, (int)cfg.stack_depth, (unsigned)blocks, block, st); break;
    case RMG_MODEL_O1DN: e = launch_trace<ORIGIN_SINGLE>(P, (int)cfg.stack_depth, (unsigned)blocks, block, st); break;
    default: e = launch_trace<ORIGIN_TABLE>(P, (int)cfg.stack_depth, (unsigned)blocks, block, st); break;
  }
  return cuda_status(e, "trace launch");
}

}  // namespace rmg

using namespace rmg;

extern "C" int rmg_default_launch_config(const rmg_map* map, const rmg_sensor* sensor,
                                         rmg_launch_config* cfg) {
  return guarded("rmg_default_launch_config", [&]() -> int {
    (void)map;
    if (!cfg) return fail(RMG_ERR_INVALID_ARG, "rmg_default_launch_config: cfg is NULL");
    return default_config(sensor, cfg);
  });
}

extern "C" int rmg_simulate_ex(const rmg_map* map, const rmg_sensor* sensor, const rmg_transform* Tsb,
                               const rmg_transform* Tbm, uint32_t n_poses, const rmg_outputs* out,
                               const rmg_launch_config* cfg_in, void* stream) {
  return guarded("rmg_simulate_ex", [&]() -> int {
    if (!map || !sensor || !Tsb || !out)
      return fail(RMG_ERR_INVALID_ARG, "rmg_simulate: NULL map, sensor, Tsb or outputs");
    if (n_poses == 0) return RMG_OK;
    if (!Tbm) return fail(RMG_ERR_INVALID_ARG, "rmg_simulate: Tbm is NULL");
    rmg_launch_config cfg;
    if (cfg_in) cfg = *cfg_in; else default_config(sensor, &cfg);
    int s = check_config(cfg);
    if (s != RMG_OK) return s;
    if (!out->hits && !out->ranges && !out->points && !out->normals && !out->face_ids &&
        !out->geom_ids && !out->object_ids)
      return RMG_OK;  // nothing requested: the reference writes nothing either
    TraceParams P;
    make_trace_params(map, sensor, Tsb, Tbm, n_poses, out, cfg, P);
    return launch_plain(P, sensor, cfg, as_stream(stream));
  });
}

extern "C" int rmg_simulate(const rmg_map* map, const rmg_sensor* sensor, const rmg_transform* Tsb,
                            const rmg_transform* Tbm, uint32_t n_poses, const rmg_outputs* out,
                            void* stream) {
  return guarded("rmg_simulate", [&]() -> int {
    return rmg_simulate_ex(map, sensor, Tsb, Tbm, n_poses, out, nullptr, stream);
  });
}

// Launch autotuner for one (map, sensor, pose set): times a fixed list of
// candidate configurations -- per-ray binary walk, warp packet walk and 4-wide
// walk, each with three tile shapes and two CTA sizes -- on the caller's own
// poses and output buffers (every candidate writes the same results) and
// returns the fastest by median of `reps` timed runs after one warm-up run.
// Synchronises.  No counterpart in the reference.
extern "C" int rmg_autotune_launch_config(const rmg_map* map, const rmg_sensor* sensor, const rmg_transform* Tsb,
                                          const rmg_transform* Tbm, uint32_t n_poses, const rmg_outputs* out,
                                          uint32_t reps, rmg_launch_config* best, void* stream) {
  return guarded("rmg_autotune_launch_config", [&]() -> int {
    if (!map || !sensor || !Tsb || !Tbm || !out || !best || n_poses == 0)
      return fail(RMG_ERR_INVALID_ARG, "rmg_autotune_launch_config: NULL argument or no poses");
    reps = std::max(1u, std::min(reps, 50u));
    cudaStream_t st = as_stream(stream);
    rmg_launch_config base;
    default_config(sensor, &base);
    struct Walk { uint32_t bvh_width, packet; };
    const Walk walks[4] = {{2, 0}, {2, 1}, {4, 0}, {8, 0}};
    const uint32_t tiles[3][2] = {{8, 4}, {16, 2}, {4, 8}};
    const uint32_t warps[2] = {4, 2};
    cudaEvent_t e0, e1;
    RMG_CUDA_TRY(cudaEventCreate(&e0));
    RMG_CUDA_TRY(cudaEventCreate(&e1));
    float best_ms = 1e30f;
    int s = RMG_OK;
    bool any = false;
    for (const Walk& w : walks) {
      for (const auto& t : tiles) {
        for (uint32_t bw : warps) {
          rmg_launch_config c = base;
          c.bvh_width = w.bvh_width;
          c.packet = w.packet;
          c.tile_w = t[0];
          c.tile_h = t[1];
          c.block_warps = bw;
          if (c.tile_w > sensor->width && c.tile_w != base.tile_w) continue;
          if (check_config(c) != RMG_OK) continue;
          TraceParams P;
          make_trace_params(map, sensor, Tsb, Tbm, n_poses, out, c, P);
          if ((w.bvh_width == 4 && !P.wide) || (w.bvh_width == 8 && !P.wide8) || (w.packet == 1 && !P.packet))
            continue;  // not available here
          s = launch_plain(P, sensor, c, st);
          if (s != RMG_OK) break;
          std::vector<float> ms;
          for (uint32_t r = 0; r < reps && s == RMG_OK; ++r) {
            s = cuda_status(cudaEventRecord(e0, st), "event");
            if (s == RMG_OK) s = launch_plain(P, sensor, c, st);
            if (s == RMG_OK) s = cuda_status(cudaEventRecord(e1, st), "event");
            if (s == RMG_OK) s = cuda_status(cudaEventSynchronize(e1), "event sync");
            float x = 0.f;
            if (s == RMG_OK) s = cuda_status(cudaEventElapsedTime(&x, e0, e1), "event time");
            ms.push_back(x);
          }
          if (s != RMG_OK) break;
          std::sort(ms.begin(), ms.end());
          const float med = ms[ms.size() / 2];
          if (med < best_ms) { best_ms = med; *best = c; any = true; }
        }
        if (s != RMG_OK) break;
      }
      if (s != RMG_OK) break;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (s != RMG_OK) return s;
    if (!any) *best = base;
    return RMG_OK;
  });
}
