// Host-buffer forms of rmg_simulate, rmg_simulate_scene and
// rmg_simulate_statistics: poses, inputs and results in host memory, like the
// Embree simulators' RAM bundles
// (SphereSimulatorEmbree.hpp:130-155).  The poses are uploaded once; the rays
// are cast in pose chunks into device staging slots, alternating between the
// caller's stream and further compute streams so that one chunk's last warps
// overlap the next chunk's first ones (a small launch is otherwise as long as
// its slowest warp), and each chunk's outputs are copied to the host on a copy
// stream while later chunks are cast.  Chunks are launched ahead of the copies
// that free their slots' predecessors, so a pageable destination (whose
// device->host copy returns to the host only when it is done) still overlaps
// with the casting.
#include <atomic>
#include <algorithm>
#include <cstring>
#include <functional>
#include <memory>
#include <mutex>
#include <thread>
#include <vector>

#include "internal.h"

namespace rmg {
namespace {

constexpr int kMaxCompute = 3;   // compute streams at most (the caller's and up to two more)
constexpr int kSlots = 4;        // staging chunks in flight; more than the compute streams (see host_pipeline)
constexpr int kMaxDevices = 64;
constexpr size_t kDefaultChunkBytes = size_t(128) << 20;
constexpr int kDefaultCompute = 2;
std::atomic<size_t> g_chunk_bytes{kDefaultChunkBytes};
std::atomic<int> g_compute{kDefaultCompute};

// Staging memory comes from one stream-ordered pool per device that keeps what
// it holds between calls (release threshold: everything), so a repeated call
// allocates nothing from the driver; rmg_host_staging_trim gives it back.
std::mutex g_pool_mu;
cudaMemPool_t g_pool[kMaxDevices] = {};

int staging_pool(cudaMemPool_t* out) {
  int dev = 0;
  RMG_CUDA_TRY(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) return fail(RMG_ERR_UNSUPPORTED, "host staging: device ordinal out of range");
  std::lock_guard<std::mutex> lock(g_pool_mu);
  if (!g_pool[dev]) {
    cudaMemPoolProps p{};
    p.allocType = cudaMemAllocationTypePinned;
    p.handleTypes = cudaMemHandleTypeNone;
    p.location.type = cudaMemLocationTypeDevice;
    p.location.id = dev;
    cudaMemPool_t pool;
    RMG_CUDA_TRY(cudaMemPoolCreate(&pool, &p));
    uint64_t keep = UINT64_MAX;
    const cudaError_t e = cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
    if (e != cudaSuccess) {
      cudaMemPoolDestroy(pool);
      return cuda_status(e, "cudaMemPoolSetAttribute");
    }
    g_pool[dev] = pool;
  }
  *out = g_pool[dev];
  return RMG_OK;
}

// The seven output attributes as (pointer, bytes per ray) pairs, rmg_outputs order.
struct AttrList {
  char* ptr[7];
  size_t size[7];
};

AttrList attrs_of(const rmg_outputs& o) {
  return AttrList{{reinterpret_cast<char*>(o.hits), reinterpret_cast<char*>(o.ranges),
                   reinterpret_cast<char*>(o.points), reinterpret_cast<char*>(o.normals),
                   reinterpret_cast<char*>(o.face_ids), reinterpret_cast<char*>(o.geom_ids),
                   reinterpret_cast<char*>(o.object_ids)},
                  {1, 4, 12, 12, 4, 4, 4}};
}

rmg_outputs outputs_at(const AttrList& a) {
  rmg_outputs o;
  o.hits = reinterpret_cast<uint8_t*>(a.ptr[0]);
  o.ranges = reinterpret_cast<float*>(a.ptr[1]);
  o.points = reinterpret_cast<rmg_vec3*>(a.ptr[2]);
  o.normals = reinterpret_cast<rmg_vec3*>(a.ptr[3]);
  o.face_ids = reinterpret_cast<uint32_t*>(a.ptr[4]);
  o.geom_ids = reinterpret_cast<uint32_t*>(a.ptr[5]);
  o.object_ids = reinterpret_cast<uint32_t*>(a.ptr[6]);
  return o;
}

using Launch = std::function<int(const rmg_transform* Tbm, uint32_t n, const rmg_outputs* out, cudaStream_t st)>;

// Pose chunks of the simulate host forms: full chunks of `chunk` poses, then
// the last two chunks' worth split in halving sizes (at least chunk / 8 poses),
// so that the work left after the final launch -- its copy, and forming its
// points -- is a small chunk's.  Returns the first pose of every chunk and n.
std::vector<uint32_t> chunk_schedule(uint32_t n, size_t chunk) {
  std::vector<uint32_t> first{0};
  uint64_t p = 0;
  while (n - p > 2 * chunk) {
    p += chunk;
    first.push_back((uint32_t)p);
  }
  const uint64_t min_tail = std::max<uint64_t>(1, chunk / 8);
  while (p < n) {
    const uint64_t rem = n - p;
    const uint64_t take = rem <= min_tail ? rem : std::max<uint64_t>(min_tail, std::min<uint64_t>(chunk, (rem + 1) / 2));
    p += take;
    first.push_back((uint32_t)p);
  }
  return first;
}

// Points follow from the range of a ray (the attribute rules of
// SphereSimulatorEmbree.tcc:104-249, as the traversal kernels write them): a
// ray hit iff its range is at most range.max (a miss writes range.max + 1), and
// points = dir_s * range (+ orig_s for O1Dn / OnDn) for a hit, NaN for a miss.
// When the caller wants Ranges and Points of many rays, the host forms copy the
// ranges over the host link (which bounds these calls) but not the 12-byte
// points, and form the points on host threads from the ranges as each chunk
// lands, in the same binary32 operations as the kernel (one product, one sum,
// no contraction): the same bytes in the results, 12 fewer per ray on the
// link.  Hits (1 byte per ray) are cheaper to copy than to form.  Not used
// when range.max + 1 rounds to range.max (a hit at range.max would look like a
// miss), nor below kDeriveMinBytes of points (threads cost more than they save).
constexpr uint64_t kDeriveMinBytes = uint64_t(64) << 20;
// rmg_host_set_points_policy: 0 form points on the host threads, 1 copy them over the link
std::atomic<uint32_t> g_points_policy{0};
struct HostDerive {
  bool points = false;
  float rmax = 0.f;
  int kind = 0;                    // rmg_model_kind
  std::vector<float> dirs, origs;  // sensor frame, 3 per ray of one pose
  float orig[3] = {0.f, 0.f, 0.f};
  uint64_t rays_per_pose = 0;
  const float* ranges_h = nullptr;
  float* points_h = nullptr;

  bool active() const { return points; }

  // rays [r0, r1) of the whole output, pose segment by pose segment (contiguous
  // ranges, directions and points: loops the compiler vectorizes)
  void run(uint64_t r0, uint64_t r1) const {
    while (r0 < r1) {
      const uint64_t loc0 = r0 % rays_per_pose;
      const uint64_t len = std::min<uint64_t>(r1 - r0, rays_per_pose - loc0);
      segment(r0, loc0, len);
      r0 += len;
    }
  }

  void segment(uint64_t i0, uint64_t loc0, uint64_t len) const {
    const float* __restrict__ rr = ranges_h + i0;
    const float hi = rmax;
    uint32_t nan_bits = 0x7fc00000u;
    float nan_;
    std::memcpy(&nan_, &nan_bits, 4);
    const float* __restrict__ dd = dirs.data() + 3 * loc0;
    float* __restrict__ pp = points_h + 3 * i0;
    if (kind == RMG_MODEL_O1DN) {
      const float ox = orig[0], oy = orig[1], oz = orig[2];
      for (uint64_t j = 0; j < len; ++j) {
        const float r = rr[j];
        const bool hit = r <= hi;
        const float x = dd[3 * j] * r + ox, y = dd[3 * j + 1] * r + oy, z = dd[3 * j + 2] * r + oz;
        pp[3 * j] = hit ? x : nan_;
        pp[3 * j + 1] = hit ? y : nan_;
        pp[3 * j + 2] = hit ? z : nan_;
      }
    } else if (kind == RMG_MODEL_ONDN) {
      const float* __restrict__ oo = origs.data() + 3 * loc0;
      for (uint64_t j = 0; j < len; ++j) {
        const float r = rr[j];
        const bool hit = r <= hi;
        const float x = dd[3 * j] * r + oo[3 * j], y = dd[3 * j + 1] * r + oo[3 * j + 1],
                    z = dd[3 * j + 2] * r + oo[3 * j + 2];
        pp[3 * j] = hit ? x : nan_;
        pp[3 * j + 1] = hit ? y : nan_;
        pp[3 * j + 2] = hit ? z : nan_;
      }
    } else {
      for (uint64_t j = 0; j < len; ++j) {
        const float r = rr[j];
        const bool hit = r <= hi;
        const float x = dd[3 * j] * r, y = dd[3 * j + 1] * r, z = dd[3 * j + 2] * r;
        pp[3 * j] = hit ? x : nan_;
        pp[3 * j + 1] = hit ? y : nan_;
        pp[3 * j + 2] = hit ? z : nan_;
      }
    }
  }
};

// Sets up the host-side derivation of Points for `out` (and removes them from
// the device outputs) when the caller wants Ranges and Points of n_poses poses.
int host_derive_setup(const rmg_sensor* sensor, uint32_t n_poses, rmg_outputs& out, HostDerive& d) {
  if (!out.ranges || !out.points || g_points_policy.load() == 1) return RMG_OK;
  if ((uint64_t)n_poses * sensor->width * sensor->height * 12 < kDeriveMinBytes) return RMG_OK;
  const float rmax = sensor->model.range.max;
  const float miss = rmax + 1.0f;  // the kernels' miss range, binary32
  if (!(miss > rmax)) return RMG_OK;
  d.rmax = rmax;
  d.kind = (int)sensor->model.kind;
  d.rays_per_pose = (uint64_t)sensor->width * sensor->height;
  {
    d.dirs.resize(3 * d.rays_per_pose);
    RMG_CUDA_TRY(cudaMemcpy(d.dirs.data(), sensor->d_dirs, d.dirs.size() * 4, cudaMemcpyDeviceToHost));
    if (d.kind == RMG_MODEL_ONDN) {
      d.origs.resize(3 * d.rays_per_pose);
      RMG_CUDA_TRY(cudaMemcpy(d.origs.data(), sensor->d_origs, d.origs.size() * 4, cudaMemcpyDeviceToHost));
    }
    d.orig[0] = sensor->model.orig.x;
    d.orig[1] = sensor->model.orig.y;
    d.orig[2] = sensor->model.orig.z;
  }
  d.points = true;
  d.ranges_h = out.ranges;
  d.points_h = reinterpret_cast<float*>(out.points);
  out.points = nullptr;
  return RMG_OK;
}

// Streams and events of one call; released in every exit path.
struct Pipeline {
  cudaStream_t side[kMaxCompute - 1] = {};  // compute streams besides the caller's
  cudaStream_t copy = nullptr;
  cudaEvent_t cast[kSlots] = {};     // chunk in slot s written (its compute stream)
  cudaEvent_t copied[kSlots] = {};   // chunk in slot s read back (copy stream)
  cudaEvent_t ready = nullptr;       // poses uploaded (caller's stream)
  cudaEvent_t side_done[kMaxCompute - 1] = {};
  cudaEvent_t done = nullptr;
  ~Pipeline() {
    for (int s = 0; s < kSlots; ++s) {
      if (cast[s]) cudaEventDestroy(cast[s]);
      if (copied[s]) cudaEventDestroy(copied[s]);
    }
    for (int k = 0; k < kMaxCompute - 1; ++k) {
      if (side_done[k]) cudaEventDestroy(side_done[k]);
      if (side[k]) cudaStreamDestroy(side[k]);
    }
    for (cudaEvent_t e : {ready, done})
      if (e) cudaEventDestroy(e);
    if (copy) cudaStreamDestroy(copy);
  }
};

// The streams and events of the simulate host forms, made once per host
// thread and device and kept (creating them took a measurable share of a
// small call): a call is synchronous, so the next call of the same thread
// finds them idle; other threads have their own.
int cached_pipeline(Pipeline** out) {
  int dev = 0;
  RMG_CUDA_TRY(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) return fail(RMG_ERR_UNSUPPORTED, "host forms: device ordinal out of range");
  thread_local std::unique_ptr<Pipeline> cache[kMaxDevices];
  if (!cache[dev]) {
    std::unique_ptr<Pipeline> pl(new Pipeline);
    for (int k = 0; k + 1 < kMaxCompute; ++k) {
      RMG_CUDA_TRY(cudaStreamCreateWithFlags(&pl->side[k], cudaStreamNonBlocking));
      RMG_CUDA_TRY(cudaEventCreateWithFlags(&pl->side_done[k], cudaEventDisableTiming));
    }
    RMG_CUDA_TRY(cudaStreamCreateWithFlags(&pl->copy, cudaStreamNonBlocking));
    for (int k = 0; k < kSlots; ++k) {
      RMG_CUDA_TRY(cudaEventCreateWithFlags(&pl->cast[k], cudaEventDisableTiming));
      RMG_CUDA_TRY(cudaEventCreateWithFlags(&pl->copied[k], cudaEventDisableTiming));
    }
    RMG_CUDA_TRY(cudaEventCreateWithFlags(&pl->ready, cudaEventDisableTiming));
    RMG_CUDA_TRY(cudaEventCreateWithFlags(&pl->done, cudaEventDisableTiming));
    cache[dev] = std::move(pl);
  }
  *out = cache[dev].get();
  return RMG_OK;
}

// Chunk k is cast on compute stream k % nc into slot k % kSlots (nc compute
// streams).  Chunks 0..nc-1 are launched first; then iteration k launches
// chunk k+nc and issues chunk k's copies.  The launch of chunk j waits for the
// copy of chunk j-kSlots (same slot), which was issued at iteration j-kSlots <
// j-nc, i.e. before the wait is enqueued, because kSlots > nc.
int host_pipeline(const char* what, const rmg_sensor* sensor, const rmg_transform* Tbm_host, uint32_t n_poses,
                  const rmg_outputs& out_caller, cudaStream_t st, const Launch& launch) {
  static_assert(kSlots > kMaxCompute, "a slot is reused only after its copy was issued");
  const uint64_t rays_per_pose = (uint64_t)sensor->width * sensor->height;
  const uint32_t nc = (uint32_t)std::min(std::max(g_compute.load(), 1), kMaxCompute);
  rmg_outputs out_host = out_caller;
  HostDerive derive;
  const int r = host_derive_setup(sensor, n_poses, out_host, derive);
  if (r != RMG_OK) return r;
  const AttrList host = attrs_of(out_host);
  size_t bytes_per_ray = derive.points ? 12 : 0;  // chunks sized by the results, derived ones included
  for (int a = 0; a < 7; ++a)
    if (host.ptr[a]) bytes_per_ray += host.size[a];
  if (bytes_per_ray == 0 || rays_per_pose == 0) return RMG_OK;
  const size_t bytes_per_pose = bytes_per_ray * rays_per_pose;
  // at least one pose, at most ceil(n/2) so that two chunks overlap
  size_t chunk = std::max<size_t>(1, g_chunk_bytes.load() / bytes_per_pose);
  chunk = std::min<size_t>(chunk, std::max<uint32_t>(1u, (n_poses + 1) / 2));
  const std::vector<uint32_t> first = chunk_schedule(n_poses, chunk);  // chunk k: poses [first[k], first[k+1])
  const uint32_t n_chunks = (uint32_t)first.size() - 1;
  const int slots = (int)std::min<uint32_t>(kSlots, n_chunks);

  cudaMemPool_t pool;
  int s = staging_pool(&pool);
  if (s != RMG_OK) return s;
  Pipeline* pp = nullptr;
  s = cached_pipeline(&pp);
  if (s != RMG_OK) return s;
  Pipeline& pl = *pp;
  cudaStream_t compute[kMaxCompute] = {st};
  for (uint32_t k = 0; k + 1 < nc; ++k) compute[k + 1] = pl.side[k];

  // staging: all poses, then `slots` output chunks, every array 256-byte aligned
  const size_t pose_bytes = ((size_t)n_poses * sizeof(rmg_transform) + 255) & ~size_t(255);
  size_t slot_bytes = 0;
  size_t offset[7] = {};
  for (int a = 0; a < 7; ++a) {
    if (!host.ptr[a]) continue;
    offset[a] = slot_bytes;
    slot_bytes += (chunk * rays_per_pose * host.size[a] + 255) & ~size_t(255);
  }
  std::vector<cudaEvent_t> chunk_copied;  // per chunk: its outputs are in host memory (host derivation)
  struct EventsGuard {
    std::vector<cudaEvent_t>& v;
    ~EventsGuard() { for (cudaEvent_t e : v) if (e) cudaEventDestroy(e); }
  } events_guard{chunk_copied};
  if (derive.active()) {
    chunk_copied.assign(n_chunks, nullptr);
    for (uint32_t k = 0; k < n_chunks; ++k)
      RMG_CUDA_TRY(cudaEventCreateWithFlags(&chunk_copied[k], cudaEventDisableTiming | cudaEventBlockingSync));
  }
  char* staging = nullptr;
  RMG_CUDA_TRY(cudaMallocFromPoolAsync(reinterpret_cast<void**>(&staging), pose_bytes + slots * slot_bytes, pool, st));
  const auto* Tbm_dev = reinterpret_cast<const rmg_transform*>(staging);
  s = cuda_status(cudaMemcpyAsync(staging, Tbm_host, (size_t)n_poses * sizeof(rmg_transform), cudaMemcpyDefault, st),
                  what);
  if (s == RMG_OK) s = cuda_status(cudaEventRecord(pl.ready, st), what);
  for (uint32_t k = 0; s == RMG_OK && k + 1 < nc; ++k) s = cuda_status(cudaStreamWaitEvent(pl.side[k], pl.ready, 0), what);

  auto slot_outputs = [&](int slot) {
    AttrList d = host;
    for (int a = 0; a < 7; ++a)
      d.ptr[a] = host.ptr[a] ? staging + pose_bytes + slot * slot_bytes + offset[a] : nullptr;
    return d;
  };
  auto cast_chunk = [&](uint32_t k) -> int {
    const int slot = (int)(k % slots);
    const cudaStream_t cs = compute[k % nc];
    const uint32_t p0 = first[k], np = first[k + 1] - first[k];
    if (k >= (uint32_t)slots) RMG_CUDA_TRY(cudaStreamWaitEvent(cs, pl.copied[slot], 0));
    const rmg_outputs o = outputs_at(slot_outputs(slot));
    const int r = launch(Tbm_dev + p0, np, &o, cs);
    if (r != RMG_OK) return r;
    RMG_CUDA_TRY(cudaEventRecord(pl.cast[slot], cs));
    return RMG_OK;
  };
  auto copy_chunk = [&](uint32_t k) -> int {
    const int slot = (int)(k % slots);
    const uint64_t p0 = first[k], np = first[k + 1] - first[k];
    RMG_CUDA_TRY(cudaStreamWaitEvent(pl.copy, pl.cast[slot], 0));
    const AttrList d = slot_outputs(slot);
    for (int a = 0; a < 7; ++a) {
      if (!host.ptr[a]) continue;
      const size_t row = rays_per_pose * host.size[a];
      RMG_CUDA_TRY(cudaMemcpyAsync(host.ptr[a] + p0 * row, d.ptr[a], np * row, cudaMemcpyDefault, pl.copy));
    }
    RMG_CUDA_TRY(cudaEventRecord(pl.copied[slot], pl.copy));
    if (!chunk_copied.empty()) RMG_CUDA_TRY(cudaEventRecord(chunk_copied[k], pl.copy));
    return RMG_OK;
  };

  for (uint32_t k = 0; s == RMG_OK && k < std::min<uint32_t>(nc, n_chunks); ++k) s = cast_chunk(k);
  for (uint32_t k = 0; s == RMG_OK && k < n_chunks; ++k) {
    if (k + nc < n_chunks) s = cast_chunk(k + nc);
    if (s == RMG_OK) s = copy_chunk(k);
  }
  // Hits / Points on host threads, chunk by chunk as each chunk's ranges land,
  // while the later chunks are still cast and copied
  if (s == RMG_OK && derive.active()) {
    const uint64_t total = (uint64_t)n_poses * rays_per_pose;
    const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
    const unsigned T = (unsigned)std::min<uint64_t>(std::min(hw, 32u), std::max<uint64_t>(1, total >> 20));
    std::atomic<int> err{RMG_OK};
    auto worker = [&](unsigned w) {
      for (uint32_t k = 0; k < n_chunks; ++k) {
        if (cudaEventSynchronize(chunk_copied[k]) != cudaSuccess) { err.store(RMG_ERR_CUDA); return; }
        const uint64_t c0 = (uint64_t)first[k] * rays_per_pose;
        const uint64_t c1 = (uint64_t)first[k + 1] * rays_per_pose;
        const uint64_t len = c1 - c0;
        derive.run(c0 + len * w / T, c0 + len * (w + 1) / T);
      }
    };
    std::vector<std::thread> pool_threads;
    unsigned started = 1;
    try {  // no exception may leave the C entry points: slices whose thread did not start run here
      for (unsigned w = 1; w < T; ++w) {
        pool_threads.emplace_back(worker, w);
        started = w + 1;
      }
    } catch (...) {
    }
    worker(0);
    for (unsigned w = started; w < T; ++w) worker(w);
    for (auto& t : pool_threads) t.join();
    if (err.load() != RMG_OK) s = fail(RMG_ERR_CUDA, std::string(what) + ": waiting for a chunk's copy failed");
  }
  // the staging is freed in stream order after the last copy and the side
  // streams' last launches, whatever happened
  cudaEventRecord(pl.done, pl.copy);
  cudaStreamWaitEvent(st, pl.done, 0);
  for (uint32_t k = 0; k + 1 < nc; ++k) {
    cudaEventRecord(pl.side_done[k], pl.side[k]);
    cudaStreamWaitEvent(st, pl.side_done[k], 0);
  }
  cudaFreeAsync(staging, st);
  const cudaError_t e = cudaStreamSynchronize(st);
  if (s != RMG_OK) return s;
  return cuda_status(e, what);
}

uint64_t rays_of(const rmg_sensor* sensor) { return (uint64_t)sensor->width * sensor->height; }

inline size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

// Host form of the fused correction step.  Poses, pre-transforms and the small
// per-pose results move in one copy each; per-pose scans (per_pose = 1) are
// uploaded in pose chunks on an upload stream into device slots while earlier
// chunks are reduced, the launches alternating between compute streams.  A
// slot is refilled only after the launch that read it has finished (the
// upload of chunk j waits for the launch of chunk j - slots, issued one
// iteration earlier at least).
int statistics_pipeline(const rmg_map* map, const rmg_sensor* sensor, const rmg_transform* Tsb,
                        const rmg_transform* Tbm_h, uint32_t n, const rmg_scan& scan_h, const rmg_transform* pre_h,
                        uint32_t pre_stride, const rmg_umeyama_constraints* params, int p2l,
                        rmg_cross_stats* stats_h, rmg_transform* T_h, cudaStream_t st) {
  const char* what = "rmg_simulate_statistics_host";
  const uint64_t rays = rays_of(sensor);
  const bool per_pose = scan_h.per_pose != 0;
  const size_t in_per_ray = 12 + (scan_h.mask ? 1 : 0) + (scan_h.ids ? 4 : 0);
  const size_t in_per_pose = in_per_ray * rays;
  const uint32_t nc = (uint32_t)std::min(std::max(g_compute.load(), 1), kMaxCompute);
  size_t chunk = n;
  if (per_pose) {
    chunk = std::max<size_t>(1, g_chunk_bytes.load() / std::max<size_t>(1, in_per_pose));
    chunk = std::min<size_t>(chunk, std::max<uint32_t>(1u, (n + 1) / 2));
  }
  const uint32_t n_chunks = (uint32_t)((n + chunk - 1) / chunk);
  const int slots = per_pose ? (int)std::min<uint32_t>(kSlots, n_chunks) : 1;
  const size_t scan_poses = per_pose ? chunk : 1;  // poses' worth of scan per slot

  cudaMemPool_t pool;
  int s = staging_pool(&pool);
  if (s != RMG_OK) return s;
  Pipeline pl;  // copy = the upload stream here
  RMG_CUDA_TRY(cudaStreamCreateWithFlags(&pl.copy, cudaStreamNonBlocking));
  for (uint32_t k = 0; k + 1 < nc; ++k) {
    RMG_CUDA_TRY(cudaStreamCreateWithFlags(&pl.side[k], cudaStreamNonBlocking));
    RMG_CUDA_TRY(cudaEventCreateWithFlags(&pl.side_done[k], cudaEventDisableTiming));
  }
  for (int k = 0; k < slots; ++k) {
    RMG_CUDA_TRY(cudaEventCreateWithFlags(&pl.cast[k], cudaEventDisableTiming));    // slot uploaded
    RMG_CUDA_TRY(cudaEventCreateWithFlags(&pl.copied[k], cudaEventDisableTiming));  // slot consumed
  }
  RMG_CUDA_TRY(cudaEventCreateWithFlags(&pl.ready, cudaEventDisableTiming));
  RMG_CUDA_TRY(cudaEventCreateWithFlags(&pl.done, cudaEventDisableTiming));
  cudaStream_t compute[kMaxCompute] = {st};
  for (uint32_t k = 0; k + 1 < nc; ++k) compute[k + 1] = pl.side[k];

  // staging layout
  const size_t n_pre = pre_h ? (pre_stride ? (size_t)n : 1) : 0;
  size_t off = 0;
  const size_t o_T = off;    off += align256((size_t)n * sizeof(rmg_transform));
  const size_t o_pre = off;  off += align256(n_pre * sizeof(rmg_transform));
  const size_t o_st = off;   off += align256(stats_h ? (size_t)n * sizeof(rmg_cross_stats) : 0);
  const size_t o_Tout = off; off += align256(T_h ? (size_t)n * sizeof(rmg_transform) : 0);
  const size_t sp_pts = align256(scan_poses * rays * 12);
  const size_t sp_mask = scan_h.mask ? align256(scan_poses * rays) : 0;
  const size_t sp_ids = scan_h.ids ? align256(scan_poses * rays * 4) : 0;
  const size_t slot_bytes = sp_pts + sp_mask + sp_ids;
  const size_t o_slots = off;
  off += slots * slot_bytes;
  char* stg = nullptr;
  RMG_CUDA_TRY(cudaMallocFromPoolAsync(reinterpret_cast<void**>(&stg), off, pool, st));
  auto* Tbm_d = reinterpret_cast<rmg_transform*>(stg + o_T);
  auto* pre_d = pre_h ? reinterpret_cast<rmg_transform*>(stg + o_pre) : nullptr;
  auto* stats_d = stats_h ? reinterpret_cast<rmg_cross_stats*>(stg + o_st) : nullptr;
  auto* Tout_d = T_h ? reinterpret_cast<rmg_transform*>(stg + o_Tout) : nullptr;
  s = cuda_status(cudaMemcpyAsync(Tbm_d, Tbm_h, (size_t)n * sizeof(rmg_transform), cudaMemcpyDefault, st), what);
  if (s == RMG_OK && pre_d)
    s = cuda_status(cudaMemcpyAsync(pre_d, pre_h, n_pre * sizeof(rmg_transform), cudaMemcpyDefault, st), what);
  if (s == RMG_OK) s = cuda_status(cudaEventRecord(pl.ready, st), what);
  if (s == RMG_OK) s = cuda_status(cudaStreamWaitEvent(pl.copy, pl.ready, 0), what);
  for (uint32_t k = 0; s == RMG_OK && k + 1 < nc; ++k) s = cuda_status(cudaStreamWaitEvent(pl.side[k], pl.ready, 0), what);

  auto upload = [&](uint32_t k) -> int {
    const int slot = (int)(k % slots);
    const uint64_t p0 = per_pose ? (uint64_t)k * chunk : 0;
    const uint64_t np = per_pose ? std::min<uint64_t>(chunk, n - p0) : 1;
    char* base = stg + o_slots + slot * slot_bytes;
    if (k >= (uint32_t)slots) RMG_CUDA_TRY(cudaStreamWaitEvent(pl.copy, pl.copied[slot], 0));
    RMG_CUDA_TRY(cudaMemcpyAsync(base, scan_h.points + p0 * rays, np * rays * 12, cudaMemcpyDefault, pl.copy));
    if (scan_h.mask)
      RMG_CUDA_TRY(cudaMemcpyAsync(base + sp_pts, scan_h.mask + p0 * rays, np * rays, cudaMemcpyDefault, pl.copy));
    if (scan_h.ids)
      RMG_CUDA_TRY(cudaMemcpyAsync(base + sp_pts + sp_mask, scan_h.ids + p0 * rays, np * rays * 4, cudaMemcpyDefault,
                                   pl.copy));
    RMG_CUDA_TRY(cudaEventRecord(pl.cast[slot], pl.copy));
    return RMG_OK;
  };
  auto reduce = [&](uint32_t k) -> int {
    const int slot = per_pose ? (int)(k % slots) : 0;
    const cudaStream_t cs = compute[k % nc];
    const uint32_t p0 = (uint32_t)(k * chunk), np = (uint32_t)std::min<size_t>(chunk, n - p0);
    char* base = stg + o_slots + slot * slot_bytes;
    if (per_pose || k == 0) RMG_CUDA_TRY(cudaStreamWaitEvent(cs, pl.cast[slot], 0));
    rmg_scan sc;
    sc.points = reinterpret_cast<const rmg_vec3*>(base);
    sc.mask = scan_h.mask ? reinterpret_cast<const uint8_t*>(base + sp_pts) : nullptr;
    sc.ids = scan_h.ids ? reinterpret_cast<const uint32_t*>(base + sp_pts + sp_mask) : nullptr;
    sc.per_pose = scan_h.per_pose;
    const int r = rmg_simulate_statistics(map, sensor, Tsb, Tbm_d + p0, np, &sc,
                                          pre_d ? pre_d + (pre_stride ? p0 : 0) : nullptr, pre_stride, params, p2l,
                                          stats_d ? stats_d + p0 : nullptr, Tout_d ? Tout_d + p0 : nullptr, cs);
    if (r != RMG_OK) return r;
    if (per_pose) RMG_CUDA_TRY(cudaEventRecord(pl.copied[slot], cs));
    return RMG_OK;
  };
  if (per_pose) {
    for (uint32_t k = 0; s == RMG_OK && k < n_chunks; ++k) {
      s = upload(k);
      if (s == RMG_OK) s = reduce(k);
    }
  } else {
    s = upload(0);
    for (uint32_t k = 0; s == RMG_OK && k < n_chunks; ++k) s = reduce(k);
  }
  // join, download the per-pose results, free in stream order
  cudaEventRecord(pl.done, pl.copy);
  cudaStreamWaitEvent(st, pl.done, 0);
  for (uint32_t k = 0; k + 1 < nc; ++k) {
    cudaEventRecord(pl.side_done[k], pl.side[k]);
    cudaStreamWaitEvent(st, pl.side_done[k], 0);
  }
  if (s == RMG_OK && stats_h)
    s = cuda_status(cudaMemcpyAsync(stats_h, stats_d, (size_t)n * sizeof(rmg_cross_stats), cudaMemcpyDefault, st),
                    what);
  if (s == RMG_OK && T_h)
    s = cuda_status(cudaMemcpyAsync(T_h, Tout_d, (size_t)n * sizeof(rmg_transform), cudaMemcpyDefault, st), what);
  cudaFreeAsync(stg, st);
  const cudaError_t e = cudaStreamSynchronize(st);
  if (s != RMG_OK) return s;
  return cuda_status(e, what);
}

// A three-stage pipeline over pose chunks: per-pose host inputs are uploaded
// into a device slot (upload stream), the chunk is computed (alternating
// compute streams) and its per-pose outputs are downloaded (download stream),
// so the copies of neighbouring chunks overlap the computation.  A slot is
// uploaded into again only after its previous chunk's downloads (which wait
// for that chunk's computation) were issued, at least one iteration earlier.
struct HostArray {
  const void* src;  // input: host (or device) array of n * per_pose bytes, or NULL
  void* dst;        // output: host (or device) array of n * per_pose bytes, or NULL
  size_t per_pose;
};
using ChunkLaunch = std::function<int(uint32_t p0, uint32_t np, char* const* dev, cudaStream_t st)>;

int io_pipeline(const char* what, uint32_t n, const std::vector<HostArray>& arrays, size_t max_chunk,
                const ChunkLaunch& launch, cudaStream_t st) {
  const size_t na = arrays.size();
  size_t per_pose = 0;
  for (const HostArray& a : arrays) per_pose += a.per_pose;
  size_t chunk = std::max<size_t>(1, g_chunk_bytes.load() / std::max<size_t>(1, per_pose));
  chunk = std::min<size_t>(chunk, std::max<uint32_t>(1u, (n + 1) / 2));
  chunk = std::min<size_t>(chunk, std::max<size_t>(1, max_chunk));
  const uint32_t n_chunks = (uint32_t)((n + chunk - 1) / chunk);
  const int slots = (int)std::min<uint32_t>(kSlots, n_chunks);
  const uint32_t nc = (uint32_t)std::min(std::max(g_compute.load(), 1), kMaxCompute);

  cudaMemPool_t pool;
  int s = staging_pool(&pool);
  if (s != RMG_OK) return s;
  Pipeline pl;  // copy = upload stream, down = the download stream below
  cudaStream_t down = nullptr;
  cudaEvent_t uploaded[kSlots] = {}, computed[kSlots] = {}, released[kSlots] = {};
  struct Release {
    cudaStream_t* s;
    cudaEvent_t* ev[3];
    int n;
    ~Release() {
      for (int k = 0; k < n; ++k)
        for (cudaEvent_t* e : ev)
          if (e[k]) cudaEventDestroy(e[k]);
      if (*s) cudaStreamDestroy(*s);
    }
  } rel{&down, {uploaded, computed, released}, kSlots};
  RMG_CUDA_TRY(cudaStreamCreateWithFlags(&pl.copy, cudaStreamNonBlocking));
  RMG_CUDA_TRY(cudaStreamCreateWithFlags(&down, cudaStreamNonBlocking));
  for (uint32_t k = 0; k + 1 < nc; ++k) {
    RMG_CUDA_TRY(cudaStreamCreateWithFlags(&pl.side[k], cudaStreamNonBlocking));
    RMG_CUDA_TRY(cudaEventCreateWithFlags(&pl.side_done[k], cudaEventDisableTiming));
  }
  for (int k = 0; k < slots; ++k) {
    RMG_CUDA_TRY(cudaEventCreateWithFlags(&uploaded[k], cudaEventDisableTiming));
    RMG_CUDA_TRY(cudaEventCreateWithFlags(&computed[k], cudaEventDisableTiming));
    RMG_CUDA_TRY(cudaEventCreateWithFlags(&released[k], cudaEventDisableTiming));
  }
  RMG_CUDA_TRY(cudaEventCreateWithFlags(&pl.ready, cudaEventDisableTiming));
  RMG_CUDA_TRY(cudaEventCreateWithFlags(&pl.done, cudaEventDisableTiming));
  cudaStream_t compute[kMaxCompute] = {st};
  for (uint32_t k = 0; k + 1 < nc; ++k) compute[k + 1] = pl.side[k];

  std::vector<size_t> offset(na);
  size_t slot_bytes = 0;
  for (size_t a = 0; a < na; ++a) {
    offset[a] = slot_bytes;
    slot_bytes += align256(chunk * arrays[a].per_pose);
  }
  char* stg = nullptr;
  RMG_CUDA_TRY(cudaMallocFromPoolAsync(reinterpret_cast<void**>(&stg), std::max<size_t>(256, slots * slot_bytes), pool,
                                       st));
  s = cuda_status(cudaEventRecord(pl.ready, st), what);
  if (s == RMG_OK) s = cuda_status(cudaStreamWaitEvent(pl.copy, pl.ready, 0), what);
  if (s == RMG_OK) s = cuda_status(cudaStreamWaitEvent(down, pl.ready, 0), what);
  for (uint32_t k = 0; s == RMG_OK && k + 1 < nc; ++k) s = cuda_status(cudaStreamWaitEvent(pl.side[k], pl.ready, 0), what);

  std::vector<char*> dev(na);
  auto place = [&](int slot) {
    for (size_t a = 0; a < na; ++a) dev[a] = stg + (size_t)slot * slot_bytes + offset[a];
  };
  auto upload = [&](uint32_t k) -> int {
    const int slot = (int)(k % slots);
    const uint64_t p0 = (uint64_t)k * chunk, np = std::min<uint64_t>(chunk, n - p0);
    place(slot);
    if (k >= (uint32_t)slots) RMG_CUDA_TRY(cudaStreamWaitEvent(pl.copy, released[slot], 0));
    for (size_t a = 0; a < na; ++a) {
      if (!arrays[a].src) continue;
      const size_t b = arrays[a].per_pose;
      RMG_CUDA_TRY(cudaMemcpyAsync(dev[a], static_cast<const char*>(arrays[a].src) + p0 * b, np * b, cudaMemcpyDefault,
                                   pl.copy));
    }
    RMG_CUDA_TRY(cudaEventRecord(uploaded[slot], pl.copy));
    return RMG_OK;
  };
  auto run = [&](uint32_t k) -> int {
    const int slot = (int)(k % slots);
    const cudaStream_t cs = compute[k % nc];
    const uint32_t p0 = (uint32_t)(k * chunk), np = (uint32_t)std::min<size_t>(chunk, n - p0);
    place(slot);
    RMG_CUDA_TRY(cudaStreamWaitEvent(cs, uploaded[slot], 0));
    const int r = launch(p0, np, dev.data(), cs);
    if (r != RMG_OK) return r;
    RMG_CUDA_TRY(cudaEventRecord(computed[slot], cs));
    return RMG_OK;
  };
  auto download = [&](uint32_t k) -> int {
    const int slot = (int)(k % slots);
    const uint64_t p0 = (uint64_t)k * chunk, np = std::min<uint64_t>(chunk, n - p0);
    place(slot);
    RMG_CUDA_TRY(cudaStreamWaitEvent(down, computed[slot], 0));
    for (size_t a = 0; a < na; ++a) {
      if (!arrays[a].dst) continue;
      const size_t b = arrays[a].per_pose;
      RMG_CUDA_TRY(cudaMemcpyAsync(static_cast<char*>(arrays[a].dst) + p0 * b, dev[a], np * b, cudaMemcpyDefault, down));
    }
    RMG_CUDA_TRY(cudaEventRecord(released[slot], down));
    return RMG_OK;
  };
  for (uint32_t k = 0; s == RMG_OK && k < n_chunks; ++k) {
    s = upload(k);
    if (s == RMG_OK) s = run(k);
    if (s == RMG_OK && k > 0) s = download(k - 1);
  }
  if (s == RMG_OK) s = download(n_chunks - 1);
  // join everything into the caller's stream, free in stream order
  cudaEventRecord(pl.done, down);
  cudaStreamWaitEvent(st, pl.done, 0);
  cudaEventRecord(pl.done, pl.copy);
  cudaStreamWaitEvent(st, pl.done, 0);
  for (uint32_t k = 0; k + 1 < nc; ++k) {
    cudaEventRecord(pl.side_done[k], pl.side[k]);
    cudaStreamWaitEvent(st, pl.side_done[k], 0);
  }
  cudaFreeAsync(stg, st);
  const cudaError_t e = cudaStreamSynchronize(st);
  if (s != RMG_OK) return s;
  return cuda_status(e, what);
}

}  // namespace
}  // namespace rmg

using namespace rmg;

extern "C" int rmg_simulate_host(const rmg_map* map, const rmg_sensor* sensor, const rmg_transform* Tsb,
                                 const rmg_transform* Tbm, uint32_t n_poses, const rmg_outputs* out,
                                 const rmg_launch_config* cfg, void* stream) {
  return guarded("rmg_simulate_host", [&]() -> int {
    if (!map || !sensor || !Tsb || !out)
      return fail(RMG_ERR_INVALID_ARG, "rmg_simulate_host: NULL map, sensor, Tsb or outputs");
    if (n_poses == 0) return RMG_OK;
    if (!Tbm) return fail(RMG_ERR_INVALID_ARG, "rmg_simulate_host: Tbm is NULL");
    return host_pipeline("rmg_simulate_host", sensor, Tbm, n_poses, *out, as_stream(stream),
                         [&](const rmg_transform* T, uint32_t n, const rmg_outputs* o, cudaStream_t st) {
                           return rmg_simulate_ex(map, sensor, Tsb, T, n, o, cfg, st);
                         });
  });
}

extern "C" int rmg_simulate_scene_host(const rmg_scene* scene, const rmg_sensor* sensor, const rmg_transform* Tsb,
                                       const rmg_transform* Tbm, uint32_t n_poses, const rmg_outputs* out,
                                       void* stream) {
  return guarded("rmg_simulate_scene_host", [&]() -> int {
    if (!scene || !sensor || !Tsb || !out)
      return fail(RMG_ERR_INVALID_ARG, "rmg_simulate_scene_host: NULL scene, sensor, Tsb or outputs");
    if (n_poses == 0) return RMG_OK;
    if (!Tbm) return fail(RMG_ERR_INVALID_ARG, "rmg_simulate_scene_host: Tbm is NULL");
    return host_pipeline("rmg_simulate_scene_host", sensor, Tbm, n_poses, *out, as_stream(stream),
                         [&](const rmg_transform* T, uint32_t n, const rmg_outputs* o, cudaStream_t st) {
                           return rmg_simulate_scene(scene, sensor, Tsb, T, n, o, st);
                         });
  });
}

extern "C" int rmg_simulate_statistics_host(const rmg_map* map, const rmg_sensor* sensor, const rmg_transform* Tsb,
                                            const rmg_transform* Tbm, uint32_t n_poses, const rmg_scan* dataset,
                                            const rmg_transform* pre_transforms, uint32_t pre_transform_stride,
                                            const rmg_umeyama_constraints* params, int point_to_plane,
                                            rmg_cross_stats* stats, rmg_transform* transforms, void* stream) {
  return guarded("rmg_simulate_statistics_host", [&]() -> int {
    if (!map || !sensor || !Tsb || !dataset || !params)
      return fail(RMG_ERR_INVALID_ARG, "rmg_simulate_statistics_host: NULL map, sensor, Tsb, dataset or params");
    if (n_poses == 0) return RMG_OK;
    if (!Tbm || !dataset->points) return fail(RMG_ERR_INVALID_ARG, "rmg_simulate_statistics_host: Tbm or points NULL");
    if (!stats && !transforms) return RMG_OK;
    return statistics_pipeline(map, sensor, Tsb, Tbm, n_poses, *dataset, pre_transforms, pre_transform_stride ? 1u : 0u,
                               params, point_to_plane, stats, transforms, as_stream(stream));
  });
}

extern "C" int rmg_range_pose_grad_host(const rmg_map* map, const rmg_sensor* sensor, const rmg_transform* Tsb,
                                        const rmg_transform* Tbm, uint32_t n_poses, const float* ranges_obs,
                                        float huber_delta, float* grad, float* loss, float* ranges_sim,
                                        uint32_t* face_ids, void* stream) {
  return guarded("rmg_range_pose_grad_host", [&]() -> int {
    if (!map || !sensor || !Tsb)
      return fail(RMG_ERR_INVALID_ARG, "rmg_range_pose_grad_host: NULL map, sensor or Tsb");
    if (n_poses == 0) return RMG_OK;
    if (!Tbm || !ranges_obs) return fail(RMG_ERR_INVALID_ARG, "rmg_range_pose_grad_host: Tbm or ranges_obs NULL");
    if (!grad && !loss) return fail(RMG_ERR_INVALID_ARG, "rmg_range_pose_grad_host: grad and loss are both NULL");
    const size_t rays = rays_of(sensor);
    // device arrays of a chunk: Tbm, observed ranges (inputs); grad, loss, ranges, face ids (outputs)
    const std::vector<HostArray> arrays = {
        {Tbm, nullptr, sizeof(rmg_transform)}, {ranges_obs, nullptr, 4 * rays},
        {nullptr, grad, grad ? size_t(24) : size_t(0)}, {nullptr, loss, loss ? size_t(4) : size_t(0)},
        {nullptr, ranges_sim, ranges_sim ? 4 * rays : 0}, {nullptr, face_ids, face_ids ? 4 * rays : 0}};
    return io_pipeline("rmg_range_pose_grad_host", n_poses, arrays, 65535,
                       [&](uint32_t, uint32_t np, char* const* d, cudaStream_t cs) {
                         return rmg_range_pose_grad(map, sensor, Tsb, reinterpret_cast<const rmg_transform*>(d[0]), np,
                                                    reinterpret_cast<const float*>(d[1]), huber_delta,
                                                    grad ? reinterpret_cast<float*>(d[2]) : nullptr,
                                                    loss ? reinterpret_cast<float*>(d[3]) : nullptr,
                                                    ranges_sim ? reinterpret_cast<float*>(d[4]) : nullptr,
                                                    face_ids ? reinterpret_cast<uint32_t*>(d[5]) : nullptr, cs);
                       },
                       as_stream(stream));
  });
}

extern "C" int rmg_host_set_pipeline(uint64_t chunk_bytes, uint32_t compute_streams) {
  return guarded("rmg_host_set_pipeline", [&]() -> int {
    if (compute_streams > (uint32_t)kMaxCompute)
      return fail(RMG_ERR_UNSUPPORTED, "rmg_host_set_pipeline: compute_streams must be 0..3");
    g_chunk_bytes.store(chunk_bytes ? (size_t)chunk_bytes : kDefaultChunkBytes);
    g_compute.store(compute_streams ? (int)compute_streams : kDefaultCompute);
    return RMG_OK;
  });
}

extern "C" int rmg_host_set_points_policy(uint32_t policy) {
  return guarded("rmg_host_set_points_policy", [&]() -> int {
    if (policy > 1) return fail(RMG_ERR_UNSUPPORTED, "rmg_host_set_points_policy: policy must be 0 or 1");
    g_points_policy.store(policy);
    return RMG_OK;
  });
}

extern "C" int rmg_host_staging_trim(void) {
  return guarded("rmg_host_staging_trim", [&]() -> int {
    std::lock_guard<std::mutex> lock(g_pool_mu);
    for (int d = 0; d < kMaxDevices; ++d)
      if (g_pool[d]) RMG_CUDA_TRY(cudaMemPoolTrimTo(g_pool[d], 0));
    return RMG_OK;
  });
}
