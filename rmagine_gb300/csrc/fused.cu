// Fused simulate -> statistics: one launch casts the model scan at each
// estimated pose and reduces the ray-index correspondences with a dataset scan
// straight into CrossStatistics (and, optionally, the Umeyama transform).
//
// It replaces, per pose, the inner step of rmagine's RCC / MICP-L correction
// loop (tests/embree/correction_rcc.cpp:139-160):
//     sim.simulate(Tbm_est, model)                         // points, normals, hits
//     stats = statistics_p2l(Tpre, dataset, model, params) // statistics.cpp:84-126
//     T = umeyama_transform(stats)                         // optimization.cpp:12-49
// with the model bundle never written to memory.  Ray i of pose p pairs the
// dataset point i of the pose's scan (pre-transformed) with the model hit of
// ray i; the model side is valid when the ray hits with range >= range.min (the
// Hits attribute, the model mask of the RCC loop); the model point / normal are
// the Points / Normals attributes of the plain simulator bit for bit
// (hit_point / hit_normal in trace.cuh), and the pairing / filter arithmetic is
// that of the statistics kernels (stats.cuh).  Rays whose dataset point is
// masked out (mask == 0 or id != dataset_id) are not cast at all.
//
// Reduction: a warp casts one 32-ray tile at a time; the tile's correspondences
// are summed around the tile's first valid correspondence in binary32 (a
// 5-level butterfly), then lanes 0..15 turn the 16 sums into raw moments about
// the sensor origin in binary64 (one moment per lane) and accumulate them over
// the warp's tiles.  A CTA adds its warps in a fixed order into one partial
// record; k_fused_final adds a pose's partials in a fixed order, forms the
// means and the covariance E[m d^T] - E[m] E[d]^T and runs Umeyama in binary64.
// Deterministic; the result differs from simulate + statistics only by the
// order of the binary32/binary64 additions (n_meas is exact).
#include "internal.h"
#include "linalg.cuh"
#include "stats.cuh"
#include "trace.cuh"

namespace rmg {
namespace {

#ifndef RMG_FUSED_MIN_BLOCKS
#define RMG_FUSED_MIN_BLOCKS 5
#endif
// tiles (32 rays) each warp reduces before its CTA writes one partial record
#ifndef RMG_FUSED_TILES_PER_WARP
#define RMG_FUSED_TILES_PER_WARP 8
#endif

struct FusedParams {
  TraceParams T;
  const float* dp;        // dataset points (float3), [n_scans][width*height]
  const uint8_t* dmask;   // may be NULL
  const uint32_t* dids;   // may be NULL
  uint64_t d_stride;      // rays per scan when every pose has its own scan, else 0
  const rmg_transform* pre;
  uint32_t pre_stride;    // 1: one pre-transform per pose, 0: one for every pose
  float max_dist;
  uint32_t dataset_id;
  uint32_t ctas_per_pose;
  uint32_t tiles_per_cta;
  double* partial;        // [n_poses * ctas_per_pose][16]
};

// v[0..15] = (n, sum d', sum m', sum m' d'^T row-major) around the shift
// (sd, sm); returns, for lane k < 16, moment k about the origin in binary64:
//   n, sum d = sum d' + n sd, sum m = sum m' + n sm,
//   sum m d^T = sum m' d'^T + sm (sum d')^T + (sum m') sd^T + n sm sd^T.
__device__ __forceinline__ double raw_moment(const float v[16], uint32_t k, const V& sd, const V& sm) {
  float x = v[0];
#pragma unroll
  for (int j = 1; j < 16; ++j) x = k == (uint32_t)j ? v[j] : x;
  const double n = (double)v[0];
  if (k == 0) return n;
  if (k < 4) {
    const float s = k == 1 ? sd.x : (k == 2 ? sd.y : sd.z);
    return (double)x + n * (double)s;
  }
  if (k < 7) {
    const float s = k == 4 ? sm.x : (k == 5 ? sm.y : sm.z);
    return (double)x + n * (double)s;
  }
  const uint32_t i = (k - 7) / 3, j = (k - 7) - 3 * ((k - 7) / 3);
  const float smi = i == 0 ? sm.x : (i == 1 ? sm.y : sm.z);
  const float sdj = j == 0 ? sd.x : (j == 1 ? sd.y : sd.z);
  const float sum_dj = j == 0 ? v[1] : (j == 1 ? v[2] : v[3]);
  const float sum_mi = i == 0 ? v[4] : (i == 1 ? v[5] : v[6]);
  return (double)x + (double)smi * (double)sum_dj + (double)sum_mi * (double)sdj + n * (double)smi * (double)sdj;
}

template <bool P2L, int OK, int SS, int TB>
__global__ void __launch_bounds__(256, RMG_FUSED_MIN_BLOCKS) k_trace_stats(const FusedParams F) {
  const TraceParams& P = F.T;
  const uint32_t pose = blockIdx.x / F.ctas_per_pose;
  const uint32_t cta = blockIdx.x - pose * F.ctas_per_pose;
  const uint32_t lane = threadIdx.x & 31, wib = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const uint32_t W = P.sen.width, H = P.sen.height;
  const Tf Tsm = tmul(load_tf(P.Tbm[pose]), P.Tsb);
  const Tf pre = F.pre ? load_tf(F.pre[F.pre_stride ? pose : 0]) : Tf{Q{0.f, 0.f, 0.f, 1.f}, V{0.f, 0.f, 0.f}};
  const uint64_t dbase = (uint64_t)pose * F.d_stride;
  const uint32_t tile_w = 1u << P.tile_w_log2;
  double acc = 0.0;
  const uint32_t t0 = cta * F.tiles_per_cta;
  const uint32_t t1 = min(P.tiles_per_pose, t0 + F.tiles_per_cta);
  for (uint32_t tile = t0 + wib; tile < t1; tile += nw) {  // warp-uniform
    const uint32_t ty = tile / P.tiles_x, tx = tile - ty * P.tiles_x;
    const uint32_t vid = ty * P.tile_h + (lane >> P.tile_w_log2);
    const uint32_t hid = tx * tile_w + (lane & (tile_w - 1));
    bool ok = false;
    V D{0.f, 0.f, 0.f}, M{0.f, 0.f, 0.f};
    if (vid < H && hid < W) {
      const uint32_t loc = visit_loc(P.sen, vid * W + hid);
      const uint64_t di = dbase + loc;
      if ((!F.dmask || F.dmask[di] != 0) && (!F.dids || F.dids[di] == F.dataset_id)) {
        V dir_s, orig_s, o, d;
        setup_ray<OK>(P.sen, Tsm, loc, dir_s, orig_s, o, d);
        Hit h;
        bool over = false;
        trace_ray<SS, TB>(P.map, o, d, P.sen.range_max, P.budget, h, over);
        if (over) atomicExch(P.map.status, (unsigned)RMG_ERR_TRAVERSAL_BUDGET);
        if (h.tri >= 0 && h.t >= P.sen.range_min) {
          const V mpt = hit_point<OK>(dir_s, orig_s, h.t);
          const V npt = P2L ? hit_normal(P.map, h, dir_s, Tsm) : V{0.f, 0.f, 0.f};
          const V dpt{__ldg(F.dp + 3 * di), __ldg(F.dp + 3 * di + 1), __ldg(F.dp + 3 * di + 2)};
          D = F.pre ? tf_point(pre, dpt) : dpt;
          ok = match<P2L>(D, mpt, npt, F.max_dist, M);
        }
      }
    }
    const unsigned bal = __ballot_sync(0xffffffffu, ok);
    if (bal == 0u) continue;
    const int src = __ffs(bal) - 1;
    const V sd{__shfl_sync(0xffffffffu, D.x, src), __shfl_sync(0xffffffffu, D.y, src),
               __shfl_sync(0xffffffffu, D.z, src)};
    const V sm{__shfl_sync(0xffffffffu, M.x, src), __shfl_sync(0xffffffffu, M.y, src),
               __shfl_sync(0xffffffffu, M.z, src)};
    float v[16];
    {
      const float dx = ok ? D.x - sd.x : 0.f, dy = ok ? D.y - sd.y : 0.f, dz = ok ? D.z - sd.z : 0.f;
      const float mx = ok ? M.x - sm.x : 0.f, my = ok ? M.y - sm.y : 0.f, mz = ok ? M.z - sm.z : 0.f;
      v[0] = ok ? 1.f : 0.f;
      v[1] = dx; v[2] = dy; v[3] = dz;
      v[4] = mx; v[5] = my; v[6] = mz;
      v[7] = mx * dx; v[8] = mx * dy; v[9] = mx * dz;
      v[10] = my * dx; v[11] = my * dy; v[12] = my * dz;
      v[13] = mz * dx; v[14] = mz * dy; v[15] = mz * dz;
    }
#pragma unroll
    for (int k = 0; k < 16; ++k)
      for (int o = 16; o > 0; o >>= 1) v[k] += __shfl_xor_sync(0xffffffffu, v[k], o);
    if (lane < 16) acc += raw_moment(v, lane, sd, sm);
  }
  __shared__ double red[16][8];
  if (lane < 16) red[lane][wib] = acc;
  __syncthreads();
  if (threadIdx.x < 16) {
    double s = 0.0;
    for (uint32_t w = 0; w < nw; ++w) s += red[threadIdx.x][w];
    F.partial[16ull * blockIdx.x + threadIdx.x] = s;
  }
}

// One warp per pose: lanes 0..15 add moment k over the pose's partial records
// in order; lane 0 forms the statistics and the Umeyama transform.
__global__ void k_fused_final(const double* partial, uint32_t n_poses, uint32_t ctas, rmg_cross_stats* stats,
                              rmg_transform* transforms) {
  const uint32_t pose = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const uint32_t lane = threadIdx.x & 31;
  if (pose >= n_poses) return;
  double s = 0.0;
  if (lane < 16)
    for (uint32_t c = 0; c < ctas; ++c) s += partial[16ull * ((uint64_t)pose * ctas + c) + lane];
  double S[16];
#pragma unroll
  for (int k = 0; k < 16; ++k) S[k] = __shfl_sync(0xffffffffu, s, k);
  if (lane != 0) return;
  const double n = S[0];
  double dm[3] = {0, 0, 0}, mm[3] = {0, 0, 0}, C[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
  if (n > 0.0) {
    for (int k = 0; k < 3; ++k) { dm[k] = S[1 + k] / n; mm[k] = S[4 + k] / n; }
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) C[3 * i + j] = S[7 + 3 * i + j] / n - mm[i] * dm[j];
  }
  if (stats) store_cross_stats(n, dm, mm, C, stats + pose);
  if (transforms) {
    M3d Cm, R;
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) Cm.a[i][j] = C[3 * i + j];
    double q[4], t[3];
    umeyama_d(Cm, dm, mm, (unsigned int)n, R, q, t);
    store_tf(transforms + pose, q, t);
  }
}

// out[i] = a[i or 0] * b[i or 0] (Transform::mult, Transform.tcc:34-42), exact order.
__global__ void k_compose(const rmg_transform* a, uint32_t a_stride, const rmg_transform* b, uint32_t b_stride,
                          rmg_transform* out, uint32_t n) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const Tf r = tmul(load_tf(a[a_stride ? i : 0]), load_tf(b[b_stride ? i : 0]));
  rmg_transform T;
  T.R = rmg_quat{r.R.x, r.R.y, r.R.z, r.R.w};
  T.t = rmg_vec3{r.t.x, r.t.y, r.t.z};
  T.stamp = 0;
  out[i] = T;
}

template <bool P2L, int OK>
cudaError_t launch_fused_ok(const FusedParams& F, unsigned grid, unsigned block, cudaStream_t st) {
  if (F.T.full_stack) {
    k_trace_stats<P2L, OK, kFullStack, 0><<<grid, block, 0, st>>>(F);
    return cudaGetLastError();
  }
  switch (F.T.trail_bits) {
    case 32: k_trace_stats<P2L, OK, 16, 32><<<grid, block, 0, st>>>(F); break;
    case 64: k_trace_stats<P2L, OK, 16, 64><<<grid, block, 0, st>>>(F); break;
    default: k_trace_stats<P2L, OK, 16, 128><<<grid, block, 0, st>>>(F); break;
  }
  return cudaGetLastError();
}

template <bool P2L>
cudaError_t launch_fused(const FusedParams& F, int kind, unsigned grid, unsigned block, cudaStream_t st) {
  switch (kind) {
    case RMG_MODEL_SPHERICAL:
    case RMG_MODEL_PINHOLE: return launch_fused_ok<P2L, ORIGIN_POSE>(F, grid, block, st);
    case RMG_MODEL_O1DN: return launch_fused_ok<P2L, ORIGIN_SINGLE>(F, grid, block, st);
    default: return launch_fused_ok<P2L, ORIGIN_TABLE>(F, grid, block, st);
  }
}

}  // namespace

int default_config(const rmg_sensor* s, rmg_launch_config* cfg);
int make_trace_params(const rmg_map* map, const rmg_sensor* sensor, const rmg_transform* Tsb,
                      const rmg_transform* Tbm, uint32_t n_poses, const rmg_outputs* out,
                      const rmg_launch_config& cfg, TraceParams& P);

}  // namespace rmg

using namespace rmg;

extern "C" int rmg_simulate_statistics(const rmg_map* map, const rmg_sensor* sensor, const rmg_transform* Tsb,
                                       const rmg_transform* Tbm, uint32_t n_poses, const rmg_scan* dataset,
                                       const rmg_transform* pre_transforms, uint32_t pre_transform_stride,
                                       const rmg_umeyama_constraints* params, int point_to_plane,
                                       rmg_cross_stats* stats, rmg_transform* transforms, void* stream) {
  return guarded("rmg_simulate_statistics", [&]() -> int {
    if (!map || !sensor || !Tsb || !dataset || !params)
      return fail(RMG_ERR_INVALID_ARG, "rmg_simulate_statistics: NULL map, sensor, Tsb, dataset or params");
    if (n_poses == 0) return RMG_OK;
    if (!Tbm || !dataset->points) return fail(RMG_ERR_INVALID_ARG, "rmg_simulate_statistics: NULL Tbm or dataset points");
    if (!stats && !transforms) return fail(RMG_ERR_INVALID_ARG, "rmg_simulate_statistics: no output requested");
    rmg_launch_config cfg;
    default_config(sensor, &cfg);
    rmg_outputs out{};
    FusedParams F;
    make_trace_params(map, sensor, Tsb, Tbm, n_poses, &out, cfg, F.T);
    F.dp = reinterpret_cast<const float*>(dataset->points);
    F.dmask = dataset->mask;
    F.dids = dataset->ids;
    F.d_stride = dataset->per_pose ? (uint64_t)sensor->width * sensor->height : 0ull;
    F.pre = pre_transforms;
    F.pre_stride = pre_transform_stride ? 1u : 0u;
    F.max_dist = params->max_dist;
    F.dataset_id = params->dataset_id;
    F.tiles_per_cta = cfg.block_warps * RMG_FUSED_TILES_PER_WARP;
    F.ctas_per_pose = (F.T.tiles_per_pose + F.tiles_per_cta - 1) / F.tiles_per_cta;
    const uint64_t grid = (uint64_t)F.ctas_per_pose * n_poses;
    if (grid > 0x7fffffffull) return fail(RMG_ERR_INVALID_ARG, "rmg_simulate_statistics: too many rays for one launch");
    cudaStream_t st = as_stream(stream);
    double* partial = nullptr;
    RMG_CUDA_TRY(cudaMallocAsync(reinterpret_cast<void**>(&partial), 16 * sizeof(double) * (size_t)grid, st));
    F.partial = partial;
    const unsigned block = 32u * cfg.block_warps;
    const cudaError_t e = point_to_plane ? launch_fused<true>(F, sensor->model.kind, (unsigned)grid, block, st)
                                         : launch_fused<false>(F, sensor->model.kind, (unsigned)grid, block, st);
    int s = cuda_status(e, "k_trace_stats");
    if (s == RMG_OK) {
      const uint64_t threads = 32ull * n_poses;
      k_fused_final<<<(unsigned)((threads + 127) / 128), 128, 0, st>>>(partial, n_poses, F.ctas_per_pose, stats,
                                                                       transforms);
      s = cuda_status(cudaGetLastError(), "k_fused_final");
    }
    cudaFreeAsync(partial, st);
    return s;
  });
}

extern "C" int rmg_transforms_compose(const rmg_transform* a, uint32_t a_stride, const rmg_transform* b,
                                      uint32_t b_stride, rmg_transform* out, uint32_t n, void* stream) {
  return guarded("rmg_transforms_compose", [&]() -> int {
    if (n == 0) return RMG_OK;
    if (!a || !b || !out) return fail(RMG_ERR_INVALID_ARG, "rmg_transforms_compose: NULL argument");
    k_compose<<<(n + 255) / 256, 256, 0, as_stream(stream)>>>(a, a_stride, b, b_stride, out, n);
    return cuda_status(cudaGetLastError(), "k_compose");
  });
}
