// Range adjoint: dL/d(6-DoF pose) of a Huber range loss, fused with the
// forward ray cast.  No counterpart in the reference (rmagine has no
// differentiable simulator); it differentiates the range r = n.(p0 - o)/(n.d)
// of the hit triangle.
//
// Pose parameterisation: right perturbation T_bm * exp(xi^), xi = (rho, omega)
// (translation first), the convention of rmagine's lie.h:57-114.  In the base
// frame, with d_b = R_sb d_s, o_b = t_sb + R_sb o_s, n_b = R_bm^T n (face
// normal), p_b = o_b + r d_b and b = n_b . d_b:
//     dr/drho   = -n_b / b
//     dr/domega = -(p_b x n_b) / b
// (the scale of n cancels, so the unnormalised cross product of two edges is
// used).  Loss per ray: Huber_delta(r_sim - r_obs) over rays whose simulated
// hit has range.min <= t and whose observation lies in [range.min, range.max];
// dL/dxi = sum psi(e) dr/dxi, psi = clamp(e, -delta, delta).
//
// One CTA covers block_warps ray tiles of ONE pose (grid: tiles x poses); it
// reduces its rays' 7 values (6 gradient components + loss) with warp
// shuffles and shared memory into one partial record; a second kernel sums a
// pose's partials in a fixed order in binary64.  Deterministic.
#include "internal.h"
#include "launch.h"
#include "trace.cuh"

namespace rmg {
namespace {

struct GradParams {
  TraceParams T;
  const float* r_obs;
  float delta;
  float* partial;         // [n_poses][warps_per_pose][8]: one slot per warp (tile), written without a barrier
  uint32_t warps_per_pose;
};

#ifndef RMG_GRAD_MIN_BLOCKS
#define RMG_GRAD_MIN_BLOCKS 5
#endif

template <int OK, int SS, int TB>
__global__ void __launch_bounds__(256, RMG_GRAD_MIN_BLOCKS) k_range_grad(const GradParams G) {
  const TraceParams& P = G.T;
  const uint32_t pose = blockIdx.y;
  const uint32_t lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const uint32_t tile = blockIdx.x * (blockDim.x >> 5) + wib;
  float acc[7] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
  if (tile < P.tiles_per_pose) {
    const uint32_t ty = tile / P.tiles_x, tx = tile - ty * P.tiles_x;
    const uint32_t tile_w = 1u << P.tile_w_log2;
    const uint32_t vid = ty * P.tile_h + (lane >> P.tile_w_log2);
    const uint32_t hid = tx * tile_w + (lane & (tile_w - 1));
    const uint32_t W = P.sen.width, H = P.sen.height;
    if (vid < H && hid < W) {
      const uint32_t loc = visit_loc(P.sen, vid * W + hid);
      const uint64_t gid = (uint64_t)pose * W * H + loc;
      const Tf Tbm = load_tf(P.Tbm[pose]);
      const Tf Tsm = tmul(Tbm, P.Tsb);
      V dir_s, orig_s, o, d;
      setup_ray<OK>(P.sen, Tsm, loc, dir_s, orig_s, o, d);
      Hit h;
      bool over = false;
      trace_ray<SS, TB>(P.map, o, d, P.sen.range_max, P.budget, h, over);
      if (over) atomicExch(P.map.status, (unsigned)RMG_ERR_TRAVERSAL_BUDGET);
      if (P.out.ranges) P.out.ranges[gid] = h.tri >= 0 ? h.t : add(P.sen.range_max, 1.0f);
      if (P.out.face_ids) P.out.face_ids[gid] = h.tri >= 0 ? h.face : 0xffffffffu;
      const float obs = __ldg(G.r_obs + gid);
      const float rmin = P.sen.range_min, rmax = P.sen.range_max;
      if (h.tri >= 0 && h.t >= rmin && obs >= rmin && obs <= rmax) {
        const float e = h.t - obs;
        const float ae = fabsf(e);
        const float psi = fminf(fmaxf(e, -G.delta), G.delta);
        const float loss = ae <= G.delta ? 0.5f * e * e : G.delta * (ae - 0.5f * G.delta);
        const Tri* tp = P.map.tris + h.tri;
        const float4 p0 = __ldg(&tp->v0), p1 = __ldg(&tp->v1), p2 = __ldg(&tp->v2);
        const float e1x = p1.x - p0.x, e1y = p1.y - p0.y, e1z = p1.z - p0.z;
        const float e2x = p2.x - p0.x, e2y = p2.y - p0.y, e2z = p2.z - p0.z;
        const V nm{e1y * e2z - e1z * e2y, e1z * e2x - e1x * e2z, e1x * e2y - e1y * e2x};
        const V nb = qrot(qconj(Tbm.R), nm);
        const V db = qrot(P.Tsb.R, dir_s);
        V ob = P.Tsb.t;
        if (OK != ORIGIN_POSE) {
          const V r = qrot(P.Tsb.R, orig_s);
          ob = V{ob.x + r.x, ob.y + r.y, ob.z + r.z};
        }
        const float b = nb.x * db.x + nb.y * db.y + nb.z * db.z;
        if (fabsf(b) > 1e-30f) {
          const float s = -psi / b;
          const V pb{ob.x + h.t * db.x, ob.y + h.t * db.y, ob.z + h.t * db.z};
          acc[0] = s * nb.x;
          acc[1] = s * nb.y;
          acc[2] = s * nb.z;
          acc[3] = s * (pb.y * nb.z - pb.z * nb.y);
          acc[4] = s * (pb.z * nb.x - pb.x * nb.z);
          acc[5] = s * (pb.x * nb.y - pb.y * nb.x);
          acc[6] = loss;
        }
      }
    }
  }
#pragma unroll
  for (int k = 0; k < 7; ++k)
    for (int off = 16; off > 0; off >>= 1) acc[k] += __shfl_xor_sync(0xffffffffu, acc[k], off);
  // Each warp stores its sums in its own slot (no barrier: a warp whose rays end
  // early retires at once instead of waiting for the CTA's slowest warp).
  if (lane == 0) {
    float4* slot = reinterpret_cast<float4*>(
        G.partial + 8ull * ((uint64_t)pose * G.warps_per_pose + (uint64_t)blockIdx.x * (blockDim.x >> 5) + wib));
    slot[0] = make_float4(acc[0], acc[1], acc[2], acc[3]);
    slot[1] = make_float4(acc[4], acc[5], acc[6], 0.0f);
  }
}

// Per pose and component, the warps' sums in slot order in binary64 (a fixed
// order: the result does not depend on scheduling).
__global__ void k_grad_final(const float* partial, uint32_t n_poses, uint32_t warps, float* grad, float* loss) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= 7u * n_poses) return;
  const uint32_t pose = i / 7, k = i - pose * 7;
  double s = 0.0;
  for (uint32_t c = 0; c < warps; ++c) s += partial[8ull * ((uint64_t)pose * warps + c) + k];
  if (k < 6) {
    if (grad) grad[6ull * pose + k] = (float)s;
  } else if (loss) {
    loss[pose] = (float)s;
  }
}

template <int OK, int SS>
cudaError_t launch_grad_tb(const GradParams& G, dim3 grid, unsigned block, cudaStream_t st) {
  if (G.T.full_stack) {
    k_range_grad<OK, kFullStack, 0><<<grid, block, 0, st>>>(G);
    return cudaGetLastError();
  }
  switch (G.T.trail_bits) {
    case 32: k_range_grad<OK, SS, 32><<<grid, block, 0, st>>>(G); break;
    case 64: k_range_grad<OK, SS, 64><<<grid, block, 0, st>>>(G); break;
    default: k_range_grad<OK, SS, 128><<<grid, block, 0, st>>>(G); break;
  }
  return cudaGetLastError();
}

template <int OK>
cudaError_t launch_grad(const GradParams& G, int ss, dim3 grid, unsigned block, cudaStream_t st) {
  switch (ss) {
    case 8: return launch_grad_tb<OK, 8>(G, grid, block, st);
    case 16: return launch_grad_tb<OK, 16>(G, grid, block, st);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace

int default_config(const rmg_sensor* s, rmg_launch_config* cfg);
int check_config(const rmg_launch_config& c);
int make_trace_params(const rmg_map* map, const rmg_sensor* sensor, const rmg_transform* Tsb,
                      const rmg_transform* Tbm, uint32_t n_poses, const rmg_outputs* out,
                      const rmg_launch_config& cfg, TraceParams& P);

}  // namespace rmg

using namespace rmg;

extern "C" int rmg_range_pose_grad(const rmg_map* map, const rmg_sensor* sensor, const rmg_transform* Tsb,
                                   const rmg_transform* Tbm, uint32_t n_poses, const float* ranges_obs,
                                   float huber_delta, float* grad, float* loss, float* ranges_sim,
                                   uint32_t* face_ids, void* stream) {
  return guarded("rmg_range_pose_grad", [&]() -> int {
    if (!map || !sensor || !Tsb) return fail(RMG_ERR_INVALID_ARG, "rmg_range_pose_grad: NULL map, sensor or Tsb");
    if (n_poses == 0) return RMG_OK;
    if (!Tbm || !ranges_obs) return fail(RMG_ERR_INVALID_ARG, "rmg_range_pose_grad: NULL Tbm or ranges_obs");
    if (!grad && !loss) return fail(RMG_ERR_INVALID_ARG, "rmg_range_pose_grad: no output requested");
    if (!(huber_delta > 0.0f)) return fail(RMG_ERR_INVALID_ARG, "rmg_range_pose_grad: huber_delta must be > 0");
    if (n_poses > 65535u) return fail(RMG_ERR_INVALID_ARG, "rmg_range_pose_grad: at most 65535 poses per call");
    rmg_launch_config cfg;
    default_config(sensor, &cfg);
    rmg_outputs out{};
    out.ranges = ranges_sim;
    out.face_ids = face_ids;
    GradParams G;
    make_trace_params(map, sensor, Tsb, Tbm, n_poses, &out, cfg, G.T);
    G.r_obs = ranges_obs;
    G.delta = huber_delta;
    const uint32_t ctas_per_pose = (G.T.tiles_per_pose + cfg.block_warps - 1) / cfg.block_warps;
    G.warps_per_pose = ctas_per_pose * cfg.block_warps;
    cudaStream_t st = as_stream(stream);
    float* partial = nullptr;
    RMG_CUDA_TRY(cudaMallocAsync(reinterpret_cast<void**>(&partial),
                                 8 * sizeof(float) * (size_t)n_poses * G.warps_per_pose, st));
    G.partial = partial;
    const dim3 grid(ctas_per_pose, n_poses);
    const unsigned block = 32u * cfg.block_warps;
    cudaError_t e;
    switch (sensor->model.kind) {
      case RMG_MODEL_SPHERICAL:
      case RMG_MODEL_PINHOLE: e = launch_grad<ORIGIN_POSE>(G, (int)cfg.stack_depth, grid, block, st); break;
      case RMG_MODEL_O1DN: e = launch_grad<ORIGIN_SINGLE>(G, (int)cfg.stack_depth, grid, block, st); break;
      default: e = launch_grad<ORIGIN_TABLE>(G, (int)cfg.stack_depth, grid, block, st); break;
    }
    int s = cuda_status(e, "k_range_grad");
    if (s == RMG_OK) {
      k_grad_final<<<(7 * n_poses + 255) / 256, 256, 0, st>>>(partial, n_poses, G.warps_per_pose, grad, loss);
      s = cuda_status(cudaGetLastError(), "k_grad_final");
    }
    cudaFreeAsync(partial, st);
    return s;
  });
}
