// Batched CrossStatistics (point-to-point and point-to-plane), Umeyama, and the
// Umeyama backward.
//
// Replaces rmagine's statistics_p2p / statistics_p2l (CPU
// src/rmagine_core/src/math/statistics.cpp:19-126, GPU
// src/rmagine_cuda/src/math/statistics.cu:58-160, 190-276) and the batched
// umeyama_transform (src/rmagine_cuda/src/math/memory_math.cu:1627-1708).
//
// Layout: batch b owns correspondences [b*n_per, (b+1)*n_per) of the
// dataset/model arrays (float3, 12 B each).  One or more CTAs reduce a batch.
// Each thread accumulates, around a per-batch shift (the batch's first
// pre-transformed dataset point and first model point), binary32 sums of
// d', m' and m' d'^T over runs of at most 32 correspondences; the warp sums its
// 32 runs pairwise in binary32 and folds the result into binary64 accumulators
// (one lane, one fold per 1024 correspondences); the CTA combines in binary64, and
// batches split over several CTAs are combined in a fixed order by the last
// CTA to finish, so results are deterministic.  The mean and covariance are
// formed in binary64 (cov = E[m' d'^T] - E[m'] E[d']^T), then rounded to the
// binary32 CrossStatistics record.  Umeyama runs in binary64 (linalg.cuh).
//
// Filters follow the reference GPU kernels: mask > 0, ids equal to the
// constraint ids, and ||M - D||^2 < max_dist^2 (p2p) or
// |(I - D) . N| < max_dist (p2l, with M = D + N ((I - D) . N)).
#include <algorithm>

#include "internal.h"
#include "linalg.cuh"
#include "stats.cuh"

namespace rmg {
namespace {

constexpr int kStatsThreads = 256;
constexpr int kFold = 8;  // vector groups (4 correspondences) per binary32 run

struct StatsParams {
  const rmg_transform* pre;
  uint32_t pre_stride;
  const float* dp;
  const uint8_t* dmask;
  const uint32_t* dids;
  const float* mp;
  const float* mn;  // model normals (p2l)
  const uint8_t* mmask;
  const uint32_t* mids;
  float max_dist;
  uint32_t dataset_id, model_id;
  uint32_t n_batches;
  uint32_t n_per;
  uint32_t chunks;     // CTAs per batch
  uint32_t chunk_len;  // correspondences per CTA (multiple of 4)
  double* partial;     // [n_batches * chunks][16] (chunks > 1)
  unsigned int* counters;  // [n_batches] (chunks > 1)
  double* dstats;      // [n_batches][16]: d mean, m mean, C (row-major), n  (may be NULL)
  rmg_cross_stats* stats;  // may be NULL
};

__device__ __forceinline__ Tf batch_pre(const StatsParams& P, uint32_t b) {
  if (!P.pre) return Tf{Q{0.f, 0.f, 0.f, 1.f}, V{0.f, 0.f, 0.f}};
  return load_tf(P.pre[P.pre_stride ? b : 0]);
}

// PRE = false: no pre-transform (rotating by the identity quaternion is exact, so
// skipping it changes no bit).
template <bool P2L, bool PRE = true>
__device__ __forceinline__ bool correspondence(const StatsParams& P, const Tf& pre, uint64_t i, const V& dpt,
                                               const V& mpt, const V& npt, V& D, V& M) {
  if (P.dmask && P.dmask[i] == 0) return false;
  if (P.mmask && P.mmask[i] == 0) return false;
  if (P.dids && P.dids[i] != P.dataset_id) return false;
  if (P.mids && P.mids[i] != P.model_id) return false;
  D = PRE ? tf_point(pre, dpt) : dpt;
  return match<P2L>(D, mpt, npt, P.max_dist, M);
}

struct FAcc {
  float n, d[3], m[3], md[9];
  __device__ __forceinline__ void zero() {
    n = 0.f;
    for (int k = 0; k < 3; ++k) { d[k] = 0.f; m[k] = 0.f; }
    for (int k = 0; k < 9; ++k) md[k] = 0.f;
  }
  __device__ __forceinline__ void add_pt(const V& D, const V& M, const V& sd, const V& sm) {
    const float dx = D.x - sd.x, dy = D.y - sd.y, dz = D.z - sd.z;
    const float mx = M.x - sm.x, my = M.y - sm.y, mz = M.z - sm.z;
    n += 1.f;
    d[0] += dx; d[1] += dy; d[2] += dz;
    m[0] += mx; m[1] += my; m[2] += mz;
    md[0] = fmaf(mx, dx, md[0]); md[1] = fmaf(mx, dy, md[1]); md[2] = fmaf(mx, dz, md[2]);
    md[3] = fmaf(my, dx, md[3]); md[4] = fmaf(my, dy, md[4]); md[5] = fmaf(my, dz, md[5]);
    md[6] = fmaf(mz, dx, md[6]); md[7] = fmaf(mz, dy, md[7]); md[8] = fmaf(mz, dz, md[8]);
  }
};

// Folding a binary32 run into binary64: the 32 lanes' runs are first summed
// pairwise across the warp in binary32 (a 5-level butterfly), then ONE lane
// adds the 16 warp sums to the warp's binary64 accumulators in shared memory.
// The GB300's binary64 pipe is narrow; this keeps it at 16 operations per 1024
// correspondences instead of 16 per 32.  All lanes must call fold together.
__device__ __forceinline__ void fold(double (*acc)[kStatsThreads / 32], FAcc& f) {
  float v[16] = {f.n, f.d[0], f.d[1], f.d[2], f.m[0], f.m[1], f.m[2], f.md[0], f.md[1], f.md[2],
                 f.md[3], f.md[4], f.md[5], f.md[6], f.md[7], f.md[8]};
#pragma unroll
  for (int k = 0; k < 16; ++k)
    for (int o = 16; o > 0; o >>= 1) v[k] += __shfl_xor_sync(0xffffffffu, v[k], o);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane < 16) {
    float x = v[0];
#pragma unroll
    for (int k = 1; k < 16; ++k) x = lane == k ? v[k] : x;
    acc[lane][warp] += (double)x;
  }
  f.zero();
}

__device__ __forceinline__ V ldv(const float* p, uint64_t i) {
  return V{__ldg(p + 3 * i), __ldg(p + 3 * i + 1), __ldg(p + 3 * i + 2)};
}

__device__ void finalize(const StatsParams& P, uint32_t b, const double* acc, const V& sd, const V& sm) {
  const double n = acc[0];
  double dm[3] = {0, 0, 0}, mm[3] = {0, 0, 0}, C[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
  if (n > 0.0) {
    const double ds[3] = {acc[1] / n, acc[2] / n, acc[3] / n};
    const double ms[3] = {acc[4] / n, acc[5] / n, acc[6] / n};
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) C[3 * i + j] = acc[7 + 3 * i + j] / n - ms[i] * ds[j];
    dm[0] = (double)sd.x + ds[0]; dm[1] = (double)sd.y + ds[1]; dm[2] = (double)sd.z + ds[2];
    mm[0] = (double)sm.x + ms[0]; mm[1] = (double)sm.y + ms[1]; mm[2] = (double)sm.z + ms[2];
  }
  if (P.stats) store_cross_stats(n, dm, mm, C, P.stats + b);
  if (P.dstats) {
    double* o = P.dstats + 16ull * b;
    for (int k = 0; k < 3; ++k) { o[k] = dm[k]; o[3 + k] = mm[k]; }
    for (int k = 0; k < 9; ++k) o[6 + k] = C[k];
    o[15] = n;
  }
}

template <bool P2L, bool VEC, bool PRE>
__global__ void __launch_bounds__(kStatsThreads, 3) k_stats(const StatsParams P) {
  const uint32_t b = blockIdx.x / P.chunks;
  const uint32_t c = blockIdx.x - b * P.chunks;
  const uint64_t base = (uint64_t)b * P.n_per;
  const uint32_t lo = c * P.chunk_len;
  const uint32_t hi = min(P.n_per, lo + P.chunk_len);
  const Tf pre = batch_pre(P, b);
  // per-batch shift: first correspondence of the batch (any value works; it only
  // keeps the binary32 partial sums small)
  const V sd = P.n_per ? tf_point(pre, ldv(P.dp, base)) : V{0, 0, 0};
  const V sm = P.n_per ? ldv(P.mp, base) : V{0, 0, 0};

  __shared__ double acc[16][kStatsThreads / 32];
  if (threadIdx.x < 16 * (kStatsThreads / 32)) acc[threadIdx.x / (kStatsThreads / 32)][threadIdx.x % (kStatsThreads / 32)] = 0.0;
  __syncthreads();
  FAcc f;
  f.zero();
  const V zero{0.f, 0.f, 0.f};
  if (VEC) {
    // thread t takes groups of 4 consecutive correspondences: 3 x 16-byte loads per array
    const uint32_t g0 = lo / 4, g1 = (hi + 3) / 4;
    int run = 0;
    // warp-uniform trip count (lanes past the end skip the loads)
    const uint32_t iters = (g1 - g0 + blockDim.x - 1) / blockDim.x;
    for (uint32_t it = 0; it < iters; ++it) {
      const uint32_t g = g0 + threadIdx.x + it * blockDim.x;
      if (g < g1) {
      const uint64_t e = base + 4ull * g;
      const float4* dv = reinterpret_cast<const float4*>(P.dp + 3 * e);
      const float4* mv = reinterpret_cast<const float4*>(P.mp + 3 * e);
      float dd[12], mmv[12], nn[12];
      *reinterpret_cast<float4*>(dd + 0) = __ldg(dv + 0);
      *reinterpret_cast<float4*>(dd + 4) = __ldg(dv + 1);
      *reinterpret_cast<float4*>(dd + 8) = __ldg(dv + 2);
      *reinterpret_cast<float4*>(mmv + 0) = __ldg(mv + 0);
      *reinterpret_cast<float4*>(mmv + 4) = __ldg(mv + 1);
      *reinterpret_cast<float4*>(mmv + 8) = __ldg(mv + 2);
      if (P2L) {
        const float4* nv = reinterpret_cast<const float4*>(P.mn + 3 * e);
        *reinterpret_cast<float4*>(nn + 0) = __ldg(nv + 0);
        *reinterpret_cast<float4*>(nn + 4) = __ldg(nv + 1);
        *reinterpret_cast<float4*>(nn + 8) = __ldg(nv + 2);
      }
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        const uint32_t j = 4 * g + k;
        if (j < lo || j >= hi) continue;
        V D, M;
        const V np = P2L ? V{nn[3 * k], nn[3 * k + 1], nn[3 * k + 2]} : zero;
        if (correspondence<P2L, PRE>(P, pre, base + j, V{dd[3 * k], dd[3 * k + 1], dd[3 * k + 2]},
                                V{mmv[3 * k], mmv[3 * k + 1], mmv[3 * k + 2]}, np, D, M))
          f.add_pt(D, M, sd, sm);
      }
      }
      if (++run == kFold) { fold(acc, f); run = 0; }
    }
  } else {
    int run = 0;
    const uint32_t iters = (hi - lo + blockDim.x - 1) / blockDim.x;
    for (uint32_t it = 0; it < iters; ++it) {
      const uint32_t j = lo + threadIdx.x + it * blockDim.x;
      if (j < hi) {
        V D, M;
        const V np = P2L ? ldv(P.mn, base + j) : zero;
        if (correspondence<P2L, PRE>(P, pre, base + j, ldv(P.dp, base + j), ldv(P.mp, base + j), np, D, M))
          f.add_pt(D, M, sd, sm);
      }
      if (++run == 4 * kFold) { fold(acc, f); run = 0; }
    }
  }
  fold(acc, f);

  // CTA reduction in binary64: warp accumulators in a fixed order
  __syncthreads();
  if (threadIdx.x >= 16) return;
  double v = 0.0;
  for (int w = 0; w < kStatsThreads / 32; ++w) v += acc[threadIdx.x][w];
  __shared__ double tot[16];
  __shared__ bool last;
  tot[threadIdx.x] = v;
  if (P.chunks == 1) {
    __syncwarp(0xffffu);
    if (threadIdx.x == 0) finalize(P, b, tot, sd, sm);
    return;
  }
  P.partial[16ull * blockIdx.x + threadIdx.x] = v;
  __threadfence();
  __syncwarp(0xffffu);
  if (threadIdx.x == 0) last = atomicAdd(&P.counters[b], 1u) == P.chunks - 1;
  __syncwarp(0xffffu);
  if (!last) return;
  __threadfence();
  double s = 0.0;
  for (uint32_t k = 0; k < P.chunks; ++k) s += __ldcg(&P.partial[16ull * (b * P.chunks + k) + threadIdx.x]);
  tot[threadIdx.x] = s;
  __syncwarp(0xffffu);
  if (threadIdx.x == 0) finalize(P, b, tot, sd, sm);
}

__global__ void k_umeyama_dstats(const double* dstats, uint32_t n, rmg_transform* out) {
  const uint32_t b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= n) return;
  const double* s = dstats + 16ull * b;
  M3d C;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) C.a[i][j] = s[6 + 3 * i + j];
  M3d R;
  double q[4], t[3];
  umeyama_d(C, s, s + 3, (unsigned int)s[15], R, q, t);
  store_tf(out + b, q, t);
}

__device__ __forceinline__ void load_stats(const rmg_cross_stats& s, M3d& C, double d[3], double m[3]) {
  d[0] = s.dataset_mean.x; d[1] = s.dataset_mean.y; d[2] = s.dataset_mean.z;
  m[0] = s.model_mean.x; m[1] = s.model_mean.y; m[2] = s.model_mean.z;
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c) C.a[r][c] = s.covariance.data[3 * c + r];
}

__global__ void k_umeyama_stats(const rmg_cross_stats* stats, uint32_t n, rmg_transform* out) {
  const uint32_t b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= n) return;
  const rmg_cross_stats s = stats[b];
  M3d C, R;
  double d[3], m[3], q[4], t[3];
  load_stats(s, C, d, m);
  umeyama_d(C, d, m, s.n_meas, R, q, t);
  store_tf(out + b, q, t);
}

// ---- backward --------------------------------------------------------------------
// Per batch: coefficients of the affine per-correspondence gradients
//   dL/dM_i = A D_i + cm,   dL/dD_i = B M_i + cd
// with A = G_C / n, B = G_C^T / n, cm = g_t/n - A d_mean,
// cd = -R^T g_t / n - B m_mean, G_C = rotation_backward(dL/dR - g_t d_mean^T).
struct Coef { float A[9], cm[3], B[9], cd[3]; };

__global__ void k_umeyama_bwd_coef(const rmg_cross_stats* stats, const float* grad_R, const float* grad_t,
                                   uint32_t n_batches, Coef* coef) {
  const uint32_t b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= n_batches) return;
  const rmg_cross_stats s = stats[b];
  Coef c;
  for (int k = 0; k < 9; ++k) { c.A[k] = 0.f; c.B[k] = 0.f; }
  for (int k = 0; k < 3; ++k) { c.cm[k] = 0.f; c.cd[k] = 0.f; }
  if (s.n_meas > 0) {
    M3d C, U, V;
    double d[3], m[3], sv[3];
    load_stats(s, C, d, m);
    svd3_rot(C, U, sv, V);
    const M3d R = m3_mul_nt(U, V);
    double gt[3] = {0, 0, 0};
    if (grad_t)
      for (int k = 0; k < 3; ++k) gt[k] = grad_t[3ull * b + k];
    M3d gR;
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) gR.a[i][j] = (grad_R ? (double)grad_R[9ull * b + 3 * i + j] : 0.0) - gt[i] * d[j];
    const M3d GC = rotation_backward(U, sv, V, gR);
    const double n = (double)s.n_meas;
    double A[3][3], B[3][3];
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) { A[i][j] = GC.a[i][j] / n; B[i][j] = GC.a[j][i] / n; }
    double gd[3];
    for (int i = 0; i < 3; ++i) gd[i] = -(R.a[0][i] * gt[0] + R.a[1][i] * gt[1] + R.a[2][i] * gt[2]);
    bool finite = true;
    for (int i = 0; i < 3; ++i) {
      c.cm[i] = (float)(gt[i] / n - (A[i][0] * d[0] + A[i][1] * d[1] + A[i][2] * d[2]));
      c.cd[i] = (float)(gd[i] / n - (B[i][0] * m[0] + B[i][1] * m[1] + B[i][2] * m[2]));
      for (int j = 0; j < 3; ++j) {
        c.A[3 * i + j] = (float)A[i][j];
        c.B[3 * i + j] = (float)B[i][j];
        finite = finite && isfinite(A[i][j]);
      }
    }
    if (!finite) {  // the forward fell back to the identity: no gradient flows
      for (int k = 0; k < 9; ++k) { c.A[k] = 0.f; c.B[k] = 0.f; }
      for (int k = 0; k < 3; ++k) { c.cm[k] = 0.f; c.cd[k] = 0.f; }
    }
  }
  coef[b] = c;
}

struct BwdParams {
  StatsParams S;
  const Coef* coef;
  float* gd;  // dL/d(dataset point), 3 per correspondence (may be NULL)
  float* gm;  // dL/d(model point)
};

__global__ void __launch_bounds__(kStatsThreads) k_umeyama_bwd_stream(const BwdParams B) {
  const StatsParams& P = B.S;
  const uint32_t b = blockIdx.x / P.chunks;
  const uint32_t c = blockIdx.x - b * P.chunks;
  const uint64_t base = (uint64_t)b * P.n_per;
  const uint32_t lo = c * P.chunk_len;
  const uint32_t hi = min(P.n_per, lo + P.chunk_len);
  const Tf pre = batch_pre(P, b);
  const Q preinv = qconj(pre.R);
  __shared__ Coef cf;
  if (threadIdx.x == 0) cf = B.coef[b];
  __syncthreads();
  const V zero{0.f, 0.f, 0.f};
  for (uint32_t j = lo + threadIdx.x; j < hi; j += blockDim.x) {
    const uint64_t i = base + j;
    V D, M;
    const bool ok = correspondence<false>(P, pre, i, ldv(P.dp, i), ldv(P.mp, i), zero, D, M);
    float gm[3] = {0.f, 0.f, 0.f}, gdv[3] = {0.f, 0.f, 0.f};
    if (ok) {
      const float Dv[3] = {D.x, D.y, D.z}, Mv[3] = {M.x, M.y, M.z};
      float gD[3];
      for (int r = 0; r < 3; ++r) {
        gm[r] = cf.cm[r] + cf.A[3 * r] * Dv[0] + cf.A[3 * r + 1] * Dv[1] + cf.A[3 * r + 2] * Dv[2];
        gD[r] = cf.cd[r] + cf.B[3 * r] * Mv[0] + cf.B[3 * r + 1] * Mv[1] + cf.B[3 * r + 2] * Mv[2];
      }
      const V g = qrot(preinv, V{gD[0], gD[1], gD[2]});  // dataset point = R_pre^T dL/dD
      gdv[0] = g.x; gdv[1] = g.y; gdv[2] = g.z;
    }
    if (B.gm) { B.gm[3 * i] = gm[0]; B.gm[3 * i + 1] = gm[1]; B.gm[3 * i + 2] = gm[2]; }
    if (B.gd) { B.gd[3 * i] = gdv[0]; B.gd[3 * i + 1] = gdv[1]; B.gd[3 * i + 2] = gdv[2]; }
  }
}

int fill_params(const rmg_transform* pre, uint32_t pre_stride, const rmg_vec3* dp, const uint8_t* dmask,
                const uint32_t* dids, const rmg_vec3* mp, const rmg_vec3* mn, const uint8_t* mmask,
                const uint32_t* mids, const rmg_umeyama_constraints* params, uint32_t n_batches, uint32_t n_per,
                StatsParams& P) {
  if (!dp || !mp || !params) return fail(RMG_ERR_INVALID_ARG, "statistics: NULL points or params");
  P.pre = pre;
  P.pre_stride = pre_stride ? 1u : 0u;
  P.dp = reinterpret_cast<const float*>(dp);
  P.dmask = dmask;
  P.dids = dids;
  P.mp = reinterpret_cast<const float*>(mp);
  P.mn = reinterpret_cast<const float*>(mn);
  P.mmask = mmask;
  P.mids = mids;
  P.max_dist = params->max_dist;
  P.dataset_id = params->dataset_id;
  P.model_id = params->model_id;
  P.n_batches = n_batches;
  P.n_per = n_per;
  // CTAs per batch: enough CTAs to fill the GPU, chunks of >= 4096 correspondences
  const uint32_t target = 8u * (uint32_t)device_sm_count();
  uint32_t chunks = 1;
  if (n_batches < target && n_per > 8192) {
    chunks = std::min<uint32_t>((target + n_batches - 1) / n_batches, (n_per + 4095) / 4096);
    chunks = std::max<uint32_t>(chunks, 1);
  }
  P.chunks = chunks;
  P.chunk_len = ((n_per + chunks - 1) / chunks + 3) & ~3u;
  P.partial = nullptr;
  P.counters = nullptr;
  P.dstats = nullptr;
  P.stats = nullptr;
  if ((uint64_t)n_batches * chunks > 0x7fffffffull) return fail(RMG_ERR_INVALID_ARG, "statistics: too many batches");
  return RMG_OK;
}

bool vec_ok(const StatsParams& P, bool p2l) {
  auto al = [](const void* p, uintptr_t a) { return p == nullptr || (reinterpret_cast<uintptr_t>(p) % a) == 0; };
  return (P.n_per % 4 == 0) && al(P.dp, 16) && al(P.mp, 16) && (!p2l || al(P.mn, 16));
}

int launch_stats(StatsParams& P, bool p2l, cudaStream_t st) {
  const unsigned grid = P.n_batches * P.chunks;
  void* scratch = nullptr;
  if (P.chunks > 1) {
    const size_t bytes = 16 * sizeof(double) * (size_t)grid + 4 * (size_t)P.n_batches;
    RMG_CUDA_TRY(cudaMallocAsync(&scratch, bytes, st));
    P.partial = static_cast<double*>(scratch);
    P.counters = reinterpret_cast<unsigned int*>(P.partial + 16ull * grid);
    RMG_CUDA_TRY(cudaMemsetAsync(P.counters, 0, 4 * (size_t)P.n_batches, st));
  }
  const bool vec = vec_ok(P, p2l);
  const int variant = (p2l ? 4 : 0) | (vec ? 2 : 0) | (P.pre ? 1 : 0);
  switch (variant) {
    case 0: k_stats<false, false, false><<<grid, kStatsThreads, 0, st>>>(P); break;
    case 1: k_stats<false, false, true><<<grid, kStatsThreads, 0, st>>>(P); break;
    case 2: k_stats<false, true, false><<<grid, kStatsThreads, 0, st>>>(P); break;
    case 3: k_stats<false, true, true><<<grid, kStatsThreads, 0, st>>>(P); break;
    case 4: k_stats<true, false, false><<<grid, kStatsThreads, 0, st>>>(P); break;
    case 5: k_stats<true, false, true><<<grid, kStatsThreads, 0, st>>>(P); break;
    case 6: k_stats<true, true, false><<<grid, kStatsThreads, 0, st>>>(P); break;
    default: k_stats<true, true, true><<<grid, kStatsThreads, 0, st>>>(P); break;
  }
  const int s = cuda_status(cudaGetLastError(), "k_stats");
  if (scratch) cudaFreeAsync(scratch, st);
  return s;
}

int stats_entry(const rmg_transform* pre, uint32_t pre_stride, const rmg_vec3* dp, const uint8_t* dmask,
                const uint32_t* dids, const rmg_vec3* mp, const rmg_vec3* mn, const uint8_t* mmask,
                const uint32_t* mids, const rmg_umeyama_constraints* params, uint32_t n_batches, uint32_t n_per,
                rmg_cross_stats* stats, rmg_transform* transforms, void* stream, bool p2l) {
  if (n_batches == 0) return RMG_OK;
  if (!stats && !transforms) return fail(RMG_ERR_INVALID_ARG, "statistics: no output requested");
  if (p2l && !mn) return fail(RMG_ERR_INVALID_ARG, "statistics_p2l: model normals are NULL");
  StatsParams P;
  int s = fill_params(pre, pre_stride, dp, dmask, dids, mp, mn, mmask, mids, params, n_batches, n_per, P);
  if (s != RMG_OK) return s;
  cudaStream_t st = as_stream(stream);
  P.stats = stats;
  double* dstats = nullptr;
  if (transforms) {
    RMG_CUDA_TRY(cudaMallocAsync(reinterpret_cast<void**>(&dstats), 16 * sizeof(double) * (size_t)n_batches, st));
    P.dstats = dstats;
  }
  s = launch_stats(P, p2l, st);
  if (s == RMG_OK && transforms) {
    k_umeyama_dstats<<<(n_batches + 127) / 128, 128, 0, st>>>(dstats, n_batches, transforms);
    s = cuda_status(cudaGetLastError(), "k_umeyama_dstats");
  }
  if (dstats) cudaFreeAsync(dstats, st);
  return s;
}

}  // namespace
}  // namespace rmg

using namespace rmg;

extern "C" int rmg_statistics_p2p(const rmg_transform* pre_transforms, uint32_t pre_transform_stride,
                                  const rmg_vec3* dataset_points, const uint8_t* dataset_mask,
                                  const uint32_t* dataset_ids, const rmg_vec3* model_points,
                                  const uint8_t* model_mask, const uint32_t* model_ids,
                                  const rmg_umeyama_constraints* params, uint32_t n_batches, uint32_t n_per_batch,
                                  rmg_cross_stats* stats, rmg_transform* transforms, void* stream) {
  return guarded("rmg_statistics_p2p", [&]() -> int {
    return stats_entry(pre_transforms, pre_transform_stride, dataset_points, dataset_mask, dataset_ids, model_points,
                       nullptr, model_mask, model_ids, params, n_batches, n_per_batch, stats, transforms, stream, false);
  });
}

extern "C" int rmg_statistics_p2l(const rmg_transform* pre_transforms, uint32_t pre_transform_stride,
                                  const rmg_vec3* dataset_points, const uint8_t* dataset_mask,
                                  const uint32_t* dataset_ids, const rmg_vec3* model_points,
                                  const rmg_vec3* model_normals, const uint8_t* model_mask,
                                  const uint32_t* model_ids, const rmg_umeyama_constraints* params,
                                  uint32_t n_batches, uint32_t n_per_batch, rmg_cross_stats* stats,
                                  rmg_transform* transforms, void* stream) {
  return guarded("rmg_statistics_p2l", [&]() -> int {
    return stats_entry(pre_transforms, pre_transform_stride, dataset_points, dataset_mask, dataset_ids, model_points,
                       model_normals, model_mask, model_ids, params, n_batches, n_per_batch, stats, transforms, stream,
                       true);
  });
}

// One 3x3 SVD per thread (binary64 inside, binary32 in and out; column-major
// matrices as in rmagine's Matrix3x3).  rotations == 0 gives the usual form
// (W >= 0 on the diagonal, sorted descending; U, V orthogonal); rotations != 0
// gives U and V both rotations with the last singular value carrying the sign
// of det A, the form the Umeyama step uses.
__global__ void k_svd3(const float* A, float* U, float* W, float* w, float* V, uint32_t n, int rotations) {
  const uint32_t b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= n) return;
  M3d C, u, v;
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c) C.a[r][c] = A[9ull * b + 3 * c + r];
  double sv[3];
  svd3_rot(C, u, sv, v);
  if (!rotations) {
    if (sv[2] < 0.0) {  // move the sign into U's third column
      sv[2] = -sv[2];
      for (int k = 0; k < 3; ++k) u.a[k][2] = -u.a[k][2];
    }
    // W >= 0 in descending order (rank-deficient inputs can leave the two
    // smallest values swapped at rounding level): swap columns of U and V alike
    for (int i = 0; i < 2; ++i)
      for (int j = 0; j < 2 - i; ++j)
        if (sv[j] < sv[j + 1]) {
          const double t = sv[j]; sv[j] = sv[j + 1]; sv[j + 1] = t;
          for (int k = 0; k < 3; ++k) {
            double x = u.a[k][j]; u.a[k][j] = u.a[k][j + 1]; u.a[k][j + 1] = x;
            x = v.a[k][j]; v.a[k][j] = v.a[k][j + 1]; v.a[k][j + 1] = x;
          }
        }
  }
  for (int r = 0; r < 3; ++r) {
    for (int c = 0; c < 3; ++c) {
      if (U) U[9ull * b + 3 * c + r] = (float)u.a[r][c];
      if (V) V[9ull * b + 3 * c + r] = (float)v.a[r][c];
      if (W) W[9ull * b + 3 * c + r] = r == c ? (float)sv[r] : 0.0f;
    }
    if (w) w[3ull * b + r] = (float)sv[r];
  }
}

extern "C" int rmg_svd3(const float* A, float* U, float* W, float* w, float* V, uint32_t n, int rotations,
                        void* stream) {
  return guarded("rmg_svd3", [&]() -> int {
    if (n == 0) return RMG_OK;
    if (!A) return fail(RMG_ERR_INVALID_ARG, "rmg_svd3: A is NULL");
    if (!U && !W && !w && !V) return RMG_OK;
    const uint64_t grid = (n + 127ull) / 128ull;
    k_svd3<<<(unsigned)grid, 128, 0, as_stream(stream)>>>(A, U, W, w, V, n, rotations);
    return cuda_status(cudaGetLastError(), "k_svd3");
  });
}

extern "C" int rmg_umeyama_transform(const rmg_cross_stats* stats, uint32_t n, rmg_transform* out, void* stream) {
  return guarded("rmg_umeyama_transform", [&]() -> int {
    if (n == 0) return RMG_OK;
    if (!stats || !out) return fail(RMG_ERR_INVALID_ARG, "rmg_umeyama_transform: NULL argument");
    k_umeyama_stats<<<(n + 127) / 128, 128, 0, as_stream(stream)>>>(stats, n, out);
    return cuda_status(cudaGetLastError(), "k_umeyama_stats");
  });
}

extern "C" int rmg_umeyama_backward(const rmg_transform* pre_transforms, uint32_t pre_transform_stride,
                                    const rmg_vec3* dataset_points, const uint8_t* dataset_mask,
                                    const uint32_t* dataset_ids, const rmg_vec3* model_points,
                                    const uint8_t* model_mask, const uint32_t* model_ids,
                                    const rmg_umeyama_constraints* params, uint32_t n_batches, uint32_t n_per_batch,
                                    const rmg_cross_stats* stats, const float* grad_R, const float* grad_t,
                                    rmg_vec3* grad_dataset, rmg_vec3* grad_model, void* stream) {
  return guarded("rmg_umeyama_backward", [&]() -> int {
    if (n_batches == 0) return RMG_OK;
    if (!stats) return fail(RMG_ERR_INVALID_ARG, "rmg_umeyama_backward: stats is NULL");
    if (!grad_dataset && !grad_model) return RMG_OK;
    BwdParams B;
    int s = fill_params(pre_transforms, pre_transform_stride, dataset_points, dataset_mask, dataset_ids, model_points,
                        nullptr, model_mask, model_ids, params, n_batches, n_per_batch, B.S);
    if (s != RMG_OK) return s;
    cudaStream_t st = as_stream(stream);
    Coef* coef = nullptr;
    RMG_CUDA_TRY(cudaMallocAsync(reinterpret_cast<void**>(&coef), sizeof(Coef) * (size_t)n_batches, st));
    k_umeyama_bwd_coef<<<(n_batches + 127) / 128, 128, 0, st>>>(stats, grad_R, grad_t, n_batches, coef);
    s = cuda_status(cudaGetLastError(), "k_umeyama_bwd_coef");
    if (s == RMG_OK) {
      B.coef = coef;
      B.gd = reinterpret_cast<float*>(grad_dataset);
      B.gm = reinterpret_cast<float*>(grad_model);
      k_umeyama_bwd_stream<<<n_batches * B.S.chunks, kStatsThreads, 0, st>>>(B);
      s = cuda_status(cudaGetLastError(), "k_umeyama_bwd_stream");
    }
    cudaFreeAsync(coef, st);
    return s;
  });
}
