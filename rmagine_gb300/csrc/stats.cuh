// Correspondence arithmetic shared by the statistics kernels (stats.cu) and
// the fused ray-cast -> statistics kernel (fused.cu), so both form the same
// D -> M pairs bit for bit.
//
// statistics_p2p / statistics_p2l (src/rmagine_core/src/math/statistics.cpp:19-126,
// src/rmagine_cuda/src/math/statistics.cu:58-160, 190-276):
//   D = pre * dataset point
//   p2p: M = model point,                 kept when ||M - D||^2 < max_dist^2
//   p2l: s = (I - D) . N, M = D + N s,    kept when |s| < max_dist
#pragma once

#include "common.cuh"

namespace rmg {

// Transform * Vector3 = R * v + t (Transform.tcc:56-60), exact order.
__device__ __forceinline__ V tf_point(const Tf& T, const V& p) {
  const V r = qrot(T.R, p);
  return V{add(r.x, T.t.x), add(r.y, T.t.y), add(r.z, T.t.z)};
}

// The distance filter and the model side of one correspondence; D is the
// pre-transformed dataset point, mpt / npt the model point / normal.
template <bool P2L>
__device__ __forceinline__ bool match(const V& D, const V& mpt, const V& npt, float max_dist, V& M) {
  if (P2L) {
    const V diff{sub(mpt.x, D.x), sub(mpt.y, D.y), sub(mpt.z, D.z)};
    const float sd = add(add(mul(diff.x, npt.x), mul(diff.y, npt.y)), mul(diff.z, npt.z));
    if (!(fabsf(sd) < max_dist)) return false;
    M = V{add(D.x, mul(npt.x, sd)), add(D.y, mul(npt.y, sd)), add(D.z, mul(npt.z, sd))};
  } else {
    M = mpt;
    const V diff{sub(M.x, D.x), sub(M.y, D.y), sub(M.z, D.z)};
    const float d2 = add(add(mul(diff.x, diff.x), mul(diff.y, diff.y)), mul(diff.z, diff.z));
    if (!(d2 < mul(max_dist, max_dist))) return false;
  }
  return true;
}

// binary64 means and covariance -> the binary32 CrossStatistics record
// (CrossStatistics.hpp: dataset_mean, model_mean, covariance, n_meas;
// covariance column-major, cov = E[m d^T] - E[m] E[d]^T).
__device__ __forceinline__ void store_cross_stats(double n, const double dm[3], const double mm[3],
                                                  const double C[9], rmg_cross_stats* out) {
  rmg_cross_stats s;
  s.dataset_mean = rmg_vec3{(float)dm[0], (float)dm[1], (float)dm[2]};
  s.model_mean = rmg_vec3{(float)mm[0], (float)mm[1], (float)mm[2]};
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c) s.covariance.data[3 * c + r] = (float)C[3 * r + c];
  s.n_meas = (uint32_t)n;
  *out = s;
}

// binary64 Umeyama result -> the binary32 Transform record.
__device__ __forceinline__ void store_tf(rmg_transform* out, const double q[4], const double t[3]) {
  rmg_transform T;
  T.R = rmg_quat{(float)q[0], (float)q[1], (float)q[2], (float)q[3]};
  T.t = rmg_vec3{(float)t[0], (float)t[1], (float)t[2]};
  T.stamp = 0;
  *out = T;
}

}  // namespace rmg
