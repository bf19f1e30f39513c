// Binary64 3x3 linear algebra for the Umeyama step: singular value
// decomposition with right-handed factors, the Kabsch/Umeyama rotation, the
// rotation-matrix -> quaternion conversion, and the rotation's derivative.
//
// Replaces rmagine's Numerical-Recipes svdcmp (src/rmagine_core/src/math/
// linalg.cpp:101, device src/rmagine_cuda/src/math/linalg.cu:61) and
// umeyama_transform (optimization.cpp:12-49, linalg.cu:1157-1200).
//
// SVD: cyclic Jacobi eigen-decomposition of the symmetric A = C^T C gives V
// and sigma^2 (sorted descending, V made right-handed); U = [u1, u2, u1 x u2]
// with u1, u2 from C V by Gram-Schmidt, and the third singular value carries
// the sign: sigma3 = u3 . (C v3).  With U and V both rotations,
// C = U diag(s1, s2, s3) V^T and the Umeyama rotation (R = U S V^T with the
// reflection fix S = diag(1, 1, sign det(U V^T)) of the usual SVD) is simply
// R = U V^T.
#pragma once

#include <math.h>

namespace rmg {

struct M3d { double a[3][3]; };  // row-major

__host__ __device__ inline M3d m3_zero() {
  M3d r;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) r.a[i][j] = 0.0;
  return r;
}

__host__ __device__ inline M3d m3_eye() {
  M3d r = m3_zero();
  r.a[0][0] = r.a[1][1] = r.a[2][2] = 1.0;
  return r;
}

__host__ __device__ inline M3d m3_mul(const M3d& x, const M3d& y) {
  M3d r;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) r.a[i][j] = x.a[i][0] * y.a[0][j] + x.a[i][1] * y.a[1][j] + x.a[i][2] * y.a[2][j];
  return r;
}

__host__ __device__ inline M3d m3_mul_tn(const M3d& x, const M3d& y) {  // x^T y
  M3d r;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) r.a[i][j] = x.a[0][i] * y.a[0][j] + x.a[1][i] * y.a[1][j] + x.a[2][i] * y.a[2][j];
  return r;
}

__host__ __device__ inline M3d m3_mul_nt(const M3d& x, const M3d& y) {  // x y^T
  M3d r;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) r.a[i][j] = x.a[i][0] * y.a[j][0] + x.a[i][1] * y.a[j][1] + x.a[i][2] * y.a[j][2];
  return r;
}

__host__ __device__ inline double m3_det(const M3d& m) {
  return m.a[0][0] * (m.a[1][1] * m.a[2][2] - m.a[1][2] * m.a[2][1]) -
         m.a[0][1] * (m.a[1][0] * m.a[2][2] - m.a[1][2] * m.a[2][0]) +
         m.a[0][2] * (m.a[1][0] * m.a[2][1] - m.a[1][1] * m.a[2][0]);
}

// C = U diag(s) V^T with U, V proper rotations; s[0] >= s[1] >= |s[2]|, s[2] signed.
__host__ __device__ inline void svd3_rot(const M3d& C, M3d& U, double s[3], M3d& V) {
  M3d A = m3_mul_tn(C, C);
  V = m3_eye();
  double scale = 0.0;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) scale = fmax(scale, fabs(A.a[i][j]));
  if (scale > 0.0) {
    for (int sweep = 0; sweep < 24; ++sweep) {
      const double off = A.a[0][1] * A.a[0][1] + A.a[0][2] * A.a[0][2] + A.a[1][2] * A.a[1][2];
      if (off <= 1e-36 * scale * scale) break;
      for (int p = 0; p < 2; ++p) {
        for (int q = p + 1; q < 3; ++q) {
          const double apq = A.a[p][q];
          if (fabs(apq) <= 1e-300) continue;
          const double theta = (A.a[q][q] - A.a[p][p]) / (2.0 * apq);
          const double t = (theta >= 0.0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
          const double c = 1.0 / sqrt(t * t + 1.0), s_ = t * c;
          for (int k = 0; k < 3; ++k) {  // A <- A J
            const double akp = A.a[k][p], akq = A.a[k][q];
            A.a[k][p] = c * akp - s_ * akq;
            A.a[k][q] = s_ * akp + c * akq;
          }
          for (int k = 0; k < 3; ++k) {  // A <- J^T A
            const double apk = A.a[p][k], aqk = A.a[q][k];
            A.a[p][k] = c * apk - s_ * aqk;
            A.a[q][k] = s_ * apk + c * aqk;
          }
          for (int k = 0; k < 3; ++k) {  // V <- V J
            const double vkp = V.a[k][p], vkq = V.a[k][q];
            V.a[k][p] = c * vkp - s_ * vkq;
            V.a[k][q] = s_ * vkp + c * vkq;
          }
        }
      }
    }
  }
  // sort eigenvalues descending (swap V columns)
  double lam[3] = {A.a[0][0], A.a[1][1], A.a[2][2]};
  for (int i = 0; i < 2; ++i) {
    for (int j = 0; j < 2 - i; ++j) {
      if (lam[j] < lam[j + 1]) {
        const double t = lam[j]; lam[j] = lam[j + 1]; lam[j + 1] = t;
        for (int k = 0; k < 3; ++k) { const double v = V.a[k][j]; V.a[k][j] = V.a[k][j + 1]; V.a[k][j + 1] = v; }
      }
    }
  }
  if (m3_det(V) < 0.0)
    for (int k = 0; k < 3; ++k) V.a[k][2] = -V.a[k][2];
  // B = C V: columns b_i = s_i u_i
  const M3d B = m3_mul(C, V);
  double u1[3] = {B.a[0][0], B.a[1][0], B.a[2][0]};
  double n1 = sqrt(u1[0] * u1[0] + u1[1] * u1[1] + u1[2] * u1[2]);
  if (!(n1 > 1e-300)) {  // C == 0: any frame, take V's
    U = V;
    s[0] = s[1] = s[2] = 0.0;
    return;
  }
  for (int k = 0; k < 3; ++k) u1[k] /= n1;
  double u2[3] = {B.a[0][1], B.a[1][1], B.a[2][1]};
  double d12 = u1[0] * u2[0] + u1[1] * u2[1] + u1[2] * u2[2];
  for (int k = 0; k < 3; ++k) u2[k] -= d12 * u1[k];
  double n2 = sqrt(u2[0] * u2[0] + u2[1] * u2[1] + u2[2] * u2[2]);
  if (!(n2 > 1e-12 * n1)) {  // rank 1: any unit vector orthogonal to u1
    const int k = (fabs(u1[0]) <= fabs(u1[1]) && fabs(u1[0]) <= fabs(u1[2])) ? 0 : (fabs(u1[1]) <= fabs(u1[2]) ? 1 : 2);
    double e[3] = {0.0, 0.0, 0.0};
    e[k] = 1.0;
    d12 = u1[k];
    for (int j = 0; j < 3; ++j) u2[j] = e[j] - d12 * u1[j];
    n2 = sqrt(u2[0] * u2[0] + u2[1] * u2[1] + u2[2] * u2[2]);
  }
  for (int k = 0; k < 3; ++k) u2[k] /= n2;
  const double u3[3] = {u1[1] * u2[2] - u1[2] * u2[1], u1[2] * u2[0] - u1[0] * u2[2], u1[0] * u2[1] - u1[1] * u2[0]};
  for (int k = 0; k < 3; ++k) { U.a[k][0] = u1[k]; U.a[k][1] = u2[k]; U.a[k][2] = u3[k]; }
  s[0] = n1;
  s[1] = u2[0] * B.a[0][1] + u2[1] * B.a[1][1] + u2[2] * B.a[2][1];
  s[2] = u3[0] * B.a[0][2] + u3[1] * B.a[1][2] + u3[2] * B.a[2][2];
}

// Rotation matrix -> unit quaternion (x, y, z, w).  Branch choice as in
// rmagine's Matrix -> Quaternion cast (math/types/MatrixOps.tcc:1492-1529),
// so both pick the same of the two signs q / -q.
__host__ __device__ inline void rot_to_quat(const M3d& R, double q[4]) {
  const double tr = R.a[0][0] + R.a[1][1] + R.a[2][2];
  if (tr > 0.0) {
    const double S = sqrt(tr + 1.0) * 2.0;
    q[3] = 0.25 * S;
    q[0] = (R.a[2][1] - R.a[1][2]) / S;
    q[1] = (R.a[0][2] - R.a[2][0]) / S;
    q[2] = (R.a[1][0] - R.a[0][1]) / S;
  } else if (R.a[0][0] > R.a[1][1] && R.a[0][0] > R.a[2][2]) {
    const double S = sqrt(1.0 + R.a[0][0] - R.a[1][1] - R.a[2][2]) * 2.0;
    q[3] = (R.a[2][1] - R.a[1][2]) / S;
    q[0] = 0.25 * S;
    q[1] = (R.a[0][1] + R.a[1][0]) / S;
    q[2] = (R.a[0][2] + R.a[2][0]) / S;
  } else if (R.a[1][1] > R.a[2][2]) {
    const double S = sqrt(1.0 + R.a[1][1] - R.a[0][0] - R.a[2][2]) * 2.0;
    q[3] = (R.a[0][2] - R.a[2][0]) / S;
    q[0] = (R.a[0][1] + R.a[1][0]) / S;
    q[1] = 0.25 * S;
    q[2] = (R.a[1][2] + R.a[2][1]) / S;
  } else {
    const double S = sqrt(1.0 + R.a[2][2] - R.a[0][0] - R.a[1][1]) * 2.0;
    q[3] = (R.a[1][0] - R.a[0][1]) / S;
    q[0] = (R.a[0][2] + R.a[2][0]) / S;
    q[1] = (R.a[1][2] + R.a[2][1]) / S;
    q[2] = 0.25 * S;
  }
  const double n = sqrt(q[0] * q[0] + q[1] * q[1] + q[2] * q[2] + q[3] * q[3]);
  for (int k = 0; k < 4; ++k) q[k] /= n;
}

// Umeyama / Kabsch: R = U V^T, t = m - R d.  n == 0 or a non-finite result
// gives the identity rotation (optimization.cpp:19-46).
__host__ __device__ inline void umeyama_d(const M3d& C, const double d[3], const double m[3], unsigned int n,
                                          M3d& R, double q[4], double t[3]) {
  if (n == 0) {
    R = m3_eye();
    q[0] = q[1] = q[2] = 0.0; q[3] = 1.0;
    t[0] = t[1] = t[2] = 0.0;
    return;
  }
  M3d U, V;
  double s[3];
  svd3_rot(C, U, s, V);
  R = m3_mul_nt(U, V);
  rot_to_quat(R, q);
  bool finite = true;
  for (int k = 0; k < 4; ++k) finite = finite && isfinite(q[k]);
  if (!finite) {
    R = m3_eye();
    q[0] = q[1] = q[2] = 0.0; q[3] = 1.0;
  }
  for (int i = 0; i < 3; ++i) t[i] = m[i] - (R.a[i][0] * d[0] + R.a[i][1] * d[1] + R.a[i][2] * d[2]);
}

// Relative size below which s_i + s_j counts as zero in rotation_backward.
// The covariance reaches the backward in binary32 (rmagine's CrossStatistics),
// so singular values carry an absolute error of about 1e-7 s0: a smaller sum
// is rounding noise, and dividing by it would only amplify that noise.
constexpr double kRotGradGap = 1e-6;

// Gradient of L through R = U V^T (C = U diag(s) V^T, rotations U, V):
// dL/dC = U K V^T with K_ij = (G_ij - G_ji) / (s_i + s_j) for i != j, K_ii = 0,
// G = U^T (dL/dR) V.  Where s_i + s_j <= kRotGradGap * s0 the optimal rotation
// about the axis u_i x u_j is not unique (collinear correspondences: s2 = s3 = 0;
// a reflection with two equal singular values: s2 = -s3) and R is not
// differentiable there: that pair contributes no gradient (K_ij = K_ji = 0).
// The rest of the gradient is exact; close to the boundary it grows like
// 1 / (s_i + s_j), as the rotation's true derivative does.
__host__ __device__ inline M3d rotation_backward(const M3d& U, const double s[3], const M3d& V, const M3d& gR) {
  const M3d G = m3_mul(m3_mul_tn(U, gR), V);
  M3d K = m3_zero();
  const double gap = kRotGradGap * fabs(s[0]);
  for (int i = 0; i < 3; ++i) {
    for (int j = 0; j < 3; ++j) {
      if (i == j) continue;
      const double den = s[i] + s[j];
      K.a[i][j] = den > gap ? (G.a[i][j] - G.a[j][i]) / den : 0.0;
    }
  }
  return m3_mul_nt(m3_mul(U, K), V);
}

}  // namespace rmg
