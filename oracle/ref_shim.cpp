// ORACLE PIN -- test infrastructure only.
//
// A C-ABI shim over the parts of rmagine (uos/rmagine v2.4.2) that compile
// from their own sources without third-party libraries: the header-only core
// math and sensor-model types plus src/rmagine_core/src/types/sensors.cpp.
// build_ref.py compiles this file against the reference tree where it lies
// and writes oracle/_ref/libref.so; the tests use it to check the oracle's
// and the library's restatements of ray generation, pose math and the
// CrossStatistics merge against the reference's own code.
//
// Not buildable here and therefore absent from the shim: the Embree simulators
// (need Embree 4 / oneTBB), statistics.cpp (oneTBB), linalg.cpp's svd and
// optimization.cpp's umeyama_transform (linalg.cpp includes Eigen),
// synthetic.cpp (Assimp).
#include <rmagine/math/types.h>
#include <rmagine/types/sensor_models.h>
#include <rmagine/types/sensors.h>

#include <cstdint>
#include <cstring>

using namespace rmagine;

namespace {
Transform load_tf(const float* p) {
  Transform T;
  T.R.x = p[0]; T.R.y = p[1]; T.R.z = p[2]; T.R.w = p[3];
  T.t.x = p[4]; T.t.y = p[5]; T.t.z = p[6];
  T.stamp = 0;
  return T;
}
void store_tf(const Transform& T, float* p) {
  p[0] = T.R.x; p[1] = T.R.y; p[2] = T.R.z; p[3] = T.R.w;
  p[4] = T.t.x; p[5] = T.t.y; p[6] = T.t.z; p[7] = 0.0f;
}
void store_stats(const CrossStatistics& s, float* out, uint32_t* n) {
  out[0] = s.dataset_mean.x; out[1] = s.dataset_mean.y; out[2] = s.dataset_mean.z;
  out[3] = s.model_mean.x; out[4] = s.model_mean.y; out[5] = s.model_mean.z;
  for (int c = 0; c < 3; ++c)
    for (int r = 0; r < 3; ++r) out[6 + 3 * c + r] = s.covariance(r, c);  // column-major
  *n = s.n_meas;
}
CrossStatistics load_stats(const float* in, uint32_t n) {
  CrossStatistics s;
  s.dataset_mean = {in[0], in[1], in[2]};
  s.model_mean = {in[3], in[4], in[5]};
  for (int c = 0; c < 3; ++c)
    for (int r = 0; r < 3; ++r) s.covariance(r, c) = in[6 + 3 * c + r];
  s.n_meas = n;
  return s;
}
void store_spherical(const SphericalModel& m, float* out) {
  out[0] = m.phi.min; out[1] = m.phi.inc; out[2] = (float)m.phi.size;
  out[3] = m.theta.min; out[4] = m.theta.inc; out[5] = (float)m.theta.size;
  out[6] = m.range.min; out[7] = m.range.max;
}
}  // namespace

extern "C" {

// 0 vlp16_900, 1 vlp16_360, 2 example_spherical (sensors.cpp:6-54)
int ref_preset_spherical(int which, float* out) {
  SphericalModel m = which == 0 ? vlp16_900() : (which == 1 ? vlp16_360() : example_spherical());
  store_spherical(m, out);
  return 0;
}

// example_pinhole (sensors.cpp:56-68): w h rmin rmax fx fy cx cy
int ref_preset_pinhole(float* out) {
  const PinholeModel m = example_pinhole();
  out[0] = (float)m.width; out[1] = (float)m.height; out[2] = m.range.min; out[3] = m.range.max;
  out[4] = m.f[0]; out[5] = m.f[1]; out[6] = m.c[0]; out[7] = m.c[1];
  return 0;
}

// example_o1dn (sensors.cpp:70-102): 200 dirs, orig, range
int ref_example_o1dn(float* dirs, float* orig, float* range) {
  const O1DnModel m = example_o1dn();
  for (uint32_t i = 0; i < m.dirs.size(); ++i) {
    dirs[3 * i] = m.dirs[i].x; dirs[3 * i + 1] = m.dirs[i].y; dirs[3 * i + 2] = m.dirs[i].z;
  }
  orig[0] = m.orig.x; orig[1] = m.orig.y; orig[2] = m.orig.z;
  range[0] = m.range.min; range[1] = m.range.max;
  return (int)m.dirs.size();
}

// example_ondn (sensors.cpp:104-137)
int ref_example_ondn(float* origs, float* dirs, float* range) {
  const OnDnModel m = example_ondn();
  for (uint32_t i = 0; i < m.dirs.size(); ++i) {
    dirs[3 * i] = m.dirs[i].x; dirs[3 * i + 1] = m.dirs[i].y; dirs[3 * i + 2] = m.dirs[i].z;
    origs[3 * i] = m.origs[i].x; origs[3 * i + 1] = m.origs[i].y; origs[3 * i + 2] = m.origs[i].z;
  }
  range[0] = m.range.min; range[1] = m.range.max;
  return (int)m.dirs.size();
}

// SphericalModel::getDirection for every (vid, hid), row-major.
void ref_dirs_spherical(float phi_min, float phi_inc, uint32_t phi_size, float theta_min, float theta_inc,
                        uint32_t theta_size, float* out) {
  SphericalModel m;
  m.phi.min = phi_min; m.phi.inc = phi_inc; m.phi.size = phi_size;
  m.theta.min = theta_min; m.theta.inc = theta_inc; m.theta.size = theta_size;
  for (uint32_t v = 0; v < phi_size; ++v)
    for (uint32_t h = 0; h < theta_size; ++h) {
      const Vector d = m.getDirection(v, h);
      float* o = out + 3 * (m.getBufferId(v, h));
      o[0] = d.x; o[1] = d.y; o[2] = d.z;
    }
}

// PinholeModel::getDirection for every (vid, hid), row-major.
void ref_dirs_pinhole(uint32_t W, uint32_t H, float fx, float fy, float cx, float cy, float* out) {
  PinholeModel m;
  m.width = W; m.height = H; m.f[0] = fx; m.f[1] = fy; m.c[0] = cx; m.c[1] = cy;
  for (uint32_t v = 0; v < H; ++v)
    for (uint32_t h = 0; h < W; ++h) {
      const Vector d = m.getDirection(v, h);
      float* o = out + 3 * m.getBufferId(v, h);
      o[0] = d.x; o[1] = d.y; o[2] = d.z;
    }
}

// Transform a*b (Transform.tcc:34-42), n records.
void ref_transform_mult(const float* a, const float* b, float* out, uint32_t n) {
  for (uint32_t i = 0; i < n; ++i) store_tf(load_tf(a + 8 * i) * load_tf(b + 8 * i), out + 8 * i);
}

void ref_transform_inv(const float* a, float* out, uint32_t n) {
  for (uint32_t i = 0; i < n; ++i) store_tf(load_tf(a + 8 * i).inv(), out + 8 * i);
}

// Quaternion * Vector3 (Quaternion.tcc:68-75), n pairs.
void ref_quat_rotate(const float* q, const float* v, float* out, uint32_t n) {
  for (uint32_t i = 0; i < n; ++i) {
    Quaternion Q;
    Q.x = q[4 * i]; Q.y = q[4 * i + 1]; Q.z = q[4 * i + 2]; Q.w = q[4 * i + 3];
    const Vector r = Q * Vector{v[3 * i], v[3 * i + 1], v[3 * i + 2]};
    out[3 * i] = r.x; out[3 * i + 1] = r.y; out[3 * i + 2] = r.z;
  }
}

// Transform * Vector3 = R*v + t (Transform.tcc:56-60), n pairs.
void ref_transform_point(const float* T, const float* v, float* out, uint32_t n) {
  for (uint32_t i = 0; i < n; ++i) {
    const Vector r = load_tf(T + 8 * i) * Vector{v[3 * i], v[3 * i + 1], v[3 * i + 2]};
    out[3 * i] = r.x; out[3 * i + 1] = r.y; out[3 * i + 2] = r.z;
  }
}

// EulerAngles -> Quaternion (EulerAngles.tcc:40-61).
void ref_euler_to_quat(const float* rpy, float* out, uint32_t n) {
  for (uint32_t i = 0; i < n; ++i) {
    EulerAngles e;
    e.roll = rpy[3 * i]; e.pitch = rpy[3 * i + 1]; e.yaw = rpy[3 * i + 2];
    const Quaternion q = e;
    out[4 * i] = q.x; out[4 * i + 1] = q.y; out[4 * i + 2] = q.z; out[4 * i + 3] = q.w;
  }
}

// Matrix3x3 -> Quaternion (MatrixOps.tcc:1492-1529); m is row-major.
void ref_matrix_to_quat(const float* m, float* out, uint32_t n) {
  for (uint32_t i = 0; i < n; ++i) {
    Matrix3x3 M;
    for (int r = 0; r < 3; ++r)
      for (int c = 0; c < 3; ++c) M(r, c) = m[9 * i + 3 * r + c];
    Quaternion q;
    q.set(M);
    out[4 * i] = q.x; out[4 * i + 1] = q.y; out[4 * i + 2] = q.z; out[4 * i + 3] = q.w;
  }
}

// acc = Identity; acc += Init(d_i, m_i) for i in order (CrossStatistics.tcc:33-58).
void ref_cross_stats_fold(const float* d, const float* m, uint32_t n, float* out, uint32_t* n_out) {
  CrossStatistics acc = CrossStatistics::Identity();
  for (uint32_t i = 0; i < n; ++i)
    acc += CrossStatistics::Init(Vector{d[3 * i], d[3 * i + 1], d[3 * i + 2]},
                                 Vector{m[3 * i], m[3 * i + 1], m[3 * i + 2]});
  store_stats(acc, out, n_out);
}

// a + b (CrossStatistics.tcc:7-31).
void ref_cross_stats_add(const float* a, uint32_t na, const float* b, uint32_t nb, float* out, uint32_t* n_out) {
  store_stats(load_stats(a, na) + load_stats(b, nb), out, n_out);
}

}  // extern "C"
