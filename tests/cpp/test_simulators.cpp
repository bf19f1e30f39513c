// C++ API test: rmagine's own simulation known answers (tests/embree/simulation_*.cpp,
// tests/optix/simulation_o1dn.cpp) and the CrossStatistics paper example
// (tests/core/math_statistics.cpp:322-384), through include/rmagine_gb300.hpp, written
// the way rmagine's tests are: an executable that throws on failure.
#include <cmath>
#include <cstdio>
#include <sstream>

#include "rmagine_gb300.hpp"

namespace rm = rmagine_gb300;

static void fail_if(bool bad, const std::string& what) {
  if (bad) throw std::runtime_error(what);
}

// The unit cube of rmagine's genCube (synthetic.cpp:183-221).
static rm::MapPtr make_cube_map() {
  rm::Memory<rm::Vector3, rm::RAM> V(8);
  const float c[8][3] = {{-0.5f, -0.5f, -0.5f}, {-0.5f, -0.5f, 0.5f}, {-0.5f, 0.5f, 0.5f}, {-0.5f, 0.5f, -0.5f},
                         {0.5f, 0.5f, -0.5f},   {0.5f, 0.5f, 0.5f},   {0.5f, -0.5f, 0.5f}, {0.5f, -0.5f, -0.5f}};
  for (int i = 0; i < 8; ++i) V[i] = {c[i][0], c[i][1], c[i][2]};
  const uint32_t f[12][3] = {{0, 1, 2}, {2, 3, 0}, {4, 5, 6}, {6, 7, 4}, {0, 7, 1}, {1, 7, 6},
                             {1, 6, 5}, {5, 2, 1}, {2, 5, 4}, {3, 2, 4}, {3, 4, 7}, {3, 7, 0}};
  rm::Memory<rm::Face, rm::RAM> F(12);
  for (int i = 0; i < 12; ++i) F[i] = {f[i][0], f[i][1], f[i][2]};
  return std::make_shared<rm::TriangleMap>(V, F);
}

static rm::Memory<rm::Transform, rm::RAM> identity_poses(size_t n) {
  rm::Memory<rm::Transform, rm::RAM> T(n);
  for (size_t i = 0; i < n; ++i) T[i] = rm::Transform::Identity();
  return T;
}

static void test_spherical(const rm::MapPtr& map) {
  rm::SphericalModel model;  // example_spherical (sensors.cpp:39-54)
  model.theta = {(float)-M_PI, (float)(0.4 * M_PI / 180.0), 900};
  model.phi = {(float)(-15.0 * M_PI / 180.0), (float)(2.0 * M_PI / 180.0), 16};
  model.range = {0.0f, 100.0f};
  rm::SphereSimulatorGB300 sim(map);
  sim.setModel(model);
  auto res = sim.simulate<rm::IntAttrAll<rm::RAM>>(identity_poses(100));
  const float r = res.ranges[model.size() * 99 + model.getBufferId(model.phi.size / 2, 0)];
  std::ostringstream ss;
  ss << "spherical: range " << r << " vs 0.500076";
  fail_if(std::fabs(r - 0.500076f) > 1e-4f, ss.str());
}

static void test_pinhole(const rm::MapPtr& map) {
  rm::PinholeModel model{200, 150, {0.0f, 100.0f}, {100.0f, 100.0f}, {100.0f, 75.0f}};  // example_pinhole
  rm::PinholeSimulatorGB300 sim(map);
  sim.setModel(model);
  rm::Bundle<rm::Ranges<rm::RAM>, rm::Points<rm::RAM>> res;
  rm::resize_memory_bundle<rm::RAM>(res, model.getWidth(), model.getHeight(), 100);
  sim.simulate(identity_poses(100), res);
  const rm::Vector3 p = res.points[model.size() * 99];
  const float err = std::fabs(p.x - 0.5f) + std::fabs(p.y - 0.5f) + std::fabs(p.z - 0.375f);
  fail_if(err > 1e-4f, "pinhole: point error");
}

static void test_o1dn(const rm::MapPtr& map) {
  rm::O1DnModel model;  // example_o1dn (sensors.cpp:70-102)
  model.width = 200;
  model.height = 1;
  model.range = {0.0f, 100.0f};
  model.orig = {0.0f, 0.0f, 0.0f};
  model.dirs.resize(200);
  for (int i = 0; i < 200; ++i) {
    const float y = -static_cast<float>(i - 100) * 0.05f;
    const float x = std::cos(y) * 2.0 + 2.0;
    const float z = -1.0f;
    const float n = std::sqrt(x * x + y * y + z * z);
    model.dirs[i] = {x / n, y / n, z / n};
  }
  rm::O1DnSimulatorGB300 sim(map);
  sim.setModel(model);
  auto res = sim.simulate<rm::IntAttrAll<rm::RAM>>(identity_poses(100));
  const size_t k = model.size() * 99;
  const rm::Vector3 p = res.points[k], n = res.normals[k];
  fail_if(std::fabs(p.x - 0.256732f) + std::fabs(p.y - 0.5f) + std::fabs(p.z + 0.1f) > 1e-4f, "o1dn: point");
  fail_if(std::sqrt(n.x * n.x + (n.y + 1.0f) * (n.y + 1.0f) + n.z * n.z) > 1e-4f, "o1dn: normal");
  fail_if(std::fabs(res.ranges[k] - 0.570887f) > 1e-4f, "o1dn: range");
}

static void test_ondn_single_ray(const rm::MapPtr& map) {
  rm::OnDnModel model;  // tests/embree/simulation_single_ray.cpp
  model.width = 1;
  model.height = 1;
  model.range = {0.0f, 100.0f};
  model.origs.resize(1);
  model.dirs.resize(1);
  model.origs[0] = {0.0f, 0.0f, 0.0f};
  model.dirs[0] = {1.0f, 0.0f, 0.0f};
  rm::OnDnSimulatorGB300 sim(map);
  sim.setModel(model);
  // device form with a device bundle
  rm::Memory<rm::Transform, rm::VRAM_CUDA> Td;
  Td = identity_poses(100);
  auto dev = sim.simulate<rm::Bundle<rm::Ranges<rm::VRAM_CUDA>, rm::FaceIds<rm::VRAM_CUDA>>>(Td);
  rm::cuda_check(cudaDeviceSynchronize(), "sync");
  rm::Memory<float, rm::RAM> r;
  r = dev.ranges;
  fail_if(std::fabs(r[0] - 0.5f) > 1e-4f, "ondn: single ray range");
}

static void test_stats_paper() {
  // four 1-D correspondences: dataset (1, 5, 6, 8), model (3, 1, 4, 8)
  rm::Memory<rm::Vector3, rm::RAM> d(4), m(4);
  const float dx[4] = {1, 5, 6, 8}, mx[4] = {3, 1, 4, 8};
  for (int i = 0; i < 4; ++i) { d[i] = {dx[i], 0, 0}; m[i] = {mx[i], 0, 0}; }
  rm::Memory<rm::Vector3, rm::VRAM_CUDA> dd, md;
  dd = d;
  md = m;
  rm::Memory<rm::CrossStatistics, rm::VRAM_CUDA> st;
  rm::Memory<rm::Transform, rm::VRAM_CUDA> T;
  rm::statistics_p2p(dd, md, {20000.0f, 0, 0}, 1, st, &T);
  rm::cuda_check(cudaDeviceSynchronize(), "sync");
  rm::Memory<rm::CrossStatistics, rm::RAM> s;
  s = st;
  fail_if(std::fabs(s[0].dataset_mean.x - 5.0f) > 1e-4f || std::fabs(s[0].model_mean.x - 4.0f) > 1e-4f ||
              std::fabs(s[0].covariance[0] - 4.0f) > 1e-4f || s[0].n_meas != 4,
          "statistics_p2p: paper example");
}

int main() {
  try {
    auto map = make_cube_map();
    test_spherical(map);
    test_pinhole(map);
    test_o1dn(map);
    test_ondn_single_ray(map);
    test_stats_paper();
    fail_if(map->status() != 0, "device status");
  } catch (const std::exception& e) {
    std::fprintf(stderr, "FAILED: %s\n", e.what());
    return 1;
  }
  std::printf("C++ API tests passed\n");
  return 0;
}
