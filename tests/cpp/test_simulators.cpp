// C++ API test: rmagine's own simulation known answers (tests/embree/simulation_*.cpp,
// tests/optix/simulation_o1dn.cpp) and the CrossStatistics paper example
// (tests/core/math_statistics.cpp:322-384), through include/rmagine_gb300.hpp, written
// the way rmagine's tests are: an executable that throws on failure.  Then the
// layer's other parts: an instanced scene, the fused correction step, noise,
// mesh and map files, and the launch autotuner.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <memory>
#include <vector>
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

static rm::SphericalModel vlp16() {
  rm::SphericalModel model;  // vlp16_900 (sensors.cpp:6-20)
  model.theta = {(float)-M_PI, (float)(0.4 * M_PI / 180.0), 900};
  model.phi = {(float)(-15.0 * M_PI / 180.0), (float)(2.0 * M_PI / 180.0), 16};
  model.range = {0.5f, 130.0f};
  return model;
}

// The cube placed by one identity instance gives the single-mesh results bit for bit.
static void test_scene_identity_instance(const rm::MapPtr& map) {
  rm::Instance inst;
  inst.geom_id = 3;
  inst.object_id = 9;
  auto scene = std::make_shared<rm::InstancedScene>(std::vector<rm::MapPtr>{map}, std::vector<rm::Instance>{inst});
  rm::SphereSimulatorGB300 a(map), b;
  a.setModel(vlp16());
  b.setModel(vlp16());
  b.setMap(scene);
  auto ra = a.simulate<rm::IntAttrAll<rm::RAM>>(identity_poses(2));
  auto rb = b.simulate<rm::IntAttrAll<rm::RAM>>(identity_poses(2));
  size_t hits = 0;
  for (size_t i = 0; i < ra.ranges.size(); ++i) {
    fail_if(std::memcmp(&ra.ranges[i], &rb.ranges[i], 4) != 0 || ra.face_ids[i] != rb.face_ids[i], "scene: ranges");
    if (ra.hits[i]) {
      ++hits;
      fail_if(rb.object_ids[i] != 9 || rb.geom_ids[i] != 3, "scene: ids");
    }
  }
  fail_if(hits == 0 || scene->status() != 0, "scene: no hits or device error");
}

// The fused step at the pose the dataset scan was taken from: identity transform.
static void test_fused_step(const rm::MapPtr& map) {
  rm::SphereSimulatorGB300 sim(map);
  sim.setModel(vlp16());
  rm::Memory<rm::Transform, rm::VRAM_CUDA> Td;
  Td = identity_poses(1);
  auto data = sim.simulate<rm::Bundle<rm::Hits<rm::VRAM_CUDA>, rm::Points<rm::VRAM_CUDA>>>(Td);
  rm::Memory<rm::CrossStatistics, rm::VRAM_CUDA> st;
  rm::Memory<rm::Transform, rm::VRAM_CUDA> T;
  sim.simulateStatistics(Td, data.points, &data.hits, false, nullptr, {1.0f, 0, 0}, true, &st, &T);
  rm::cuda_check(cudaDeviceSynchronize(), "sync");
  rm::Memory<rm::CrossStatistics, rm::RAM> s;
  s = st;
  rm::Memory<rm::Transform, rm::RAM> t;
  t = T;
  rm::Memory<uint8_t, rm::RAM> h;
  h = data.hits;
  uint32_t n = 0;
  for (size_t i = 0; i < h.size(); ++i) n += h[i] ? 1 : 0;
  fail_if(s[0].n_meas != n || n == 0, "fused: n_meas");
  fail_if(std::fabs(t[0].t.x) + std::fabs(t[0].t.y) + std::fabs(t[0].t.z) > 1e-5f ||
              std::fabs(t[0].R.w - 1.0f) > 1e-6f,
          "fused: not the identity");
  // compose on the device: identity * T == T
  rm::Memory<rm::Transform, rm::VRAM_CUDA> out;
  rm::compose(Td, T, out);
  rm::Memory<rm::Transform, rm::RAM> o;
  o = out;
  fail_if(std::memcmp(&o[0], &t[0], 28) != 0, "compose");
  // the host form on RAM copies of the same data gives the same statistics and transform
  rm::Memory<rm::Vector3, rm::RAM> pts;
  pts = data.points;
  rm::Memory<rm::CrossStatistics, rm::RAM> s_h;
  rm::Memory<rm::Transform, rm::RAM> t_h;
  sim.simulateStatistics(identity_poses(1), pts, &h, false, nullptr, {1.0f, 0, 0}, true, &s_h, &t_h);
  fail_if(std::memcmp(&s_h[0], &s[0], sizeof(rm::CrossStatistics)) != 0, "fused host form: statistics");
  fail_if(std::memcmp(&t_h[0], &t[0], sizeof(rm::Transform)) != 0, "fused host form: transform");
}

// Noise: two objects with the same seed draw the same numbers; the next call differs.  The size
// takes both the bulk-copy ring (whole chunks of 4,096 ranges) and the register path (the tail).
static void test_noise() {
  rm::Memory<float, rm::RAM> r(3 * 4096 + 1001);
  for (size_t i = 0; i < r.size(); ++i) r[i] = 1.0f + 0.01f * (float)i;
  rm::Memory<float, rm::VRAM_CUDA> a, b;
  a = r;
  b = r;
  rm::GaussianNoiseGB300 na(0.0f, 0.1f, {7, 10000.0f}), nb(0.0f, 0.1f, {7, 10000.0f});
  na.apply(a);
  nb.apply(b);
  rm::Memory<float, rm::RAM> ha, hb;
  ha = a;
  hb = b;
  fail_if(std::memcmp(ha.raw(), hb.raw(), 4 * ha.size()) != 0, "noise: not deterministic");
  double sum = 0.0;
  for (size_t i = 0; i < r.size(); ++i) sum += ha[i] - r[i];
  fail_if(std::fabs(sum / r.size()) > 0.02, "noise: mean");
  na.apply(a);
  ha = a;
  fail_if(std::memcmp(ha.raw(), hb.raw(), 4 * ha.size()) == 0, "noise: second call repeated");
  rm::UniformDustNoiseGB300 dust(0.01f, 0.9f);
  dust.apply(b);
  rm::cuda_check(cudaDeviceSynchronize(), "sync");
  rm::NoiseGB300::check_device();
}

// Mesh and map files round trip.
static void test_files(const rm::MapPtr& map) {
  rm::Memory<rm::Vector3, rm::RAM> V(8);
  rm::Memory<rm::Face, rm::RAM> F(12);
  const float c[8][3] = {{-0.5f, -0.5f, -0.5f}, {-0.5f, -0.5f, 0.5f}, {-0.5f, 0.5f, 0.5f}, {-0.5f, 0.5f, -0.5f},
                         {0.5f, 0.5f, -0.5f},   {0.5f, 0.5f, 0.5f},   {0.5f, -0.5f, 0.5f}, {0.5f, -0.5f, -0.5f}};
  for (int i = 0; i < 8; ++i) V[i] = {c[i][0], c[i][1], c[i][2]};
  for (int i = 0; i < 12; ++i) F[i] = {(uint32_t)i % 8, (uint32_t)(i + 1) % 8, (uint32_t)(i + 3) % 8};
  const std::string ply = "rmg_cpp_test_cube.ply", mp = "rmg_cpp_test_cube.rmgmap";
  rm::write_ply(ply, V, F);
  const rm::MeshData m = rm::read_mesh(ply);
  fail_if(m.vertices.size() != 8 || m.faces.size() != 12 ||
              std::memcmp(m.vertices.raw(), V.raw(), sizeof(rm::Vector3) * 8) != 0 ||
              std::memcmp(m.faces.raw(), F.raw(), sizeof(rm::Face) * 12) != 0,
          "files: PLY round trip");
  map->save(mp);
  auto loaded = rm::TriangleMap::load(mp);
  rm::SphereSimulatorGB300 a(map), b(loaded);
  a.setModel(vlp16());
  b.setModel(vlp16());
  auto ra = a.simulate<rm::IntAttrAll<rm::RAM>>(identity_poses(1));
  auto rb = b.simulate<rm::IntAttrAll<rm::RAM>>(identity_poses(1));
  fail_if(std::memcmp(ra.ranges.raw(), rb.ranges.raw(), 4 * ra.ranges.size()) != 0, "files: loaded map differs");
  std::remove(ply.c_str());
  std::remove(mp.c_str());
}

// The autotuner picks a configuration; results stay the same.
static void test_autotune(const rm::MapPtr& map) {
  rm::SphereSimulatorGB300 sim(map);
  sim.setModel(vlp16());
  rm::Memory<rm::Transform, rm::VRAM_CUDA> Td;
  Td = identity_poses(4);
  auto before = sim.simulate<rm::Bundle<rm::Ranges<rm::VRAM_CUDA>>>(Td);
  const rmg_launch_config c = sim.autotune(Td, before, 2);
  fail_if(c.tile_w * c.tile_h != 32, "autotune: config");
  auto after = sim.simulate<rm::Bundle<rm::Ranges<rm::VRAM_CUDA>>>(Td);
  rm::cuda_check(cudaDeviceSynchronize(), "sync");
  rm::Memory<float, rm::RAM> x, y;
  x = before.ranges;
  y = after.ranges;
  fail_if(std::memcmp(x.raw(), y.raw(), 4 * x.size()) != 0, "autotune: results changed");
}

// A bumpy 64 x 64 heightfield: both tree builders and the host (RAM) and device forms of
// simulate give bit-identical results.
static void test_builders_and_host_form() {
  const int G = 64;
  rm::Memory<rm::Vector3, rm::RAM> V(G * G);
  for (int y = 0; y < G; ++y)
    for (int x = 0; x < G; ++x)
      V[y * G + x] = {(float)x - G / 2, (float)y - G / 2, 0.7f * std::sin(0.31f * x) * std::cos(0.23f * y) - 2.0f};
  rm::Memory<rm::Face, rm::RAM> F(2 * (G - 1) * (G - 1));
  size_t k = 0;
  for (int y = 0; y + 1 < G; ++y)
    for (int x = 0; x + 1 < G; ++x) {
      const uint32_t a = y * G + x, b = a + 1, c = a + G, d = c + 1;
      F[k++] = {a, b, d};
      F[k++] = {a, d, c};
    }
  auto sah = std::make_shared<rm::TriangleMap>(V, F, (cudaStream_t)0, RMG_BUILD_SAH);
  auto lbvh = std::make_shared<rm::TriangleMap>(V, F, (cudaStream_t)0, RMG_BUILD_LBVH);
  rm::Memory<rm::Transform, rm::RAM> T(5);
  for (size_t i = 0; i < T.size(); ++i) {
    T[i] = rm::Transform::Identity();
    T[i].t = {-10.0f + 4.0f * i, 3.0f - 1.5f * i, 0.5f};
  }
  rm::SphereSimulatorGB300 host_sim(sah);
  host_sim.setModel(vlp16());
  auto host = host_sim.simulate<rm::Bundle<rm::Ranges<rm::RAM>, rm::Normals<rm::RAM>, rm::FaceIds<rm::RAM>>>(T);
  rm::SphereSimulatorGB300 dev_sim(lbvh);
  dev_sim.setModel(vlp16());
  rm::Memory<rm::Transform, rm::VRAM_CUDA> Td;
  Td = T;
  auto dev = dev_sim.simulate<rm::Bundle<rm::Ranges<rm::VRAM_CUDA>, rm::Normals<rm::VRAM_CUDA>,
                                         rm::FaceIds<rm::VRAM_CUDA>>>(Td);
  rm::cuda_check(cudaDeviceSynchronize(), "sync");
  rm::Memory<float, rm::RAM> r;
  rm::Memory<rm::Vector3, rm::RAM> n;
  rm::Memory<uint32_t, rm::RAM> f;
  r = dev.ranges;
  n = dev.normals;
  f = dev.face_ids;
  fail_if(r.size() != host.ranges.size() || std::memcmp(r.raw(), host.ranges.raw(), 4 * r.size()) != 0,
          "builders/host form: ranges differ");
  fail_if(std::memcmp(n.raw(), host.normals.raw(), 12 * n.size()) != 0, "builders/host form: normals differ");
  fail_if(std::memcmp(f.raw(), host.face_ids.raw(), 4 * f.size()) != 0, "builders/host form: face ids differ");
  size_t hits = 0;
  for (size_t i = 0; i < f.size(); ++i) hits += f[i] != 0xffffffffu;
  fail_if(hits == 0, "builders/host form: no ray hit the heightfield");
  // the single-pose overloads give the pose's slice of the batch
  rm::Memory<rm::SphericalModel, rm::RAM> models(1);
  models[0] = vlp16();
  rm::SphereSimulatorGB300 one(sah);
  one.setModel(models);
  auto single = one.simulate<rm::Bundle<rm::Ranges<rm::RAM>>>(T[3]);
  const size_t per = (size_t)one.width() * one.height();
  fail_if(single.ranges.size() != per ||
              std::memcmp(single.ranges.raw(), host.ranges.raw() + 3 * per, 4 * per) != 0,
          "single-pose simulate differs from the batch");
}

int main() {
  try {
    auto map = make_cube_map();
    test_spherical(map);
    test_pinhole(map);
    test_o1dn(map);
    test_ondn_single_ray(map);
    test_stats_paper();
    test_scene_identity_instance(map);
    test_fused_step(map);
    test_noise();
    test_files(map);
    test_autotune(map);
    test_builders_and_host_form();
    fail_if(map->status() != 0, "device status");
  } catch (const std::exception& e) {
    std::fprintf(stderr, "FAILED: %s\n", e.what());
    return 1;
  }
  std::printf("C++ API tests passed\n");
  return 0;
}
