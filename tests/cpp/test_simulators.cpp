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
#include <type_traits>

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


// MemoryView slices, the const-view overloads, setTsb(MemoryView), the pinned / managed memory
// kinds and the factory (SphereSimulatorEmbree.hpp:140-155, SimulatorEmbree.hpp:60,
// MemoryCuda.hpp:78-89, Simulator.hpp:52-78).
static void test_views_kinds_and_factory(const rm::MapPtr& map) {
  rm::SphericalModel model;
  model.theta = {(float)-M_PI, (float)(0.4 * M_PI / 180.0), 900};
  model.phi = {(float)(-15.0 * M_PI / 180.0), (float)(2.0 * M_PI / 180.0), 16};
  model.range = {0.0f, 100.0f};
  auto sim = rm::make_simulator<rm::SphericalModel, rm::GB300>(map);
  static_assert(std::is_same<decltype(sim), rm::SimulatorPtr<rm::SphericalModel, rm::GB300>>::value, "factory type");
  static_assert(std::is_same<decltype(rm::make_simulator<rm::SphericalModel, rm::NoneType>()), bool>::value,
                "unknown backend");
  sim->setModel(model);
  rm::Memory<rm::Transform, rm::RAM> T(20);
  for (int i = 0; i < 20; ++i) {
    T[i] = rm::Transform::Identity();
    T[i].t = {0.01f * i, -0.005f * i, 0.002f * i};
    T[i].R = {0.0f, 0.0f, std::sin(0.05f * i), std::cos(0.05f * i)};
  }
  const size_t n = model.size();
  auto full = sim->simulate<rm::Bundle<rm::Ranges<rm::RAM>, rm::FaceIds<rm::RAM>>>(T);
  // a slice of the poses gives the matching slice of the results
  rm::Bundle<rm::Ranges<rm::RAM>, rm::FaceIds<rm::RAM>> part;
  rm::resize_memory_bundle<rm::RAM>(part, model.getWidth(), model.getHeight(), 5);
  sim->simulate(T(10, 15), part);
  fail_if(std::memcmp(part.ranges.raw(), full.ranges.raw() + 10 * n, 5 * n * sizeof(float)) != 0, "slice ranges");
  fail_if(std::memcmp(part.face_ids.raw(), full.face_ids.raw() + 10 * n, 5 * n * 4) != 0, "slice face ids");
  // a view of const poses
  const rm::Memory<rm::Transform, rm::RAM>& Tc = T;
  rm::MemoryView<const rm::Transform, rm::RAM> cv = Tc(3, 4);
  auto one = sim->simulate<rm::Bundle<rm::Ranges<rm::RAM>>>(cv);
  fail_if(std::memcmp(one.ranges.raw(), full.ranges.raw() + 3 * n, n * sizeof(float)) != 0, "const view");
  // pinned poses and a pinned bundle take the host form; managed poses the device form
  rm::Memory<rm::Transform, rm::RAM_CUDA> Tp;
  Tp = T;
  rm::Bundle<rm::Ranges<rm::RAM_CUDA>> pinned;
  rm::resize_memory_bundle<rm::RAM_CUDA>(pinned, model.getWidth(), model.getHeight(), 20);
  sim->simulate(Tp, pinned);
  fail_if(std::memcmp(pinned.ranges.raw(), full.ranges.raw(), 20 * n * sizeof(float)) != 0, "pinned kinds");
  rm::Memory<rm::Transform, rm::UNIFIED_CUDA> Tu;
  Tu = T;
  rm::Bundle<rm::Ranges<rm::UNIFIED_CUDA>> managed;
  rm::resize_memory_bundle<rm::UNIFIED_CUDA>(managed, model.getWidth(), model.getHeight(), 20);
  sim->simulate(Tu, managed);
  rm::cuda_check(cudaDeviceSynchronize(), "sync");
  fail_if(std::memcmp(managed.ranges.raw(), full.ranges.raw(), 20 * n * sizeof(float)) != 0, "managed kinds");
  // setTsb from a view: the first transform
  rm::Memory<rm::Transform, rm::RAM> Tsb(2);
  Tsb[0] = rm::Transform::Identity();
  Tsb[0].t = {0.1f, 0.0f, 0.0f};
  Tsb[1] = rm::Transform::Identity();
  sim->setTsb(Tsb(0, 1));
  fail_if(sim->Tsb().t.x != 0.1f, "setTsb(MemoryView)");
  auto shifted = sim->simulate<rm::Bundle<rm::Ranges<rm::RAM>>>(rm::Transform::Identity());
  // the ray at theta = 0 (1 degree up) meets the cube's x = 0.5 wall: 0.1 m closer, range x 0.4 / 0.5
  const uint32_t fwd = model.getBufferId(model.phi.size / 2, model.theta.size / 2);
  fail_if(std::fabs(shifted.ranges[fwd] - 0.8f * full.ranges[fwd]) > 1e-5f, "setTsb moves the sensor");
}

// The differentiable forms: the range adjoint (device and host forms agree; a step against the
// gradient lowers the loss) and the Umeyama backward (exact translation identities).
static void test_gradients(const rm::MapPtr& map) {
  rm::SphericalModel model;
  model.theta = {(float)-M_PI, (float)(2.0 * M_PI / 256.0), 256};
  model.phi = {(float)(-60.0 * M_PI / 180.0), (float)(120.0 * M_PI / 180.0 / 31.0), 32};
  model.range = {0.0f, 100.0f};
  rm::SphereSimulatorGB300 sim(map);
  sim.setModel(model);
  rm::Memory<rm::Transform, rm::RAM> truth(4), est(4);
  for (int i = 0; i < 4; ++i) {
    truth[i] = rm::Transform::Identity();
    truth[i].t = {0.05f * i - 0.1f, 0.02f, -0.03f};
    est[i] = truth[i];
    est[i].t.x += 0.04f;
    est[i].t.z -= 0.03f;
  }
  auto obs = sim.simulate<rm::Bundle<rm::Ranges<rm::RAM>>>(truth);
  rm::Memory<float, rm::RAM> grad_h, loss_h;
  sim.rangePoseGrad(est, obs.ranges, 0.2f, grad_h, &loss_h);
  rm::Memory<rm::Transform, rm::VRAM_CUDA> est_d;
  est_d = est;
  rm::Memory<float, rm::VRAM_CUDA> obs_d, grad_d, loss_d;
  obs_d = obs.ranges;
  sim.rangePoseGrad(est_d, obs_d, 0.2f, grad_d, &loss_d);
  rm::Memory<float, rm::RAM> grad_b, loss_b;
  grad_b = grad_d;
  loss_b = loss_d;
  fail_if(std::memcmp(grad_b.raw(), grad_h.raw(), 24 * 4) != 0, "rangePoseGrad: host and device forms differ");
  fail_if(std::memcmp(loss_b.raw(), loss_h.raw(), 4 * 4) != 0, "rangePoseGrad: host and device losses differ");
  for (int i = 0; i < 4; ++i) {
    fail_if(!(loss_h[i] > 0.0f), "rangePoseGrad: loss");
    // the translation error is (+0.04, 0, -0.03): the gradient points along it
    fail_if(!(grad_h[6 * i + 0] > 0.0f && grad_h[6 * i + 2] < 0.0f), "rangePoseGrad: gradient direction");
  }
  // Umeyama backward: shifting all model points by d moves t by d (sum of model gradients = dL/dt);
  // shifting all dataset points by d moves t by -R d (sum of dataset gradients = -R^T dL/dt)
  const uint32_t N = 64;
  rm::Memory<rm::Vector3, rm::RAM> d(N), m(N);
  for (uint32_t i = 0; i < N; ++i) {
    const float a = 0.37f * i, b = 0.11f * i * i;
    d[i] = {std::cos(a) * 3.0f, std::sin(b) * 2.0f, 0.05f * i};
    m[i] = {-d[i].y + 1.0f, d[i].x - 0.5f, d[i].z + 0.25f};  // 90 degrees about z, shifted
  }
  rm::Memory<rm::Vector3, rm::VRAM_CUDA> dd, md, gd, gm;
  dd = d;
  md = m;
  rm::Memory<rm::CrossStatistics, rm::VRAM_CUDA> st;
  rm::Memory<rm::Transform, rm::VRAM_CUDA> Td;
  const rm::UmeyamaReductionConstraints params{1e30f, 0, 0};
  rm::statistics_p2p(dd, md, params, 1, st, &Td);
  rm::Memory<float, rm::RAM> gR_h(9), gt_h(3);
  for (int k = 0; k < 9; ++k) gR_h[k] = 0.1f * (k - 4);
  gt_h[0] = 1.0f; gt_h[1] = -2.0f; gt_h[2] = 0.5f;
  rm::Memory<float, rm::VRAM_CUDA> gR, gt;
  gR = gR_h;
  gt = gt_h;
  rm::umeyama_backward(dd, md, params, 1, st, &gR, &gt, &gd, &gm);
  rm::Memory<rm::Vector3, rm::RAM> gd_h, gm_h;
  gd_h = gd;
  gm_h = gm;
  double sm[3] = {0, 0, 0}, sd[3] = {0, 0, 0};
  for (uint32_t i = 0; i < N; ++i) {
    sm[0] += gm_h[i].x; sm[1] += gm_h[i].y; sm[2] += gm_h[i].z;
    sd[0] += gd_h[i].x; sd[1] += gd_h[i].y; sd[2] += gd_h[i].z;
  }
  // R = 90 degrees about z: R^T gt = (gt.y, -gt.x, gt.z)
  const double want_d[3] = {-gt_h[1], gt_h[0], -gt_h[2]};
  for (int k = 0; k < 3; ++k) {
    fail_if(std::fabs(sm[k] - gt_h[k]) > 1e-4, "umeyama_backward: sum of model gradients");
    fail_if(std::fabs(sd[k] - want_d[k]) > 1e-4, "umeyama_backward: sum of dataset gradients");
  }
}

// Batched SVD of rmagine's column-major Matrix3x3 records (tests/cuda/math_svd.cpp:38-109).
static void test_svd() {
  const size_t n = 1000;
  rm::Memory<float, rm::RAM> A(9 * n);
  uint32_t x = 12345u;
  for (size_t i = 0; i < 9 * n; ++i) {
    x = x * 1664525u + 1013904223u;
    A[i] = (float)((x >> 8) * (1.0 / 16777216.0) * 2.0 - 1.0);
  }
  rm::Memory<float, rm::VRAM_CUDA> Ad, Ud, Wd, Vd;
  Ad = A;
  rm::svd(Ad, Ud, Wd, Vd);
  rm::Memory<float, rm::RAM> U, W, V;
  U = Ud;
  W = Wd;
  V = Vd;
  double err = 0.0;
  for (size_t b = 0; b < n; ++b) {
    const float* u = U.raw() + 9 * b;  // column-major: element (r, c) at 3 c + r
    const float* w = W.raw() + 9 * b;
    const float* v = V.raw() + 9 * b;
    fail_if(w[0] < w[4] || w[4] < w[8] || w[8] < 0.0f, "svd: W sorted, non-negative");
    for (int r = 0; r < 3; ++r)
      for (int c = 0; c < 3; ++c) {
        double acc = 0.0;
        for (int k = 0; k < 3; ++k) acc += (double)u[3 * k + r] * w[4 * k] * v[3 * k + c];
        err = std::fmax(err, std::fabs(acc - A[9 * b + 3 * c + r]));
      }
  }
  fail_if(err > 2e-6, "svd: U W V^T != A");
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
    test_views_kinds_and_factory(map);
    test_gradients(map);
    test_svd();
    fail_if(map->status() != 0, "device status");
  } catch (const std::exception& e) {
    std::fprintf(stderr, "FAILED: %s\n", e.what());
    return 1;
  }
  std::printf("C++ API tests passed\n");
  return 0;
}
