// Compiles and links integration/SphereSimulatorGB300.hpp -- the rmagine-side binding -- against
// rmagine's own headers and librmg_gb300.so: every overload is instantiated with rmagine's
// Bundle / Memory / MemoryView types.  Run with "run" as the first argument (needs a GPU) it
// simulates rmagine's unit-cube known answer (tests/embree/simulation_spherical.cpp:57-66).
#include "SphereSimulatorGB300.hpp"

#include <cmath>
#include <cstdio>
#include <cstring>

namespace rm = rmagine;

using DevBundle = rm::Bundle<rm::Hits<rm::VRAM_CUDA>, rm::Ranges<rm::VRAM_CUDA>, rm::Points<rm::VRAM_CUDA>,
                             rm::Normals<rm::VRAM_CUDA>, rm::FaceIds<rm::VRAM_CUDA>>;
using RamBundle = rm::Bundle<rm::Hits<rm::RAM>, rm::Ranges<rm::RAM>, rm::Points<rm::RAM>, rm::Normals<rm::RAM>,
                             rm::FaceIds<rm::RAM>, rm::GeomIds<rm::RAM>, rm::ObjectIds<rm::RAM>>;

template void rm::SphereSimulatorGB300::simulate<DevBundle>(const rm::MemoryView<rm::Transform, rm::VRAM_CUDA>&,
                                                            DevBundle&, cudaStream_t) const;
template void rm::SphereSimulatorGB300::simulate<RamBundle>(const rm::MemoryView<const rm::Transform, rm::RAM>&,
                                                            RamBundle&) const;

int main(int argc, char** argv) {
  if (argc < 2 || std::strcmp(argv[1], "run") != 0) return 0;
  // rmagine's genCube (synthetic.cpp:183-221)
  rm::Memory<rm::Vector, rm::RAM> V(8);
  const float c[8][3] = {{-0.5f, -0.5f, -0.5f}, {-0.5f, -0.5f, 0.5f}, {-0.5f, 0.5f, 0.5f}, {-0.5f, 0.5f, -0.5f},
                         {0.5f, 0.5f, -0.5f},   {0.5f, 0.5f, 0.5f},   {0.5f, -0.5f, 0.5f}, {0.5f, -0.5f, -0.5f}};
  for (int i = 0; i < 8; ++i) V[i] = rm::Vector{c[i][0], c[i][1], c[i][2]};
  const unsigned f[12][3] = {{0, 1, 2}, {2, 3, 0}, {4, 5, 6}, {6, 7, 4}, {0, 7, 1}, {1, 7, 6},
                             {1, 6, 5}, {5, 2, 1}, {2, 5, 4}, {3, 2, 4}, {3, 4, 7}, {3, 7, 0}};
  rm::Memory<rm::Face, rm::RAM> F(12);
  for (int i = 0; i < 12; ++i) F[i] = rm::Face{f[i][0], f[i][1], f[i][2]};
  auto map = std::make_shared<rm::GB300Map>(V, F);
  rm::SphericalModel model;  // example_spherical (sensors.cpp:39-54)
  model.theta.min = -M_PI;
  model.theta.inc = 0.4 * M_PI / 180.0;
  model.theta.size = 900;
  model.phi.min = -15.0 * M_PI / 180.0;
  model.phi.inc = 2.0 * M_PI / 180.0;
  model.phi.size = 16;
  model.range.min = 0.0;
  model.range.max = 100.0;
  auto sim = rm::make_simulator<rm::SphericalModel, rm::GB300>();
  sim->setMap(map);
  sim->setModel(model);
  rm::Memory<rm::Transform, rm::RAM> Tbm(100);
  for (size_t i = 0; i < Tbm.size(); ++i) Tbm[i] = rm::Transform::Identity();
  RamBundle res = sim->simulate<RamBundle>(Tbm);
  const float r = res.ranges[model.getBufferId(8, 0)];
  std::printf("range %f (rmagine's known answer 0.500076)\n", r);
  return std::fabs(r - 0.500076f) < 1e-4f ? 0 : 1;
}
