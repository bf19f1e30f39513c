// SphereSimulatorGB300: rmagine's spherical simulator on librmg_gb300 (include/rmg.h), written
// against rmagine's own types (Memory / MemoryView, Bundle, SphericalModel, Transform), as a
// maintainer would add it to rmagine beside rmagine_embree and rmagine_optix.  It keeps the
// interface of SphereSimulatorEmbree (SphereSimulatorEmbree.hpp:107-159, SimulatorEmbree.hpp:52-72)
// for RAM buffers and of SphereSimulatorOptix (SphereSimulatorOptix.hpp:141-160) for VRAM_CUDA
// buffers, and registers itself with rmagine's simulator factory (Simulator.hpp:52-78) under the
// computing backend tag GB300.  rmagine's Transform, Vector and Face are byte-compatible with
// rmg_transform, rmg_vec3 and rmg_face, so buffers pass through without conversion.
// Pinhole, O1Dn and OnDn follow the same pattern with RMG_MODEL_PINHOLE / _O1DN / _ONDN.
#pragma once

#include <cuda_runtime.h>
#include <rmg.h>

#include <cstring>
#include <memory>
#include <string>
#include <utility>

#include <rmagine/simulation/SimulationResults.hpp>
#include <rmagine/simulation/Simulator.hpp>
#include <rmagine/types/MemoryCuda.hpp>
#include <rmagine/types/mesh_types.h>
#include <rmagine/types/sensor_models.h>
#include <rmagine/util/exceptions.h>

namespace rmagine {

struct GB300 {};  // computing backend tag, beside Embree / Optix / Vulkan

static_assert(sizeof(Transform) == sizeof(rmg_transform), "Transform == rmg_transform");
static_assert(sizeof(Vector) == sizeof(rmg_vec3) && sizeof(Face) == sizeof(rmg_face), "layouts");

inline void rmg_check(int st) {  // the RM_THROW convention (util/exceptions.h:48)
  if (st != RMG_OK) RM_THROW(CudaException, std::string(rmg_status_string(st)) + ": " + rmg_last_error());
}

// One triangle mesh with its BVH on the GPU (replaces EmbreeMap / OptixMap for a single mesh).
class GB300Map {
public:
  GB300Map(const MemoryView<Vector, RAM>& vertices, const MemoryView<Face, RAM>& faces) {
    rmg_check(rmg_map_build(reinterpret_cast<const rmg_vec3*>(vertices.raw()), (uint32_t)vertices.size(),
                            reinterpret_cast<const rmg_face*>(faces.raw()), (uint32_t)faces.size(), nullptr, &m_h));
  }
  ~GB300Map() { rmg_map_destroy(m_h); }
  GB300Map(const GB300Map&) = delete;
  GB300Map& operator=(const GB300Map&) = delete;
  rmg_map* handle() const { return m_h; }

private:
  rmg_map* m_h = nullptr;
};
using GB300MapPtr = std::shared_ptr<GB300Map>;

// The buffers of a bundle that the simulators fill: non-empty MemT attributes (rmg_outputs
// requests exactly the non-NULL ones, as set_simulation_flags_ does with sizes).
template<typename MemT, typename BundleT>
rmg_outputs rmg_outputs_of(BundleT& ret) {
  rmg_outputs o{};
  if constexpr (BundleT::template has<Hits<MemT>>())
    o.hits = ret.Hits<MemT>::hits.size() ? ret.Hits<MemT>::hits.raw() : nullptr;
  if constexpr (BundleT::template has<Ranges<MemT>>())
    o.ranges = ret.Ranges<MemT>::ranges.size() ? ret.Ranges<MemT>::ranges.raw() : nullptr;
  if constexpr (BundleT::template has<Points<MemT>>())
    o.points = ret.Points<MemT>::points.size() ? reinterpret_cast<rmg_vec3*>(ret.Points<MemT>::points.raw()) : nullptr;
  if constexpr (BundleT::template has<Normals<MemT>>())
    o.normals = ret.Normals<MemT>::normals.size() ? reinterpret_cast<rmg_vec3*>(ret.Normals<MemT>::normals.raw())
                                                  : nullptr;
  if constexpr (BundleT::template has<FaceIds<MemT>>())
    o.face_ids = ret.FaceIds<MemT>::face_ids.size() ? ret.FaceIds<MemT>::face_ids.raw() : nullptr;
  if constexpr (BundleT::template has<GeomIds<MemT>>())
    o.geom_ids = ret.GeomIds<MemT>::geom_ids.size() ? ret.GeomIds<MemT>::geom_ids.raw() : nullptr;
  if constexpr (BundleT::template has<ObjectIds<MemT>>())
    o.object_ids = ret.ObjectIds<MemT>::object_ids.size() ? ret.ObjectIds<MemT>::object_ids.raw() : nullptr;
  return o;
}

class SphereSimulatorGB300 {
public:
  SphereSimulatorGB300() = default;
  explicit SphereSimulatorGB300(GB300MapPtr map) : m_map(std::move(map)) {}
  ~SphereSimulatorGB300() { rmg_sensor_destroy(m_sensor); }
  SphereSimulatorGB300(const SphereSimulatorGB300&) = delete;
  SphereSimulatorGB300& operator=(const SphereSimulatorGB300&) = delete;

  void setMap(GB300MapPtr map) { m_map = std::move(map); }
  GB300MapPtr map() const { return m_map; }

  void setTsb(const Transform& Tsb) { std::memcpy(&m_Tsb, &Tsb, sizeof(m_Tsb)); }
  void setTsb(const MemoryView<Transform, RAM>& Tsb) { setTsb(Tsb[0]); }

  void setModel(const SphericalModel& m) {
    rmg_model c{};
    c.kind = RMG_MODEL_SPHERICAL;
    c.phi = {m.phi.min, m.phi.inc, m.phi.size};
    c.theta = {m.theta.min, m.theta.inc, m.theta.size};
    c.range = {m.range.min, m.range.max};
    rmg_sensor* s = nullptr;
    rmg_check(rmg_sensor_create(&c, nullptr, &s));
    rmg_sensor_destroy(m_sensor);
    m_sensor = s;
    m_model = m;
  }
  void setModel(const MemoryView<SphericalModel, RAM>& m) { setModel(m[0]); }
  SphericalModel model() const { return m_model; }

  // Device form (SphereSimulatorOptix.hpp:141-160): poses and results in VRAM_CUDA; asynchronous
  // on `stream`, like optixLaunch.
  template<typename BundleT>
  void simulate(const MemoryView<Transform, VRAM_CUDA>& Tbm, BundleT& ret, cudaStream_t stream = 0) const {
    const rmg_outputs o = rmg_outputs_of<VRAM_CUDA>(ret);
    rmg_check(rmg_simulate(m_map->handle(), m_sensor, &m_Tsb, reinterpret_cast<const rmg_transform*>(Tbm.raw()),
                           (uint32_t)Tbm.size(), &o, stream));
  }

  // Host form (SphereSimulatorEmbree.hpp:140-155): poses and results in RAM; returns when the
  // bundle is filled (pose chunks are cast while earlier chunks are copied back).
  template<typename BundleT>
  void simulate(const MemoryView<const Transform, RAM>& Tbm, BundleT& ret) const {
    const rmg_outputs o = rmg_outputs_of<RAM>(ret);
    rmg_check(rmg_simulate_host(m_map->handle(), m_sensor, &m_Tsb, reinterpret_cast<const rmg_transform*>(Tbm.raw()),
                                (uint32_t)Tbm.size(), &o, nullptr, nullptr));
  }

  template<typename BundleT>
  void simulate(const MemoryView<Transform, RAM>& Tbm, BundleT& ret) const {
    simulate(MemoryView<const Transform, RAM>(Tbm.raw(), Tbm.size()), ret);
  }

  template<typename BundleT>
  BundleT simulate(const MemoryView<Transform, RAM>& Tbm) const {
    BundleT res;
    resize_memory_bundle<RAM>(res, m_model.getWidth(), m_model.getHeight(), Tbm.size());
    simulate(Tbm, res);
    return res;
  }

  // One pose (SphereSimulatorEmbree.hpp:128-135).
  template<typename BundleT>
  void simulate(const Transform& Tbm, BundleT& ret) const {
    simulate(MemoryView<const Transform, RAM>(&Tbm, 1), ret);
  }

private:
  GB300MapPtr m_map;
  rmg_sensor* m_sensor = nullptr;
  rmg_transform m_Tsb{{0.f, 0.f, 0.f, 1.f}, {0.f, 0.f, 0.f}, 0};
  SphericalModel m_model{};
};
using SphereSimulatorGB300Ptr = std::shared_ptr<SphereSimulatorGB300>;

// make_simulator<SphericalModel, GB300>() (Simulator.hpp:52-78)
template<>
class SimulatorType<SphericalModel, GB300> {
public:
  using Class = SphereSimulatorGB300;
  using Ptr = SphereSimulatorGB300Ptr;
};

}  // namespace rmagine
