// rmagine_gb300.hpp -- header-only C++ layer over the C ABI (rmg.h), with
// rmagine's types and simulator interface, so that C++ code written against
// rmagine's simulators (SphereSimulatorEmbree / SphereSimulatorOptix and
// siblings) switches by changing the simulator type.
//
// Mirrors (uos/rmagine v2.4.2):
//   Memory<T, RAM | VRAM_CUDA |
//          RAM_CUDA | UNIFIED_CUDA>  types/Memory.hpp:59-266, types/MemoryCuda.hpp:66-100
//   MemoryView<T, MemT>, slice,
//     operator()(a, b)               types/Memory.hpp:60-173
//   SimulatorType / Simulator /
//     make_simulator<ModelT, CompT>  simulation/Simulator.hpp:52-78 (CompT = GB300)
//   Bundle / Hits / Ranges / ...     types/Bundle.hpp:72-131, simulation/SimulationResults.hpp:56-215
//   resize_memory_bundle             SimulationResults.hpp:176-215
//   SphericalModel / PinholeModel /
//   O1DnModel / OnDnModel            types/sensor_models.h:54-502
//   Transform / Quaternion / Vector3 math/types/Transform.hpp, Quaternion.hpp, Vector3.hpp (data layout)
//   SimulatorX::setMap/setTsb/
//     setModel/simulate              SimulatorEmbree.hpp:52-72, SphereSimulatorEmbree.hpp:107-159,
//                                    SphereSimulatorOptix.hpp:122-190
//   statistics_p2p / _p2l / umeyama  math/statistics.h:72-157, math/optimization.h:61-75
//   svd (batched 3x3)                 rmagine_cuda math/memory_math.cuh:561-578, math/linalg.h:164-175
//   rangePoseGrad / umeyama_backward  no counterpart (the differentiable forms of simulate and
//                                     of statistics_p2p + umeyama_transform)
//   InstancedScene / Instance        EmbreeScene / EmbreeInstance (map/embree/EmbreeScene.hpp,
//                                    EmbreeInstance.hpp), OptixScene instances
//   GaussianNoiseGB300 / ...         noise/GaussianNoiseCuda.hpp, RelGaussianNoiseCuda.hpp,
//                                    UniformDustNoiseCuda.hpp, Noise.hpp (Options)
//   read_mesh / import_map           AssimpIO::ReadFile + import_embree_map (EmbreeMap.hpp:94-117)
// Errors throw rmagine_gb300::Exception, as rmagine's RM_THROW does (util/exceptions.h:48).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <cstring>
#include <memory>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <vector>

#include "rmg.h"

namespace rmagine_gb300 {

class Exception : public std::runtime_error {
 public:
  Exception(int status, const std::string& what) : std::runtime_error(what), status(status) {}
  int status;
};

inline void check(int st, const char* where) {
  if (st != RMG_OK)
    throw Exception(st, std::string(where) + ": " + rmg_status_string(st) + " (" + rmg_last_error() + ")");
}

inline void cuda_check(cudaError_t e, const char* where) {
  if (e != cudaSuccess) throw Exception(RMG_ERR_CUDA, std::string(where) + ": " + cudaGetErrorString(e));
}

// ---- plain data (byte-compatible with rmagine and with rmg.h) --------------------
struct Vector3 {
  float x, y, z;
};
struct Quaternion {
  float x, y, z, w;
  static Quaternion Identity() { return {0.f, 0.f, 0.f, 1.f}; }
};
struct Transform {
  Quaternion R;
  Vector3 t;
  uint32_t stamp;
  static Transform Identity() { return {Quaternion::Identity(), {0.f, 0.f, 0.f}, 0}; }
};
struct Face {
  uint32_t v0, v1, v2;
};
using Vector = Vector3;
static_assert(sizeof(Transform) == sizeof(rmg_transform), "Transform is 32 bytes");
static_assert(sizeof(Vector3) == sizeof(rmg_vec3) && sizeof(Face) == sizeof(rmg_face), "layouts");

struct Interval {
  float min, max;
};
struct DiscreteInterval {
  float min, inc;
  uint32_t size;
  float getValue(uint32_t i) const { return min + static_cast<float>(i) * inc; }
};

// ---- memory -----------------------------------------------------------------------
// Memory kinds (rmagine's memory tags): RAM (pageable host), VRAM_CUDA (device), RAM_CUDA
// (pinned host, MemoryCuda.hpp:78), UNIFIED_CUDA (managed, MemoryCuda.hpp:89).
struct RAM {};
struct VRAM_CUDA {};
struct RAM_CUDA {};
struct UNIFIED_CUDA {};

// Host-side memory kinds take the host forms of the calls; device-side ones the device forms.
template <typename MemT> struct host_memory : std::false_type {};
template <> struct host_memory<RAM> : std::true_type {};
template <> struct host_memory<RAM_CUDA> : std::true_type {};

// A non-owning window of n elements (MemoryView, types/Memory.hpp:60-173): what rmagine's
// simulate / setTsb / setModel overloads take.  A view of const T binds to a view of T.
template <typename T, typename MemT = RAM>
class MemoryView {
 public:
  using DataType = T;
  using MemType = MemT;
  MemoryView(T* mem, size_t n) : p_(mem), n_(n) {}
  template <typename U, typename = std::enable_if_t<std::is_same<const U, T>::value>>
  MemoryView(const MemoryView<U, MemT>& o) : p_(o.raw()), n_(o.size()) {}
  static MemoryView Empty() { return MemoryView(nullptr, 0); }
  bool empty() const { return p_ == nullptr; }
  T* raw() const { return p_; }
  size_t size() const { return n_; }
  T& operator[](size_t i) const { return p_[i]; }  // host-accessible kinds only
  MemoryView slice(size_t a, size_t b) const { return MemoryView(p_ + a, b - a); }
  MemoryView operator()(size_t a, size_t b) const { return slice(a, b); }

 private:
  T* p_ = nullptr;
  size_t n_ = 0;
};

template <typename T, typename MemT>
class Memory;

// Views, slices and conversions shared by every owning Memory kind.
template <typename T, typename MemT, typename Derived>
struct MemoryViews {
  operator MemoryView<T, MemT>() { return MemoryView<T, MemT>(self().raw(), self().size()); }
  operator MemoryView<const T, MemT>() const { return MemoryView<const T, MemT>(self().raw(), self().size()); }
  MemoryView<T, MemT> view() { return *this; }
  MemoryView<const T, MemT> view() const { return *this; }
  MemoryView<T, MemT> slice(size_t a, size_t b) { return MemoryView<T, MemT>(self().raw() + a, b - a); }
  MemoryView<const T, MemT> slice(size_t a, size_t b) const {
    return MemoryView<const T, MemT>(self().raw() + a, b - a);
  }
  MemoryView<T, MemT> operator()(size_t a, size_t b) { return slice(a, b); }
  MemoryView<const T, MemT> operator()(size_t a, size_t b) const { return slice(a, b); }

 private:
  Derived& self() { return static_cast<Derived&>(*this); }
  const Derived& self() const { return static_cast<const Derived&>(*this); }
};

template <typename T>
class Memory<T, RAM> : public MemoryViews<T, RAM, Memory<T, RAM>> {
 public:
  Memory() = default;
  explicit Memory(size_t n) : v_(n) {}
  void resize(size_t n) { v_.resize(n); }
  size_t size() const { return v_.size(); }
  T* raw() { return v_.data(); }
  const T* raw() const { return v_.data(); }
  T& operator[](size_t i) { return v_[i]; }
  const T& operator[](size_t i) const { return v_[i]; }
  template <typename MemT2>
  Memory& operator=(const Memory<T, MemT2>& o);

 private:
  std::vector<T> v_;
};

// cudaMalloc'd (VRAM_CUDA), cudaMallocHost'd (RAM_CUDA) or cudaMallocManaged (UNIFIED_CUDA) storage.
template <typename T, typename MemT>
class CudaMemory : public MemoryViews<T, MemT, Memory<T, MemT>> {
 public:
  CudaMemory() = default;
  explicit CudaMemory(size_t n) { resize(n); }
  CudaMemory(const CudaMemory&) = delete;
  CudaMemory& operator=(const CudaMemory&) = delete;
  CudaMemory(CudaMemory&& o) noexcept : p_(o.p_), n_(o.n_) { o.p_ = nullptr; o.n_ = 0; }
  ~CudaMemory() { release(); }
  void resize(size_t n) {
    if (n == n_) return;
    release();
    if (n) {
      void* p = nullptr;
      if constexpr (std::is_same<MemT, RAM_CUDA>::value) cuda_check(cudaMallocHost(&p, n * sizeof(T)), "cudaMallocHost");
      else if constexpr (std::is_same<MemT, UNIFIED_CUDA>::value)
        cuda_check(cudaMallocManaged(&p, n * sizeof(T)), "cudaMallocManaged");
      else cuda_check(cudaMalloc(&p, n * sizeof(T)), "cudaMalloc");
      p_ = static_cast<T*>(p);
    }
    n_ = n;
  }
  size_t size() const { return n_; }
  T* raw() { return p_; }
  const T* raw() const { return p_; }

 protected:
  void release() {
    if (p_) {
      if constexpr (std::is_same<MemT, RAM_CUDA>::value) cudaFreeHost(p_);
      else cudaFree(p_);
    }
    p_ = nullptr;
    n_ = 0;
  }
  T* p_ = nullptr;
  size_t n_ = 0;
};

// Assignment between any two kinds copies (MemoryCuda.cu:10-90 semantics).
template <typename T, typename MemT, typename MemT2, typename Dst, typename Src>
void copy_memory(Dst& dst, const Src& src) {
  dst.resize(src.size());
  if (src.size())
    cuda_check(cudaMemcpy(dst.raw(), src.raw(), src.size() * sizeof(T), cudaMemcpyDefault), "cudaMemcpy");
}

template <typename T>
class Memory<T, VRAM_CUDA> : public CudaMemory<T, VRAM_CUDA> {
 public:
  using CudaMemory<T, VRAM_CUDA>::CudaMemory;
  Memory() = default;
  Memory(Memory&&) noexcept = default;
  template <typename MemT2>
  Memory& operator=(const Memory<T, MemT2>& o) { copy_memory<T, VRAM_CUDA, MemT2>(*this, o); return *this; }
};

template <typename T>
class Memory<T, RAM_CUDA> : public CudaMemory<T, RAM_CUDA> {
 public:
  using CudaMemory<T, RAM_CUDA>::CudaMemory;
  Memory() = default;
  Memory(Memory&&) noexcept = default;
  T& operator[](size_t i) { return this->p_[i]; }
  const T& operator[](size_t i) const { return this->p_[i]; }
  template <typename MemT2>
  Memory& operator=(const Memory<T, MemT2>& o) { copy_memory<T, RAM_CUDA, MemT2>(*this, o); return *this; }
};

template <typename T>
class Memory<T, UNIFIED_CUDA> : public CudaMemory<T, UNIFIED_CUDA> {
 public:
  using CudaMemory<T, UNIFIED_CUDA>::CudaMemory;
  Memory() = default;
  Memory(Memory&&) noexcept = default;
  T& operator[](size_t i) { return this->p_[i]; }  // after a device synchronisation
  const T& operator[](size_t i) const { return this->p_[i]; }
  template <typename MemT2>
  Memory& operator=(const Memory<T, MemT2>& o) { copy_memory<T, UNIFIED_CUDA, MemT2>(*this, o); return *this; }
};

template <typename T>
template <typename MemT2>
Memory<T, RAM>& Memory<T, RAM>::operator=(const Memory<T, MemT2>& o) {
  copy_memory<T, RAM, MemT2>(*this, o);
  return *this;
}

// Element type and memory kind of a pose buffer (Memory or MemoryView of Transform).
template <typename P> struct pose_buffer : std::false_type {};
template <typename MemT> struct pose_buffer<MemoryView<Transform, MemT>> : std::true_type { using Mem = MemT; };
template <typename MemT> struct pose_buffer<MemoryView<const Transform, MemT>> : std::true_type { using Mem = MemT; };
template <typename MemT> struct pose_buffer<Memory<Transform, MemT>> : std::true_type { using Mem = MemT; };

// ---- result attributes and bundles ---------------------------------------------------
template <typename MemT> struct Hits { Memory<uint8_t, MemT> hits; };
template <typename MemT> struct Ranges { Memory<float, MemT> ranges; };
template <typename MemT> struct Points { Memory<Vector3, MemT> points; };
template <typename MemT> struct Normals { Memory<Vector3, MemT> normals; };
template <typename MemT> struct FaceIds { Memory<uint32_t, MemT> face_ids; };
template <typename MemT> struct GeomIds { Memory<uint32_t, MemT> geom_ids; };
template <typename MemT> struct ObjectIds { Memory<uint32_t, MemT> object_ids; };

template <typename... Attrs>
struct Bundle : public Attrs... {
  template <typename A>
  static constexpr bool has() { return (std::is_same<A, Attrs>::value || ...); }
};

template <typename MemT>
using IntAttrAll = Bundle<Hits<MemT>, Ranges<MemT>, Points<MemT>, Normals<MemT>, FaceIds<MemT>, GeomIds<MemT>,
                          ObjectIds<MemT>>;

template <typename MemT, typename BundleT>
void resize_memory_bundle(BundleT& res, unsigned W, unsigned H, unsigned N = 1) {
  const size_t n = (size_t)W * H * N;
  if constexpr (BundleT::template has<Hits<MemT>>()) res.Hits<MemT>::hits.resize(n);
  if constexpr (BundleT::template has<Ranges<MemT>>()) res.Ranges<MemT>::ranges.resize(n);
  if constexpr (BundleT::template has<Points<MemT>>()) res.Points<MemT>::points.resize(n);
  if constexpr (BundleT::template has<Normals<MemT>>()) res.Normals<MemT>::normals.resize(n);
  if constexpr (BundleT::template has<FaceIds<MemT>>()) res.FaceIds<MemT>::face_ids.resize(n);
  if constexpr (BundleT::template has<GeomIds<MemT>>()) res.GeomIds<MemT>::geom_ids.resize(n);
  if constexpr (BundleT::template has<ObjectIds<MemT>>()) res.ObjectIds<MemT>::object_ids.resize(n);
}

// rmg_outputs of a bundle's MemT buffers: a buffer is requested iff it is non-empty
// (set_simulation_flags_, embree_common.h:79-139).
template <typename M = VRAM_CUDA, typename BundleT>
rmg_outputs outputs_of(BundleT& b) {
  rmg_outputs o{};
  if constexpr (BundleT::template has<Hits<M>>()) o.hits = b.Hits<M>::hits.size() ? b.Hits<M>::hits.raw() : nullptr;
  if constexpr (BundleT::template has<Ranges<M>>())
    o.ranges = b.Ranges<M>::ranges.size() ? b.Ranges<M>::ranges.raw() : nullptr;
  if constexpr (BundleT::template has<Points<M>>())
    o.points = b.Points<M>::points.size() ? reinterpret_cast<rmg_vec3*>(b.Points<M>::points.raw()) : nullptr;
  if constexpr (BundleT::template has<Normals<M>>())
    o.normals = b.Normals<M>::normals.size() ? reinterpret_cast<rmg_vec3*>(b.Normals<M>::normals.raw()) : nullptr;
  if constexpr (BundleT::template has<FaceIds<M>>())
    o.face_ids = b.FaceIds<M>::face_ids.size() ? b.FaceIds<M>::face_ids.raw() : nullptr;
  if constexpr (BundleT::template has<GeomIds<M>>())
    o.geom_ids = b.GeomIds<M>::geom_ids.size() ? b.GeomIds<M>::geom_ids.raw() : nullptr;
  if constexpr (BundleT::template has<ObjectIds<M>>())
    o.object_ids = b.ObjectIds<M>::object_ids.size() ? b.ObjectIds<M>::object_ids.raw() : nullptr;
  return o;
}

inline void merge_outputs(rmg_outputs& o, const rmg_outputs& b) {
  if (!o.hits) o.hits = b.hits;
  if (!o.ranges) o.ranges = b.ranges;
  if (!o.points) o.points = b.points;
  if (!o.normals) o.normals = b.normals;
  if (!o.face_ids) o.face_ids = b.face_ids;
  if (!o.geom_ids) o.geom_ids = b.geom_ids;
  if (!o.object_ids) o.object_ids = b.object_ids;
}

// The bundle's buffers that the host forms fill (RAM and RAM_CUDA attributes) and those the device
// forms fill (VRAM_CUDA and UNIFIED_CUDA attributes).
template <bool Host, typename BundleT>
rmg_outputs outputs_for(BundleT& b) {
  rmg_outputs o = outputs_of<std::conditional_t<Host, RAM, VRAM_CUDA>>(b);
  merge_outputs(o, outputs_of<std::conditional_t<Host, RAM_CUDA, UNIFIED_CUDA>>(b));
  return o;
}

// Resizes every non-empty MemT buffer of a bundle to n elements (the requested ones).
template <typename M, typename BundleT>
void resize_requested(BundleT& b, size_t n) {
  if constexpr (BundleT::template has<Hits<M>>()) if (b.Hits<M>::hits.size()) b.Hits<M>::hits.resize(n);
  if constexpr (BundleT::template has<Ranges<M>>()) if (b.Ranges<M>::ranges.size()) b.Ranges<M>::ranges.resize(n);
  if constexpr (BundleT::template has<Points<M>>()) if (b.Points<M>::points.size()) b.Points<M>::points.resize(n);
  if constexpr (BundleT::template has<Normals<M>>()) if (b.Normals<M>::normals.size()) b.Normals<M>::normals.resize(n);
  if constexpr (BundleT::template has<FaceIds<M>>()) if (b.FaceIds<M>::face_ids.size()) b.FaceIds<M>::face_ids.resize(n);
  if constexpr (BundleT::template has<GeomIds<M>>()) if (b.GeomIds<M>::geom_ids.size()) b.GeomIds<M>::geom_ids.resize(n);
  if constexpr (BundleT::template has<ObjectIds<M>>())
    if (b.ObjectIds<M>::object_ids.size()) b.ObjectIds<M>::object_ids.resize(n);
}

// ---- sensor models ---------------------------------------------------------------------
struct SphericalModel {
  DiscreteInterval phi, theta;
  Interval range;
  uint32_t getWidth() const { return theta.size; }
  uint32_t getHeight() const { return phi.size; }
  uint32_t size() const { return getWidth() * getHeight(); }
  uint32_t getBufferId(uint32_t vid, uint32_t hid) const { return vid * getWidth() + hid; }
  rmg_model to_c() const {
    rmg_model m{};
    m.kind = RMG_MODEL_SPHERICAL;
    m.range = {range.min, range.max};
    m.phi = {phi.min, phi.inc, phi.size};
    m.theta = {theta.min, theta.inc, theta.size};
    return m;
  }
};

struct PinholeModel {
  uint32_t width, height;
  Interval range;
  float f[2], c[2];
  uint32_t getWidth() const { return width; }
  uint32_t getHeight() const { return height; }
  uint32_t size() const { return width * height; }
  uint32_t getBufferId(uint32_t vid, uint32_t hid) const { return vid * width + hid; }
  rmg_model to_c() const {
    rmg_model m{};
    m.kind = RMG_MODEL_PINHOLE;
    m.width = width;
    m.height = height;
    m.range = {range.min, range.max};
    m.f[0] = f[0]; m.f[1] = f[1]; m.c[0] = c[0]; m.c[1] = c[1];
    return m;
  }
};

struct O1DnModel {
  uint32_t width, height;
  Interval range;
  Vector3 orig;
  Memory<Vector3, RAM> dirs;
  uint32_t getWidth() const { return width; }
  uint32_t getHeight() const { return height; }
  uint32_t size() const { return width * height; }
  rmg_model to_c() const {
    rmg_model m{};
    m.kind = RMG_MODEL_O1DN;
    m.width = width;
    m.height = height;
    m.range = {range.min, range.max};
    m.orig = {orig.x, orig.y, orig.z};
    m.dirs = reinterpret_cast<const rmg_vec3*>(dirs.raw());
    return m;
  }
};

struct OnDnModel {
  uint32_t width, height;
  Interval range;
  Memory<Vector3, RAM> origs, dirs;
  uint32_t getWidth() const { return width; }
  uint32_t getHeight() const { return height; }
  uint32_t size() const { return width * height; }
  rmg_model to_c() const {
    rmg_model m{};
    m.kind = RMG_MODEL_ONDN;
    m.width = width;
    m.height = height;
    m.range = {range.min, range.max};
    m.dirs = reinterpret_cast<const rmg_vec3*>(dirs.raw());
    m.origs = reinterpret_cast<const rmg_vec3*>(origs.raw());
    return m;
  }
};

// ---- map -----------------------------------------------------------------------------------
class TriangleMap {
 public:
  // builder: RMG_BUILD_SAH (the default) or RMG_BUILD_LBVH; queries give the same results with either
  TriangleMap(const Memory<Vector3, RAM>& V, const Memory<Face, RAM>& F, cudaStream_t s = 0,
              rmg_builder builder = RMG_BUILD_SAH) {
    check(rmg_map_build_ex(reinterpret_cast<const rmg_vec3*>(V.raw()), (uint32_t)V.size(),
                           reinterpret_cast<const rmg_face*>(F.raw()), (uint32_t)F.size(), builder, s, &h_),
          "rmg_map_build_ex");
  }
  // adopts a handle (rmg_map_load); used by load()
  explicit TriangleMap(rmg_map* h) : h_(h) {}
  ~TriangleMap() { rmg_map_destroy(h_); }
  TriangleMap(const TriangleMap&) = delete;
  TriangleMap& operator=(const TriangleMap&) = delete;
  rmg_map* handle() const { return h_; }
  void refit(const Memory<Vector3, RAM>& V, cudaStream_t s = 0) {
    check(rmg_map_refit(h_, reinterpret_cast<const rmg_vec3*>(V.raw()), (uint32_t)V.size(), s), "rmg_map_refit");
  }
  int status(bool clear = true) { return rmg_map_status(h_, clear ? 1 : 0); }
  // the built map (mesh + tree) to a file, and back without a rebuild
  void save(const std::string& path) const { check(rmg_map_save(h_, path.c_str()), "rmg_map_save"); }
  static std::shared_ptr<TriangleMap> load(const std::string& path, cudaStream_t s = 0) {
    rmg_map* h = nullptr;
    check(rmg_map_load(path.c_str(), s, &h), "rmg_map_load");
    return std::make_shared<TriangleMap>(h);
  }

 private:
  rmg_map* h_ = nullptr;
};
using MapPtr = std::shared_ptr<TriangleMap>;

// ---- mesh files ---------------------------------------------------------------------
struct MeshData {
  Memory<Vector3, RAM> vertices;
  Memory<Face, RAM> faces;
  Memory<uint32_t, RAM> groups;  // group (OBJ object / group) of each face
  uint32_t n_groups = 0;
};

inline MeshData read_mesh(const std::string& path) {
  rmg_mesh m{};
  check(rmg_mesh_read(path.c_str(), &m), "rmg_mesh_read");
  MeshData out;
  out.vertices.resize(m.n_vertices);
  out.faces.resize(m.n_faces);
  out.groups.resize(m.n_faces);
  if (m.n_vertices) std::memcpy(out.vertices.raw(), m.vertices, sizeof(Vector3) * m.n_vertices);
  if (m.n_faces) {
    std::memcpy(out.faces.raw(), m.faces, sizeof(Face) * m.n_faces);
    std::memcpy(out.groups.raw(), m.face_group, 4ull * m.n_faces);
  }
  out.n_groups = m.n_groups;
  rmg_mesh_free(&m);
  return out;
}

inline void write_ply(const std::string& path, const Memory<Vector3, RAM>& V, const Memory<Face, RAM>& F) {
  check(rmg_mesh_write_ply(path.c_str(), reinterpret_cast<const rmg_vec3*>(V.raw()), (uint32_t)V.size(),
                           reinterpret_cast<const rmg_face*>(F.raw()), (uint32_t)F.size()),
        "rmg_mesh_write_ply");
}

// import_embree_map for one mesh: every face of the file in one map.
inline MapPtr import_map(const std::string& path, cudaStream_t s = 0) {
  const MeshData m = read_mesh(path);
  return std::make_shared<TriangleMap>(m.vertices, m.faces, s);
}

// ---- instanced scenes ---------------------------------------------------------------
struct Instance {
  uint32_t geometry = 0;  // index into the scene's geometries
  uint32_t geom_id = 0;   // GeomIds of its hits
  uint32_t object_id = 0; // ObjectIds of its hits
  Transform T = Transform::Identity();
  Vector3 scale{1.f, 1.f, 1.f};
};

class InstancedScene {
 public:
  InstancedScene(std::vector<MapPtr> geometries, const std::vector<Instance>& instances, cudaStream_t s = 0)
      : geoms_(std::move(geometries)) {
    std::vector<const rmg_map*> h;
    for (const auto& g : geoms_) h.push_back(g->handle());
    const auto c = to_c(instances);
    check(rmg_scene_create(h.data(), (uint32_t)h.size(), c.data(), (uint32_t)c.size(), s, &h_), "rmg_scene_create");
  }
  ~InstancedScene() { rmg_scene_destroy(h_); }
  InstancedScene(const InstancedScene&) = delete;
  InstancedScene& operator=(const InstancedScene&) = delete;
  void update(const std::vector<Instance>& instances, bool rebuild = false, cudaStream_t s = 0) {
    const auto c = to_c(instances);
    check(rmg_scene_update(h_, c.data(), (uint32_t)c.size(), rebuild ? 1 : 0, s), "rmg_scene_update");
  }
  int status(bool clear = true) { return rmg_scene_status(h_, clear ? 1 : 0); }
  rmg_scene* handle() const { return h_; }

 private:
  static std::vector<rmg_instance_desc> to_c(const std::vector<Instance>& in) {
    std::vector<rmg_instance_desc> c(in.size());
    for (size_t i = 0; i < in.size(); ++i) {
      c[i].geometry = in[i].geometry;
      c[i].geom_id = in[i].geom_id;
      c[i].object_id = in[i].object_id;
      std::memcpy(&c[i].T, &in[i].T, sizeof(rmg_transform));
      c[i].scale = rmg_vec3{in[i].scale.x, in[i].scale.y, in[i].scale.z};
    }
    return c;
  }
  std::vector<MapPtr> geoms_;  // the scene references them
  rmg_scene* h_ = nullptr;
};
using ScenePtr = std::shared_ptr<InstancedScene>;

// ---- statistics types (used by the simulators' fused step) ------------------------------
struct CrossStatistics {
  Vector3 dataset_mean, model_mean;
  float covariance[9];  // column-major, like rmagine::Matrix3x3
  uint32_t n_meas;
};
static_assert(sizeof(CrossStatistics) == sizeof(rmg_cross_stats), "CrossStatistics is 64 bytes");

struct UmeyamaReductionConstraints {
  float max_dist;
  uint32_t dataset_id, model_id;
};

// ---- simulators ---------------------------------------------------------------------------
template <typename ModelT>
class SimulatorGB300 {
 public:
  SimulatorGB300() = default;
  explicit SimulatorGB300(MapPtr map) : map_(std::move(map)) {}
  ~SimulatorGB300() { rmg_sensor_destroy(sensor_); }
  SimulatorGB300(const SimulatorGB300&) = delete;
  SimulatorGB300& operator=(const SimulatorGB300&) = delete;

  void setMap(MapPtr map) { map_ = std::move(map); scene_.reset(); }
  // an instanced map (EmbreeMap over a scene with instances)
  void setMap(ScenePtr scene) { scene_ = std::move(scene); map_.reset(); }
  MapPtr map() const { return map_; }
  ScenePtr scene() const { return scene_; }
  // Fastest launch configuration for these poses and outputs (rmg_autotune_launch_config);
  // kept for later simulate calls.  Single-mesh maps.
  template <typename BundleT>
  rmg_launch_config autotune(const Memory<Transform, VRAM_CUDA>& Tbm, BundleT& ret, uint32_t reps = 3,
                             cudaStream_t stream = 0) {
    ready();
    if (!map_) throw Exception(RMG_ERR_UNSUPPORTED, "autotune: needs a single-mesh map");
    const rmg_outputs o = outputs_of(ret);
    rmg_launch_config c{};
    check(rmg_autotune_launch_config(map_->handle(), sensor_, reinterpret_cast<const rmg_transform*>(&Tsb_),
                                     reinterpret_cast<const rmg_transform*>(Tbm.raw()), (uint32_t)Tbm.size(), &o,
                                     reps, &c, stream),
          "rmg_autotune_launch_config");
    cfg_ = c;
    tuned_ = true;
    return c;
  }
  // The correction loop's inner step fused (rmg_simulate_statistics): simulate at Tbm,
  // statistics_p2l (p2l) or _p2p against `dataset` (one scan of width*height points for every
  // pose, or one per pose when per_pose), optionally pre-transformed, and Umeyama.
  void simulateStatistics(const Memory<Transform, VRAM_CUDA>& Tbm, const Memory<Vector3, VRAM_CUDA>& dataset,
                          const Memory<uint8_t, VRAM_CUDA>* dataset_mask, bool per_pose,
                          const Memory<Transform, VRAM_CUDA>* pre, const UmeyamaReductionConstraints& params,
                          bool p2l, Memory<CrossStatistics, VRAM_CUDA>* stats, Memory<Transform, VRAM_CUDA>* Ts,
                          cudaStream_t stream = 0) const {
    ready();
    if (!map_) throw Exception(RMG_ERR_UNSUPPORTED, "simulateStatistics: needs a single-mesh map");
    if (stats) stats->resize(Tbm.size());
    if (Ts) Ts->resize(Tbm.size());
    const rmg_scan scan{reinterpret_cast<const rmg_vec3*>(dataset.raw()), dataset_mask ? dataset_mask->raw() : nullptr,
                        nullptr, per_pose ? 1u : 0u};
    const rmg_umeyama_constraints c{params.max_dist, params.dataset_id, params.model_id};
    check(rmg_simulate_statistics(map_->handle(), sensor_, reinterpret_cast<const rmg_transform*>(&Tsb_),
                                  reinterpret_cast<const rmg_transform*>(Tbm.raw()), (uint32_t)Tbm.size(), &scan,
                                  pre ? reinterpret_cast<const rmg_transform*>(pre->raw()) : nullptr,
                                  pre && pre->size() > 1 ? 1u : 0u, &c, p2l ? 1 : 0,
                                  stats ? reinterpret_cast<rmg_cross_stats*>(stats->raw()) : nullptr,
                                  Ts ? reinterpret_cast<rmg_transform*>(Ts->raw()) : nullptr, stream),
          "rmg_simulate_statistics");
  }
  // Host form of simulateStatistics (rmg_simulate_statistics_host): poses, scans and results in
  // RAM; per-pose scans are uploaded in chunks while earlier chunks are reduced.  Synchronises.
  void simulateStatistics(const Memory<Transform, RAM>& Tbm, const Memory<Vector3, RAM>& dataset,
                          const Memory<uint8_t, RAM>* dataset_mask, bool per_pose, const Memory<Transform, RAM>* pre,
                          const UmeyamaReductionConstraints& params, bool p2l, Memory<CrossStatistics, RAM>* stats,
                          Memory<Transform, RAM>* Ts, cudaStream_t stream = 0) const {
    ready();
    if (!map_) throw Exception(RMG_ERR_UNSUPPORTED, "simulateStatistics: needs a single-mesh map");
    if (stats) stats->resize(Tbm.size());
    if (Ts) Ts->resize(Tbm.size());
    const rmg_scan scan{reinterpret_cast<const rmg_vec3*>(dataset.raw()), dataset_mask ? dataset_mask->raw() : nullptr,
                        nullptr, per_pose ? 1u : 0u};
    const rmg_umeyama_constraints c{params.max_dist, params.dataset_id, params.model_id};
    check(rmg_simulate_statistics_host(map_->handle(), sensor_, reinterpret_cast<const rmg_transform*>(&Tsb_),
                                       reinterpret_cast<const rmg_transform*>(Tbm.raw()), (uint32_t)Tbm.size(), &scan,
                                       pre ? reinterpret_cast<const rmg_transform*>(pre->raw()) : nullptr,
                                       pre && pre->size() > 1 ? 1u : 0u, &c, p2l ? 1 : 0,
                                       stats ? reinterpret_cast<rmg_cross_stats*>(stats->raw()) : nullptr,
                                       Ts ? reinterpret_cast<rmg_transform*>(Ts->raw()) : nullptr, stream),
          "rmg_simulate_statistics_host");
  }
  void setTsb(const Transform& T) { Tsb_ = T; }
  // setTsb(MemoryView<Transform, RAM>) (SimulatorEmbree.hpp:60): the first transform.
  void setTsb(const MemoryView<const Transform, RAM>& T) {
    if (T.size() == 0) throw Exception(RMG_ERR_INVALID_ARG, "setTsb: no transform");
    Tsb_ = T[0];
  }
  void setTsb(const MemoryView<Transform, RAM>& T) { setTsb(MemoryView<const Transform, RAM>(T)); }
  void setTsb(const Memory<Transform, RAM>& T) { setTsb(T.view()); }
  const Transform& Tsb() const { return Tsb_; }
  // setModel(MemoryView<ModelT, RAM>) (SphereSimulatorEmbree.hpp:115): the first model.
  void setModel(const MemoryView<const ModelT, RAM>& models) {
    if (models.size() == 0) throw Exception(RMG_ERR_INVALID_ARG, "setModel: no model");
    setModel(models[0]);
  }
  void setModel(const MemoryView<ModelT, RAM>& models) { setModel(MemoryView<const ModelT, RAM>(models)); }
  void setModel(const Memory<ModelT, RAM>& models) { setModel(models.view()); }
  void setModel(const ModelT& model) {
    const rmg_model c = model.to_c();
    rmg_sensor* s = nullptr;
    check(rmg_sensor_create(&c, nullptr, &s), "rmg_sensor_create");
    rmg_sensor_destroy(sensor_);
    sensor_ = s;
    rmg_sensor_size(sensor_, &W_, &H_);
  }

  // Poses in any Memory / MemoryView of Transform (const or not; RAM, RAM_CUDA, VRAM_CUDA,
  // UNIFIED_CUDA): a caller's slice Tbm(a, b) binds as in SphereSimulatorEmbree.hpp:140-155.
  //  * device kinds (VRAM_CUDA, UNIFIED_CUDA) -- the OptiX-style device form
  //    (SphereSimulatorOptix.hpp:141-160): fills the bundle's device buffers, asynchronous on `stream`;
  //  * host kinds (RAM, RAM_CUDA) -- the Embree-style host form (SphereSimulatorEmbree.hpp:130-155):
  //    fills the bundle's host buffers through rmg_simulate_host (pose chunks cast on `stream`
  //    while earlier chunks are copied back; the requested buffers are resized); synchronises.
  template <typename PosesT, typename BundleT, typename = std::enable_if_t<pose_buffer<PosesT>::value>>
  void simulate(const PosesT& Tbm, BundleT& ret, cudaStream_t stream = 0) const {
    using MemT = typename pose_buffer<PosesT>::Mem;
    const MemoryView<const Transform, MemT> T = view_of(Tbm);
    if constexpr (host_memory<MemT>::value) simulate_host(T.raw(), T.size(), ret, stream);
    else simulate_device(T.raw(), T.size(), ret, stream);
  }

  // Allocating forms: simulate<BundleT>(Tbm) returns a bundle of the poses' memory side, sized
  // width x height x poses.
  template <typename BundleT, typename PosesT, typename = std::enable_if_t<pose_buffer<PosesT>::value>>
  BundleT simulate(const PosesT& Tbm, cudaStream_t stream = 0) const {
    using MemT = typename pose_buffer<PosesT>::Mem;
    BundleT res;
    resize_memory_bundle<std::conditional_t<host_memory<MemT>::value, RAM, VRAM_CUDA>>(res, W_, H_,
                                                                                      (unsigned)Tbm.size());
    simulate(Tbm, res, stream);
    return res;
  }

  // One pose (SphereSimulatorEmbree.hpp:128-135): results in RAM; synchronises.
  template <typename BundleRAM>
  void simulate(const Transform& Tbm, BundleRAM& ret) const {
    simulate(MemoryView<const Transform, RAM>(&Tbm, 1), ret);
  }

  template <typename BundleRAM>
  BundleRAM simulate(const Transform& Tbm) const {
    return simulate<BundleRAM>(MemoryView<const Transform, RAM>(&Tbm, 1));
  }

  // d(loss)/d(pose) of the range residuals (rmg_range_pose_grad; no counterpart in rmagine, whose
  // simulators are not differentiable).  For every pose: loss = sum over rays with a simulated hit
  // and an observation in [range.min, range.max] of Huber_delta(r_sim - r_obs), and grad = dloss/dxi
  // (6 floats, translation first) for the right perturbation Tbm * exp(xi^).  ranges_obs holds
  // width x height ranges per pose; grad / loss are resized to 6 / 1 per pose, ranges_sim /
  // face_ids (optional) to width x height per pose.  Device kinds: asynchronous, at most 65,535
  // poses per call; host kinds (rmg_range_pose_grad_host): any number of poses, synchronises.
  template <typename PosesT, typename ObsT, typename MemT = typename pose_buffer<PosesT>::Mem>
  void rangePoseGrad(const PosesT& Tbm, const ObsT& ranges_obs, float huber_delta, Memory<float, MemT>& grad,
                     Memory<float, MemT>* loss = nullptr, Memory<float, MemT>* ranges_sim = nullptr,
                     Memory<uint32_t, MemT>* face_ids = nullptr, cudaStream_t stream = 0) const {
    ready();
    if (!map_) throw Exception(RMG_ERR_UNSUPPORTED, "rangePoseGrad: needs a single-mesh map");
    const MemoryView<const Transform, MemT> T = view_of(Tbm);
    const MemoryView<const float, MemT> obs = ranges_obs;
    const size_t n = T.size();
    if (obs.size() != n * W_ * H_)
      throw Exception(RMG_ERR_INVALID_ARG, "rangePoseGrad: ranges_obs must hold width*height ranges per pose");
    grad.resize(6 * n);
    if (loss) loss->resize(n);
    if (ranges_sim) ranges_sim->resize(n * W_ * H_);
    if (face_ids) face_ids->resize(n * W_ * H_);
    const auto* Tp = reinterpret_cast<const rmg_transform*>(T.raw());
    const auto* Tsb = reinterpret_cast<const rmg_transform*>(&Tsb_);
    float* lp = loss ? loss->raw() : nullptr;
    float* rp = ranges_sim ? ranges_sim->raw() : nullptr;
    uint32_t* fp = face_ids ? face_ids->raw() : nullptr;
    if constexpr (host_memory<MemT>::value)
      check(rmg_range_pose_grad_host(map_->handle(), sensor_, Tsb, Tp, (uint32_t)n, obs.raw(), huber_delta,
                                     grad.raw(), lp, rp, fp, stream),
            "rmg_range_pose_grad_host");
    else
      check(rmg_range_pose_grad(map_->handle(), sensor_, Tsb, Tp, (uint32_t)n, obs.raw(), huber_delta, grad.raw(),
                                lp, rp, fp, stream),
            "rmg_range_pose_grad");
  }

  uint32_t width() const { return W_; }
  uint32_t height() const { return H_; }

 private:
  template <typename MemT>
  static MemoryView<const Transform, MemT> view_of(const MemoryView<const Transform, MemT>& v) { return v; }
  template <typename MemT>
  static MemoryView<const Transform, MemT> view_of(const MemoryView<Transform, MemT>& v) { return v; }
  template <typename MemT>
  static MemoryView<const Transform, MemT> view_of(const Memory<Transform, MemT>& m) { return m.view(); }

  template <typename BundleT>
  void simulate_device(const Transform* Tbm, size_t n, BundleT& ret, cudaStream_t stream) const {
    ready();
    const rmg_outputs o = outputs_for<false>(ret);
    const auto* T = reinterpret_cast<const rmg_transform*>(Tbm);
    const auto* Tsb = reinterpret_cast<const rmg_transform*>(&Tsb_);
    if (scene_)
      check(rmg_simulate_scene(scene_->handle(), sensor_, Tsb, T, (uint32_t)n, &o, stream), "rmg_simulate_scene");
    else if (tuned_)
      check(rmg_simulate_ex(map_->handle(), sensor_, Tsb, T, (uint32_t)n, &o, &cfg_, stream), "rmg_simulate_ex");
    else
      check(rmg_simulate(map_->handle(), sensor_, Tsb, T, (uint32_t)n, &o, stream), "rmg_simulate");
  }

  template <typename BundleT>
  void simulate_host(const Transform* Tbm, size_t n, BundleT& ret, cudaStream_t stream) const {
    ready();
    resize_requested<RAM>(ret, (size_t)W_ * H_ * n);
    resize_requested<RAM_CUDA>(ret, (size_t)W_ * H_ * n);
    const rmg_outputs o = outputs_for<true>(ret);
    const auto* T = reinterpret_cast<const rmg_transform*>(Tbm);
    const auto* Tsb = reinterpret_cast<const rmg_transform*>(&Tsb_);
    if (scene_)
      check(rmg_simulate_scene_host(scene_->handle(), sensor_, Tsb, T, (uint32_t)n, &o, stream),
            "rmg_simulate_scene_host");
    else
      check(rmg_simulate_host(map_->handle(), sensor_, Tsb, T, (uint32_t)n, &o, tuned_ ? &cfg_ : nullptr, stream),
            "rmg_simulate_host");
  }

  void ready() const {
    if (!map_ && !scene_) throw Exception(RMG_ERR_INVALID_ARG, "simulate: no map set");
    if (!sensor_) throw Exception(RMG_ERR_INVALID_ARG, "simulate: no model set");
  }
  MapPtr map_;
  ScenePtr scene_;
  rmg_launch_config cfg_{};
  bool tuned_ = false;
  rmg_sensor* sensor_ = nullptr;
  Transform Tsb_ = Transform::Identity();
  uint32_t W_ = 0, H_ = 0;
};

using SphereSimulatorGB300 = SimulatorGB300<SphericalModel>;
using PinholeSimulatorGB300 = SimulatorGB300<PinholeModel>;
using O1DnSimulatorGB300 = SimulatorGB300<O1DnModel>;
using OnDnSimulatorGB300 = SimulatorGB300<OnDnModel>;
using SphereSimulatorGB300Ptr = std::shared_ptr<SphereSimulatorGB300>;
using PinholeSimulatorGB300Ptr = std::shared_ptr<PinholeSimulatorGB300>;
using O1DnSimulatorGB300Ptr = std::shared_ptr<O1DnSimulatorGB300>;
using OnDnSimulatorGB300Ptr = std::shared_ptr<OnDnSimulatorGB300>;

// ---- simulator factory (simulation/Simulator.hpp:52-78) ------------------------------------
// The computing backend tag of this library, beside rmagine's Embree / Optix / Vulkan tags.
struct GB300 {};
struct NoneType {};

template <typename ModelT, typename CompT>
struct SimulatorType {
  using Class = NoneType;
  using Ptr = NoneType;
};
template <typename ModelT>
struct SimulatorType<ModelT, GB300> {
  using Class = SimulatorGB300<ModelT>;
  using Ptr = std::shared_ptr<Class>;
};
template <typename ModelT, typename CompT>
using Simulator = typename SimulatorType<ModelT, CompT>::Class;
template <typename ModelT, typename CompT>
using SimulatorPtr = typename SimulatorType<ModelT, CompT>::Ptr;

// make_simulator<SphericalModel, GB300>() -> SphereSimulatorGB300Ptr (false for an unknown pair,
// as rmagine's factory returns)
template <typename ModelT, typename CompT>
auto make_simulator() {
  using SimT = SimulatorType<ModelT, CompT>;
  if constexpr (std::is_same<typename SimT::Class, NoneType>::value) {
    return false;
  } else {
    return typename SimT::Ptr(new typename SimT::Class);
  }
}

// The same with the map set.
template <typename ModelT, typename CompT>
auto make_simulator(MapPtr map) {
  auto sim = make_simulator<ModelT, CompT>();
  if constexpr (!std::is_same<decltype(sim), bool>::value) sim->setMap(std::move(map));
  return sim;
}

// ---- statistics / Umeyama -----------------------------------------------------------------

// statistics_p2p over n_batches batches of n_per_batch DEVICE correspondences.
inline void statistics_p2p(const Memory<Vector3, VRAM_CUDA>& dataset, const Memory<Vector3, VRAM_CUDA>& model,
                           const UmeyamaReductionConstraints& params, uint32_t n_batches,
                           Memory<CrossStatistics, VRAM_CUDA>& stats, Memory<Transform, VRAM_CUDA>* Ts = nullptr,
                           const Memory<uint8_t, VRAM_CUDA>* dataset_mask = nullptr, cudaStream_t s = 0) {
  const uint32_t n_per = n_batches ? (uint32_t)(dataset.size() / n_batches) : 0;
  stats.resize(n_batches);
  if (Ts) Ts->resize(n_batches);
  const rmg_umeyama_constraints c{params.max_dist, params.dataset_id, params.model_id};
  check(rmg_statistics_p2p(nullptr, 0, reinterpret_cast<const rmg_vec3*>(dataset.raw()),
                           dataset_mask ? dataset_mask->raw() : nullptr, nullptr,
                           reinterpret_cast<const rmg_vec3*>(model.raw()), nullptr, nullptr, &c, n_batches, n_per,
                           reinterpret_cast<rmg_cross_stats*>(stats.raw()),
                           Ts ? reinterpret_cast<rmg_transform*>(Ts->raw()) : nullptr, s),
        "rmg_statistics_p2p");
}

inline void umeyama_transform(const Memory<CrossStatistics, VRAM_CUDA>& stats, Memory<Transform, VRAM_CUDA>& Ts,
                              cudaStream_t s = 0) {
  Ts.resize(stats.size());
  check(rmg_umeyama_transform(reinterpret_cast<const rmg_cross_stats*>(stats.raw()), (uint32_t)stats.size(),
                              reinterpret_cast<rmg_transform*>(Ts.raw()), s),
        "rmg_umeyama_transform");
}

// statistics_p2l over n_batches batches of n_per_batch DEVICE correspondences (model points with normals).
inline void statistics_p2l(const Memory<Vector3, VRAM_CUDA>& dataset, const Memory<Vector3, VRAM_CUDA>& model,
                           const Memory<Vector3, VRAM_CUDA>& model_normals,
                           const UmeyamaReductionConstraints& params, uint32_t n_batches,
                           Memory<CrossStatistics, VRAM_CUDA>& stats, Memory<Transform, VRAM_CUDA>* Ts = nullptr,
                           const Memory<uint8_t, VRAM_CUDA>* dataset_mask = nullptr,
                           const Memory<uint8_t, VRAM_CUDA>* model_mask = nullptr, cudaStream_t s = 0) {
  const uint32_t n_per = n_batches ? (uint32_t)(dataset.size() / n_batches) : 0;
  stats.resize(n_batches);
  if (Ts) Ts->resize(n_batches);
  const rmg_umeyama_constraints c{params.max_dist, params.dataset_id, params.model_id};
  check(rmg_statistics_p2l(nullptr, 0, reinterpret_cast<const rmg_vec3*>(dataset.raw()),
                           dataset_mask ? dataset_mask->raw() : nullptr, nullptr,
                           reinterpret_cast<const rmg_vec3*>(model.raw()),
                           reinterpret_cast<const rmg_vec3*>(model_normals.raw()),
                           model_mask ? model_mask->raw() : nullptr, nullptr, &c, n_batches, n_per,
                           reinterpret_cast<rmg_cross_stats*>(stats.raw()),
                           Ts ? reinterpret_cast<rmg_transform*>(Ts->raw()) : nullptr, s),
        "rmg_statistics_p2l");
}

// Backward of statistics_p2p + umeyama_transform (rmg_umeyama_backward; no counterpart in
// rmagine): given the forward's stats and upstream gradients dL/dR (9 floats per batch,
// row-major) and dL/dt (3 per batch) -- either may be null, meaning zero -- writes dL/d(dataset
// point) and dL/d(model point) for every correspondence; filtered-out correspondences get 0.
// Same DEVICE inputs and filter as statistics_p2p.
inline void umeyama_backward(const Memory<Vector3, VRAM_CUDA>& dataset, const Memory<Vector3, VRAM_CUDA>& model,
                             const UmeyamaReductionConstraints& params, uint32_t n_batches,
                             const Memory<CrossStatistics, VRAM_CUDA>& stats, const Memory<float, VRAM_CUDA>* grad_R,
                             const Memory<float, VRAM_CUDA>* grad_t, Memory<Vector3, VRAM_CUDA>* grad_dataset,
                             Memory<Vector3, VRAM_CUDA>* grad_model,
                             const Memory<uint8_t, VRAM_CUDA>* dataset_mask = nullptr, cudaStream_t s = 0) {
  const uint32_t n_per = n_batches ? (uint32_t)(dataset.size() / n_batches) : 0;
  if (grad_dataset) grad_dataset->resize(dataset.size());
  if (grad_model) grad_model->resize(model.size());
  const rmg_umeyama_constraints c{params.max_dist, params.dataset_id, params.model_id};
  check(rmg_umeyama_backward(nullptr, 0, reinterpret_cast<const rmg_vec3*>(dataset.raw()),
                             dataset_mask ? dataset_mask->raw() : nullptr, nullptr,
                             reinterpret_cast<const rmg_vec3*>(model.raw()), nullptr, nullptr, &c, n_batches, n_per,
                             reinterpret_cast<const rmg_cross_stats*>(stats.raw()), grad_R ? grad_R->raw() : nullptr,
                             grad_t ? grad_t->raw() : nullptr,
                             grad_dataset ? reinterpret_cast<rmg_vec3*>(grad_dataset->raw()) : nullptr,
                             grad_model ? reinterpret_cast<rmg_vec3*>(grad_model->raw()) : nullptr, s),
        "rmg_umeyama_backward");
}

// Batched 3x3 SVD A = U W V^T (svd(As, Us, Ws, Vs), memory_math.cuh:561-578) of column-major
// DEVICE matrices (9 floats each, rmagine's Matrix3x3 layout): W >= 0 on the diagonal, sorted
// descending; with rotations = true, U and V are rotations and the last value carries det A's sign.
inline void svd(const Memory<float, VRAM_CUDA>& As, Memory<float, VRAM_CUDA>& Us, Memory<float, VRAM_CUDA>& Ws,
                Memory<float, VRAM_CUDA>& Vs, bool rotations = false, cudaStream_t s = 0) {
  const size_t n = As.size() / 9;
  Us.resize(9 * n);
  Ws.resize(9 * n);
  Vs.resize(9 * n);
  check(rmg_svd3(As.raw(), Us.raw(), Ws.raw(), nullptr, Vs.raw(), (uint32_t)n, rotations ? 1 : 0, s), "rmg_svd3");
}

// out[i] = a[i] * b[i] on the device (Transform::mult); a one-element operand is repeated.
inline void compose(const Memory<Transform, VRAM_CUDA>& a, const Memory<Transform, VRAM_CUDA>& b,
                    Memory<Transform, VRAM_CUDA>& out, cudaStream_t s = 0) {
  const size_t n = a.size() > b.size() ? a.size() : b.size();
  if (out.raw() != a.raw()) out.resize(n);
  check(rmg_transforms_compose(reinterpret_cast<const rmg_transform*>(a.raw()), a.size() > 1 ? 1u : 0u,
                               reinterpret_cast<const rmg_transform*>(b.raw()), b.size() > 1 ? 1u : 0u,
                               reinterpret_cast<rmg_transform*>(out.raw()), (uint32_t)n, s),
        "rmg_transforms_compose");
}

// ---- range noise --------------------------------------------------------------------------
struct NoiseOptions {  // Noise::Options
  uint64_t seed = 42;
  float max_range = 10000.0f;
};

class NoiseGB300 {
 public:
  // adds noise to DEVICE ranges in place; every call draws fresh numbers
  void apply(Memory<float, VRAM_CUDA>& ranges, cudaStream_t s = 0) {
    rmg_noise p = p_;
    p.call = call_++;
    check(rmg_noise_apply(&p, ranges.raw(), ranges.size(), s), "rmg_noise_apply");
  }

  // throws when a noise kernel on the current device recorded a lost bulk copy; synchronises
  static void check_device(bool clear = true) {
    uint32_t word = 0;
    check(rmg_noise_status(&word, clear ? 1 : 0), "rmg_noise_status");
    check((int)word, "noise kernel");
  }

 protected:
  NoiseGB300(uint32_t kind, const NoiseOptions& o) {
    p_.kind = kind;
    p_.seed = o.seed;
    p_.max_range = o.max_range;
  }
  rmg_noise p_{};
  uint64_t call_ = 0;
};

class GaussianNoiseGB300 : public NoiseGB300 {
 public:
  GaussianNoiseGB300(float mean, float stddev, const NoiseOptions& o = {}) : NoiseGB300(RMG_NOISE_GAUSSIAN, o) {
    p_.mean = mean;
    p_.stddev = stddev;
  }
};

class RelGaussianNoiseGB300 : public NoiseGB300 {
 public:
  RelGaussianNoiseGB300(float mean, float stddev, float range_exp, const NoiseOptions& o = {})
      : NoiseGB300(RMG_NOISE_REL_GAUSSIAN, o) {
    p_.mean = mean;
    p_.stddev = stddev;
    p_.range_exp = range_exp;
  }
};

class UniformDustNoiseGB300 : public NoiseGB300 {
 public:
  UniformDustNoiseGB300(float hit_probability, float return_probability, const NoiseOptions& o = {})
      : NoiseGB300(RMG_NOISE_UNIFORM_DUST, o) {
    p_.hit_probability = hit_probability;
    p_.return_probability = return_probability;
  }
};

}  // namespace rmagine_gb300
