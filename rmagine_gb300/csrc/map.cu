// Map construction: triangle mesh -> linear BVH on the GPU.
//
// Replaces the BVH build that rmagine delegates to Embree
// (src/rmagine_embree/src/map/embree/EmbreeScene.cpp:187-191, quality MEDIUM)
// and OptiX (src/rmagine_optix/src/map/optix/OptixScene.cpp:242-481).
//
// Build (Karras, "Maximizing Parallelism in the Construction of BVHs,
// Octrees, and k-d Trees", HPG 2012):
//   1. centroid bounds of all triangles (two-level reduction)
//   2. 63-bit Morton code of each centroid (21 bits per axis) in the centroids'
//      bounding cube (one scale for all axes)
//   3. stable radix sort of (code, face index): ties ordered by index
//   4. radix tree over the sorted codes, one thread per internal node; equal
//      codes are disambiguated by the index (the paper's augmentation)
//   5. triangles packed in leaf order as 48-byte records
//   6. bottom-up refit of the child boxes with per-node arrival counters
// Leaves hold exactly one triangle.  The result is a pure function of the
// input arrays (no atomics influence the topology), so the same mesh always
// yields the same tree.
#include <cub/cub.cuh>

#include <algorithm>
#include <cstring>
#include <mutex>
#include <new>

#include "internal.h"

namespace rmg {
namespace {

constexpr int kBlock = 256;

__device__ __forceinline__ float3 load_v(const float* v, uint32_t i) {
  return make_float3(v[3 * i + 0], v[3 * i + 1], v[3 * i + 2]);
}

// Centroid in a fixed operation order: ((v0 + v1) + v2) * 0.333333343f.
__device__ __forceinline__ float3 centroid(const float* v, const uint32_t* f, uint32_t i) {
  const float3 a = load_v(v, f[3 * i + 0]);
  const float3 b = load_v(v, f[3 * i + 1]);
  const float3 c = load_v(v, f[3 * i + 2]);
  const float third = 0.333333343f;
  return make_float3(__fmul_rn(__fadd_rn(__fadd_rn(a.x, b.x), c.x), third),
                     __fmul_rn(__fadd_rn(__fadd_rn(a.y, b.y), c.y), third),
                     __fmul_rn(__fadd_rn(__fadd_rn(a.z, b.z), c.z), third));
}

__global__ void k_centroid_bounds(const float* v, const uint32_t* f, uint32_t n, float* partial) {
  float lo[3] = {INFINITY, INFINITY, INFINITY};
  float hi[3] = {-INFINITY, -INFINITY, -INFINITY};
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const float3 c = centroid(v, f, i);
    lo[0] = fminf(lo[0], c.x); lo[1] = fminf(lo[1], c.y); lo[2] = fminf(lo[2], c.z);
    hi[0] = fmaxf(hi[0], c.x); hi[1] = fmaxf(hi[1], c.y); hi[2] = fmaxf(hi[2], c.z);
  }
  __shared__ float s[6][kBlock / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int k = 0; k < 3; ++k) {
    for (int o = 16; o > 0; o >>= 1) {
      lo[k] = fminf(lo[k], __shfl_xor_sync(0xffffffffu, lo[k], o));
      hi[k] = fmaxf(hi[k], __shfl_xor_sync(0xffffffffu, hi[k], o));
    }
  }
  if (lane == 0) {
    for (int k = 0; k < 3; ++k) { s[k][warp] = lo[k]; s[3 + k][warp] = hi[k]; }
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 1; w < kBlock / 32; ++w) {
      for (int k = 0; k < 3; ++k) {
        s[k][0] = fminf(s[k][0], s[k][w]);
        s[3 + k][0] = fmaxf(s[3 + k][0], s[3 + k][w]);
      }
    }
    for (int k = 0; k < 6; ++k) partial[6 * blockIdx.x + k] = s[k][0];
  }
}

__global__ void k_bounds_final(const float* partial, int nblocks, float* out) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  float r[6] = {INFINITY, INFINITY, INFINITY, -INFINITY, -INFINITY, -INFINITY};
  for (int b = 0; b < nblocks; ++b) {
    for (int k = 0; k < 3; ++k) {
      r[k] = fminf(r[k], partial[6 * b + k]);
      r[3 + k] = fmaxf(r[3 + k], partial[6 * b + 3 + k]);
    }
  }
  for (int k = 0; k < 6; ++k) out[k] = r[k];
}

// Spreads the low 21 bits of x so that bit i lands on bit 3i.
__device__ __forceinline__ uint64_t spread3(uint64_t x) {
  x &= 0x1fffffull;
  x = (x | (x << 32)) & 0x001f00000000ffffull;
  x = (x | (x << 16)) & 0x001f0000ff0000ffull;
  x = (x | (x << 8)) & 0x100f00f00f00f00full;
  x = (x | (x << 4)) & 0x10c30c30c30c30c3ull;
  x = (x | (x << 2)) & 0x1249249249249249ull;
  return x;
}

__device__ __forceinline__ uint32_t quantize(float c, float lo, float scale) {
  float q = __fmul_rn(__fsub_rn(c, lo), scale);
  q = fminf(fmaxf(q, 0.0f), 2097151.0f);
  return (uint32_t)q;
}

// code = sum_i x_i << (3i+2) | y_i << (3i+1) | z_i << 3i
__global__ void k_morton(const float* v, const uint32_t* f, uint32_t n, const float* bounds,
                         uint64_t* keys, uint32_t* vals) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float3 c = centroid(v, f, i);
  // One scale for all axes (the bounding cube of the centroids): a flat scene
  // such as a terrain keeps its aspect ratio in code space, so the radix tree
  // does not split the thin axis early (about 24% fewer node visits per ray on
  // a 500 x 500 x 40 m terrain than per-axis normalisation).
  const float ext = fmaxf(fmaxf(__fsub_rn(bounds[3], bounds[0]), __fsub_rn(bounds[4], bounds[1])),
                          __fsub_rn(bounds[5], bounds[2]));
  const float scale = ext > 0.0f ? __fdiv_rn(2097152.0f, ext) : 0.0f;
  const uint64_t qx = quantize(c.x, bounds[0], scale);
  const uint64_t qy = quantize(c.y, bounds[1], scale);
  const uint64_t qz = quantize(c.z, bounds[2], scale);
  keys[i] = (spread3(qx) << 2) | (spread3(qy) << 1) | spread3(qz);
  vals[i] = i;
}

__device__ __forceinline__ int delta(const uint64_t* k, int n, int i, int j) {
  if (j < 0 || j >= n) return -1;
  const uint64_t a = k[i], b = k[j];
  if (a == b) return 64 + __clz(i ^ j);
  return __clzll((long long)(a ^ b));
}

__global__ void k_karras(const uint64_t* keys, int n, Node* nodes, int* leaf_parent) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n - 1) return;
  const int d = (delta(keys, n, i, i + 1) - delta(keys, n, i, i - 1)) >= 0 ? 1 : -1;
  const int dmin = delta(keys, n, i, i - d);
  int lmax = 2;
  while (delta(keys, n, i, i + lmax * d) > dmin) lmax <<= 1;
  int l = 0;
  for (int t = lmax >> 1; t >= 1; t >>= 1)
    if (delta(keys, n, i, i + (l + t) * d) > dmin) l += t;
  const int j = i + l * d;
  const int dnode = delta(keys, n, i, j);
  int s = 0;
  for (int div = 2;; div <<= 1) {
    const int t = (l + div - 1) / div;
    if (delta(keys, n, i, i + (s + t) * d) > dnode) s += t;
    if (t <= 1) break;
  }
  const int gamma = i + s * d + min(d, 0);
  const int first = min(i, j), last = max(i, j);
  int left, right;
  if (first == gamma) { left = ~gamma; leaf_parent[gamma] = i; }
  else { left = gamma; nodes[gamma].d.z = i; }
  if (last == gamma + 1) { right = ~(gamma + 1); leaf_parent[gamma + 1] = i; }
  else { right = gamma + 1; nodes[gamma + 1].d.z = i; }
  nodes[i].d.x = left;
  nodes[i].d.y = right;
  nodes[i].d.w = dnode;
  if (i == 0) nodes[0].d.z = -1;
}

__global__ void k_pack(const float* v, const uint32_t* f, const uint32_t* order, uint32_t n,
                       Tri* tris, uint32_t* leaf_order) {
  const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const uint32_t fid = order[k];
  const float3 a = load_v(v, f[3 * fid + 0]);
  const float3 b = load_v(v, f[3 * fid + 1]);
  const float3 c = load_v(v, f[3 * fid + 2]);
  Tri t;
  t.v0 = make_float4(a.x, a.y, a.z, __int_as_float((int)fid));
  t.v1 = make_float4(b.x, b.y, b.z, 0.0f);
  t.v2 = make_float4(c.x, c.y, c.z, 0.0f);
  tris[k] = t;
  if (leaf_order) leaf_order[k] = fid;
}

struct Box { float lo[3], hi[3]; };

__device__ __forceinline__ Box tri_box(const Tri* tris, int k) {
  const float4 a = __ldcg(&tris[k].v0), b = __ldcg(&tris[k].v1), c = __ldcg(&tris[k].v2);
  Box r;
  r.lo[0] = fminf(fminf(a.x, b.x), c.x); r.hi[0] = fmaxf(fmaxf(a.x, b.x), c.x);
  r.lo[1] = fminf(fminf(a.y, b.y), c.y); r.hi[1] = fmaxf(fmaxf(a.y, b.y), c.y);
  r.lo[2] = fminf(fminf(a.z, b.z), c.z); r.hi[2] = fmaxf(fmaxf(a.z, b.z), c.z);
  return r;
}

__device__ __forceinline__ Box node_box(const Node* nodes, int i) {
  const float4 a = __ldcg(&nodes[i].a), b = __ldcg(&nodes[i].b), c = __ldcg(&nodes[i].c);
  Box r;
  r.lo[0] = fminf(a.x, b.x); r.hi[0] = fmaxf(a.y, b.y);
  r.lo[1] = fminf(a.z, b.z); r.hi[1] = fmaxf(a.w, b.w);
  r.lo[2] = fminf(c.x, c.z); r.hi[2] = fmaxf(c.y, c.w);
  return r;
}

__device__ __forceinline__ Box child_box(const Node* nodes, const Tri* tris, int c) {
  return c < 0 ? tri_box(tris, ~c) : node_box(nodes, c);
}

// One thread per leaf walks towards the root; the second thread to reach a
// node writes that node's two child boxes and continues.
__global__ void k_refit(Node* nodes, const Tri* tris, const int* leaf_parent, unsigned int* flags,
                        uint32_t n) {
  const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  int node = leaf_parent[k];
  while (node >= 0) {
    __threadfence();
    const unsigned int old = atomicAdd(&flags[node], 1u);
    if (old == 0) return;
    __threadfence();
    const int4 link = __ldcg(&nodes[node].d);
    const Box L = child_box(nodes, tris, link.x);
    const Box R = child_box(nodes, tris, link.y);
    __stcg(&nodes[node].a, make_float4(L.lo[0], L.hi[0], L.lo[1], L.hi[1]));
    __stcg(&nodes[node].b, make_float4(R.lo[0], R.hi[0], R.lo[1], R.hi[1]));
    __stcg(&nodes[node].c, make_float4(L.lo[2], L.hi[2], R.lo[2], R.hi[2]));
    node = link.z;
  }
}

__global__ void k_depth(const Node* nodes, const int* leaf_parent, uint32_t n, unsigned int* out) {
  const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  unsigned int d = 1;
  int node = leaf_parent[k];
  int guard = 0;
  while (node >= 0 && nodes[node].d.z >= 0 && guard < (1 << 20)) {
    node = nodes[node].d.z;
    ++d;
    ++guard;
  }
  atomicMax(out, d);
}

inline unsigned grid_for(size_t n, int block = kBlock) {
  return (unsigned)((n + block - 1) / block);
}

// Single-triangle map: one node whose right child is a phantom box far
// outside any ray's reach (t ~ 1e30 > range.max), so traversal never takes it.
void single_node(const float* v, const uint32_t* f, Node* out) {
  float lo[3], hi[3];
  for (int k = 0; k < 3; ++k) {
    const float a = v[3 * f[0] + k], b = v[3 * f[1] + k], c = v[3 * f[2] + k];
    lo[k] = std::min(std::min(a, b), c);
    hi[k] = std::max(std::max(a, b), c);
  }
  const float far = 1e30f;
  out->a = make_float4(lo[0], hi[0], lo[1], hi[1]);
  out->b = make_float4(far, far, far, far);
  out->c = make_float4(lo[2], hi[2], far, far);
  out->d = make_int4(-1, -1, -1, 0);
}

void free_map(rmg_map* m) {
  if (!m) return;
  cudaFree(m->d_vertices);
  cudaFree(m->d_faces);
  cudaFree(m->d_nodes);
  cudaFree(m->d_tris);
  cudaFree(m->d_leaf_order);
  cudaFree(m->d_leaf_parent);
  cudaFree(m->d_flags);
  cudaFree(m->d_status);
  wide_free(m);
  delete m;
}

// Packs the triangles and refits all boxes of an existing topology.
int repack_and_refit(rmg_map* m, cudaStream_t st, const uint32_t* d_order) {
  const uint32_t n = m->n_faces;
  if (n == 0) return RMG_OK;
  k_pack<<<grid_for(n), kBlock, 0, st>>>(m->d_vertices, m->d_faces, d_order, n, m->d_tris,
                                        nullptr);
  RMG_CUDA_TRY(cudaGetLastError());
  if (n == 1) {
    // recompute the single node's box on the host from the new vertices
    float v[9];
    uint32_t f[3];
    RMG_CUDA_TRY(cudaMemcpyAsync(f, m->d_faces, sizeof(f), cudaMemcpyDeviceToHost, st));
    RMG_CUDA_TRY(cudaStreamSynchronize(st));
    const uint32_t local[3] = {0, 1, 2};
    for (int k = 0; k < 3; ++k)
      RMG_CUDA_TRY(cudaMemcpyAsync(v + 3 * k, m->d_vertices + 3 * f[k], 3 * sizeof(float),
                                   cudaMemcpyDeviceToHost, st));
    RMG_CUDA_TRY(cudaStreamSynchronize(st));
    Node node;
    single_node(v, local, &node);
    RMG_CUDA_TRY(cudaMemcpyAsync(m->d_nodes, &node, sizeof(Node), cudaMemcpyHostToDevice, st));
    return RMG_OK;
  }
  RMG_CUDA_TRY(cudaMemsetAsync(m->d_flags, 0, m->n_nodes * sizeof(unsigned int), st));
  k_refit<<<grid_for(n), kBlock, 0, st>>>(m->d_nodes, m->d_tris, m->d_leaf_parent, m->d_flags, n);
  RMG_CUDA_TRY(cudaGetLastError());
  return RMG_OK;
}

void update_info(rmg_map* m, cudaStream_t st) {
  for (int k = 0; k < 3; ++k) { m->lo[k] = INFINITY; m->hi[k] = -INFINITY; }
  if (m->n_faces == 0) return;
  Node root;
  if (cudaMemcpyAsync(&root, m->d_nodes, sizeof(Node), cudaMemcpyDeviceToHost, st) != cudaSuccess)
    return;
  if (cudaStreamSynchronize(st) != cudaSuccess) return;
  if (m->n_faces == 1) {
    m->lo[0] = root.a.x; m->hi[0] = root.a.y; m->lo[1] = root.a.z; m->hi[1] = root.a.w;
    m->lo[2] = root.c.x; m->hi[2] = root.c.y;
    return;
  }
  m->lo[0] = std::min(root.a.x, root.b.x); m->hi[0] = std::max(root.a.y, root.b.y);
  m->lo[1] = std::min(root.a.z, root.b.z); m->hi[1] = std::max(root.a.w, root.b.w);
  m->lo[2] = std::min(root.c.x, root.c.z); m->hi[2] = std::max(root.c.y, root.c.w);
}

}  // namespace

DeviceMap device_view(const rmg_map* m) {
  DeviceMap d;
  d.nodes4 = m->d_nodes4;
  d.nodes8 = m->d_nodes8;
  d.tris8 = m->d_tris8;
  d.nodes = m->d_nodes;
  d.tris = m->d_tris;
  d.n_nodes = (int)m->n_nodes;
  d.n_tris = (int)m->n_faces;
  d.root = m->n_faces > 0 ? 0 : -1;
  d.status = m->d_status;
  return d;
}

}  // namespace rmg

using namespace rmg;

extern "C" int rmg_map_build_wide8(rmg_map* m, void* stream) {
  return guarded("rmg_map_build_wide8", [&]() -> int {
    if (!m) return fail(RMG_ERR_INVALID_ARG, "rmg_map_build_wide8: map is NULL");
    if (m->n_faces == 0 || m->d_nodes8) return RMG_OK;
    return wide8_build(m, as_stream(stream));
  });
}

extern "C" int rmg_map_build(const rmg_vec3* vertices, uint32_t n_vertices, const rmg_face* faces,
                             uint32_t n_faces, void* stream, rmg_map** out) {
  return guarded("rmg_map_build", [&]() -> int {
    return rmg_map_build_ex(vertices, n_vertices, faces, n_faces, RMG_BUILD_SAH, stream, out);
  });
}

extern "C" int rmg_map_build_ex(const rmg_vec3* vertices, uint32_t n_vertices, const rmg_face* faces,
                                uint32_t n_faces, uint32_t builder, void* stream, rmg_map** out) {
  return guarded("rmg_map_build_ex", [&]() -> int {
    if (!out) return fail(RMG_ERR_INVALID_ARG, "rmg_map_build: out is NULL");
    *out = nullptr;
    if (builder != RMG_BUILD_SAH && builder != RMG_BUILD_LBVH)
      return fail(RMG_ERR_UNSUPPORTED, "rmg_map_build_ex: builder must be RMG_BUILD_SAH or RMG_BUILD_LBVH");
    *out = nullptr;
    if (n_faces > 0 && (!vertices || !faces))
      return fail(RMG_ERR_INVALID_ARG, "rmg_map_build: vertices/faces are NULL");
    if (n_faces > (1u << 30)) return fail(RMG_ERR_INVALID_ARG, "rmg_map_build: too many faces");
    for (uint32_t i = 0; i < n_faces; ++i) {
      if (faces[i].v0 >= n_vertices || faces[i].v1 >= n_vertices || faces[i].v2 >= n_vertices)
        return fail(RMG_ERR_INVALID_ARG, "rmg_map_build: face index out of range");
    }
    cudaStream_t st = as_stream(stream);
    rmg_map* m = new (std::nothrow) rmg_map;
    if (!m) return fail(RMG_ERR_OOM, "rmg_map_build: host allocation");
    std::memset(m, 0, sizeof(*m));
    cudaGetDevice(&m->device);
    m->n_vertices = n_vertices;
    m->n_faces = n_faces;
    m->n_nodes = n_faces >= 2 ? n_faces - 1 : (n_faces == 1 ? 1 : 0);
  
    int s = RMG_OK;
    auto check = [&](int r) { if (s == RMG_OK) s = r; return s == RMG_OK; };
  
    check(dev_alloc(&m->d_status, 1, "status"));
    if (s == RMG_OK) s = cuda_status(cudaMemsetAsync(m->d_status, 0, sizeof(unsigned int), st), "memset");
    if (s == RMG_OK && n_faces == 0) {
      s = cuda_status(cudaStreamSynchronize(st), "sync");
      if (s != RMG_OK) { free_map(m); return s; }
      update_info(m, st);
      *out = m;
      return RMG_OK;
    }
    check(dev_alloc(&m->d_vertices, 3 * (size_t)n_vertices, "vertices"));
    check(dev_alloc(&m->d_faces, 3 * (size_t)n_faces, "faces"));
    check(dev_alloc(&m->d_nodes, m->n_nodes, "nodes"));
    check(dev_alloc(&m->d_tris, n_faces, "tris"));
    check(dev_alloc(&m->d_leaf_order, n_faces, "leaf order"));
    check(dev_alloc(&m->d_leaf_parent, n_faces, "leaf parent"));
    check(dev_alloc(&m->d_flags, m->n_nodes, "flags"));
    if (s != RMG_OK) { free_map(m); return s; }
    s = cuda_status(cudaMemcpyAsync(m->d_vertices, vertices, 12 * (size_t)n_vertices,
                                    cudaMemcpyHostToDevice, st), "copy vertices");
    if (s == RMG_OK)
      s = cuda_status(cudaMemcpyAsync(m->d_faces, faces, 12 * (size_t)n_faces,
                                      cudaMemcpyHostToDevice, st), "copy faces");
    if (s != RMG_OK) { free_map(m); return s; }
  
    if (n_faces == 1) {
      Node node;
      const uint32_t local[3] = {0, 1, 2};
      float v[9];
      for (int k = 0; k < 3; ++k) {
        const uint32_t vi = k == 0 ? faces[0].v0 : (k == 1 ? faces[0].v1 : faces[0].v2);
        v[3 * k + 0] = vertices[vi].x; v[3 * k + 1] = vertices[vi].y; v[3 * k + 2] = vertices[vi].z;
      }
      single_node(v, local, &node);
      const uint32_t zero = 0;
      const int minus1 = -1;
      s = cuda_status(cudaMemcpyAsync(m->d_nodes, &node, sizeof(Node), cudaMemcpyHostToDevice, st), "node");
      if (s == RMG_OK) s = cuda_status(cudaMemcpyAsync(m->d_leaf_order, &zero, 4, cudaMemcpyHostToDevice, st), "order");
      if (s == RMG_OK) s = cuda_status(cudaMemcpyAsync(m->d_leaf_parent, &minus1, 4, cudaMemcpyHostToDevice, st), "parent");
      if (s == RMG_OK) {
        k_pack<<<1, 32, 0, st>>>(m->d_vertices, m->d_faces, m->d_leaf_order, 1, m->d_tris, nullptr);
        s = cuda_status(cudaGetLastError(), "k_pack");
      }
      if (s == RMG_OK) s = cuda_status(cudaStreamSynchronize(st), "sync");
      if (s != RMG_OK) { free_map(m); return s; }
      m->depth = 1;
      s = wide_build(m, st);
      if (s != RMG_OK) { free_map(m); return s; }
      update_info(m, st);
      *out = m;
      return RMG_OK;
    }
  
    const uint32_t n = n_faces;
    if (builder == RMG_BUILD_SAH) {
      s = sah_build_topology(m, st, m->d_leaf_order);
      if (s == RMG_OK) s = repack_and_refit(m, st, m->d_leaf_order);
      unsigned int* d_depth = nullptr;
      if (s == RMG_OK) s = dev_alloc(&d_depth, 1, "depth");
      if (s == RMG_OK) s = cuda_status(cudaMemsetAsync(d_depth, 0, 4, st), "memset");
      if (s == RMG_OK) {
        k_depth<<<grid_for(n), kBlock, 0, st>>>(m->d_nodes, m->d_leaf_parent, n, d_depth);
        s = cuda_status(cudaGetLastError(), "depth");
      }
      unsigned int depth = 0;
      if (s == RMG_OK) s = cuda_status(cudaMemcpyAsync(&depth, d_depth, 4, cudaMemcpyDeviceToHost, st), "depth copy");
      if (s == RMG_OK) s = cuda_status(cudaStreamSynchronize(st), "sync");
      cudaFree(d_depth);
      if (s != RMG_OK) { free_map(m); return s; }
      m->depth = depth;
      s = wide_build(m, st);
      if (s != RMG_OK) { free_map(m); return s; }
      update_info(m, st);
      *out = m;
      return RMG_OK;
    }
  
    // ---- LBVH scratch -----------------------------------------------------
    const int nb = std::min<int>((int)grid_for(n), 4 * device_sm_count());
    float* d_partial = nullptr;
    float* d_bounds = nullptr;
    uint64_t *d_keys = nullptr, *d_keys2 = nullptr;
    uint32_t *d_vals = nullptr, *d_vals2 = nullptr;
    unsigned int* d_depth = nullptr;
    void* d_temp = nullptr;
    size_t temp_bytes = 0;
    check(dev_alloc(&d_partial, 6 * (size_t)nb, "partial bounds"));
    check(dev_alloc(&d_bounds, 6, "bounds"));
    check(dev_alloc(&d_keys, n, "keys"));
    check(dev_alloc(&d_keys2, n, "keys2"));
    check(dev_alloc(&d_vals, n, "vals"));
    check(dev_alloc(&d_vals2, n, "vals2"));
    check(dev_alloc(&d_depth, 1, "depth"));
    if (s == RMG_OK) {
      s = cuda_status(cub::DeviceRadixSort::SortPairs(nullptr, temp_bytes, d_keys, d_keys2, d_vals,
                                                       d_vals2, (int)n, 0, 63, st), "sort size");
    }
    if (s == RMG_OK) {
      char* tmp = nullptr;
      s = dev_alloc(&tmp, temp_bytes, "sort temp");
      d_temp = tmp;
    }
    if (s == RMG_OK) {
      k_centroid_bounds<<<nb, kBlock, 0, st>>>(m->d_vertices, m->d_faces, n, d_partial);
      k_bounds_final<<<1, 32, 0, st>>>(d_partial, nb, d_bounds);
      k_morton<<<grid_for(n), kBlock, 0, st>>>(m->d_vertices, m->d_faces, n, d_bounds, d_keys, d_vals);
      s = cuda_status(cudaGetLastError(), "morton");
    }
    if (s == RMG_OK)
      s = cuda_status(cub::DeviceRadixSort::SortPairs(d_temp, temp_bytes, d_keys, d_keys2, d_vals,
                                                       d_vals2, (int)n, 0, 63, st), "sort");
    if (s == RMG_OK) s = cuda_status(cudaMemsetAsync(m->d_nodes, 0, sizeof(Node) * m->n_nodes, st), "memset");
    if (s == RMG_OK) {
      k_karras<<<grid_for(n - 1), kBlock, 0, st>>>(d_keys2, (int)n, m->d_nodes, m->d_leaf_parent);
      k_pack<<<grid_for(n), kBlock, 0, st>>>(m->d_vertices, m->d_faces, d_vals2, n, m->d_tris,
                                            m->d_leaf_order);
      s = cuda_status(cudaGetLastError(), "karras");
    }
    if (s == RMG_OK) s = repack_and_refit(m, st, m->d_leaf_order);
    if (s == RMG_OK) s = cuda_status(cudaMemsetAsync(d_depth, 0, 4, st), "memset");
    if (s == RMG_OK) {
      k_depth<<<grid_for(n), kBlock, 0, st>>>(m->d_nodes, m->d_leaf_parent, n, d_depth);
      s = cuda_status(cudaGetLastError(), "depth");
    }
    unsigned int depth = 0;
    if (s == RMG_OK) s = cuda_status(cudaMemcpyAsync(&depth, d_depth, 4, cudaMemcpyDeviceToHost, st), "depth copy");
    if (s == RMG_OK) s = cuda_status(cudaStreamSynchronize(st), "sync");
    cudaFree(d_partial); cudaFree(d_bounds); cudaFree(d_keys); cudaFree(d_keys2);
    cudaFree(d_vals); cudaFree(d_vals2); cudaFree(d_depth); cudaFree(d_temp);
    if (s != RMG_OK) { free_map(m); return s; }
    m->depth = depth;
    s = wide_build(m, st);
    if (s != RMG_OK) { free_map(m); return s; }
    update_info(m, st);
    *out = m;
    return RMG_OK;
  });
}

extern "C" int rmg_map_refit(rmg_map* m, const rmg_vec3* vertices, uint32_t n_vertices, void* stream) {
  return guarded("rmg_map_refit", [&]() -> int {
    if (!m) return fail(RMG_ERR_INVALID_ARG, "rmg_map_refit: map is NULL");
    if (n_vertices != m->n_vertices)
      return fail(RMG_ERR_INVALID_ARG, "rmg_map_refit: vertex count differs from the build");
    if (m->n_faces == 0) return RMG_OK;
    if (!vertices) return fail(RMG_ERR_INVALID_ARG, "rmg_map_refit: vertices is NULL");
    cudaStream_t st = as_stream(stream);
    RMG_CUDA_TRY(cudaMemcpyAsync(m->d_vertices, vertices, 12 * (size_t)n_vertices,
                                 cudaMemcpyHostToDevice, st));
    int s = repack_and_refit(m, st, m->d_leaf_order);
    if (s == RMG_OK) s = wide_refit(m, st);
    if (s != RMG_OK) return s;
    RMG_CUDA_TRY(cudaStreamSynchronize(st));
    update_info(m, st);
    return RMG_OK;
  });
}

extern "C" int rmg_map_destroy(rmg_map* m) {
  return guarded("rmg_map_destroy", [&]() -> int {
    if (!m) return RMG_OK;
    free_map(m);
    return RMG_OK;
  });
}

extern "C" int rmg_map_info_get(const rmg_map* m, rmg_map_info* out) {
  return guarded("rmg_map_info_get", [&]() -> int {
    if (!m || !out) return fail(RMG_ERR_INVALID_ARG, "rmg_map_info_get: NULL argument");
    out->n_vertices = m->n_vertices;
    out->n_faces = m->n_faces;
    out->n_nodes = m->n_nodes;
    out->depth = m->depth;
    out->device_bytes = (uint64_t)m->n_nodes * sizeof(Node) + (uint64_t)m->n_faces * sizeof(Tri) +
                        12ull * m->n_vertices + 12ull * m->n_faces +
                        (uint64_t)m->n_nodes4 * (sizeof(Node4) + 4 * sizeof(int)) +
                        (uint64_t)m->n_nodes8 * (sizeof(Node8) + 8 * sizeof(int)) +
                        (m->d_tris8 ? (uint64_t)m->n_faces * sizeof(Tri) : 0ull);
    for (int k = 0; k < 3; ++k) { out->bounds_lo[k] = m->lo[k]; out->bounds_hi[k] = m->hi[k]; }
    return RMG_OK;
  });
}

extern "C" int rmg_map_export(const rmg_map* m, void* nodes, void* tris, uint32_t* leaf_order) {
  return guarded("rmg_map_export", [&]() -> int {
    if (!m) return fail(RMG_ERR_INVALID_ARG, "rmg_map_export: map is NULL");
    if (nodes && m->n_nodes)
      RMG_CUDA_TRY(cudaMemcpy(nodes, m->d_nodes, sizeof(Node) * m->n_nodes, cudaMemcpyDeviceToHost));
    if (tris && m->n_faces)
      RMG_CUDA_TRY(cudaMemcpy(tris, m->d_tris, sizeof(Tri) * m->n_faces, cudaMemcpyDeviceToHost));
    if (leaf_order && m->n_faces)
      RMG_CUDA_TRY(cudaMemcpy(leaf_order, m->d_leaf_order, 4ull * m->n_faces, cudaMemcpyDeviceToHost));
    return RMG_OK;
  });
}

// ---------------------------------------------------------------------------
// Map files: the built tree saved and loaded without a rebuild.  No
// counterpart in the reference (Embree / OptiX rebuild from the mesh on every
// import); for large maps a load is a file read plus host->device copies.
//
// Layout (little-endian):
//   char magic[8] = "RMGLBVH1"; uint32 version = 1;
//   uint32 n_vertices, n_faces, n_nodes, depth;
//   uint64 payload_bytes; uint64 fnv1a64(payload);
//   payload: vertices 12 B each, faces 12 B, nodes 64 B, packed triangles 48 B,
//            leaf order 4 B, leaf parents 4 B.
// A load checks the sizes, the checksum and every index the kernels follow
// (children, parents, face ids, leaf order, face vertex indices) on the host
// before anything reaches the device, so a damaged or crafted file is
// rejected with RMG_ERR_INVALID_ARG instead of steering a kernel out of bounds;
// the tree depth is recomputed from the links.
namespace {

constexpr char kMapMagic[8] = {'R', 'M', 'G', 'L', 'B', 'V', 'H', '1'};

struct MapFileHeader {
  char magic[8];
  uint32_t version;
  uint32_t n_vertices, n_faces, n_nodes, depth;
  uint32_t pad;
  uint64_t payload_bytes;
  uint64_t checksum;
};
static_assert(sizeof(MapFileHeader) == 48, "map file header is 48 B");

uint64_t fnv1a64(const unsigned char* p, size_t n) {
  uint64_t h = 1469598103934665603ull;
  for (size_t i = 0; i < n; ++i) {
    h ^= p[i];
    h *= 1099511628211ull;
  }
  return h;
}

uint64_t payload_size(uint64_t nv, uint64_t nf, uint64_t nn) {
  return 12 * nv + 12 * nf + sizeof(Node) * nn + sizeof(Tri) * nf + 4 * nf + 4 * nf;
}

// Index checks and depth of a loaded tree; returns RMG_OK or INVALID_ARG.
int check_tree(const MapFileHeader& h, const uint32_t* faces, const Node* nodes, const Tri* tris,
               const uint32_t* order, const int* leaf_parent, uint32_t* depth_out) {
  const uint32_t nv = h.n_vertices, nf = h.n_faces, nn = h.n_nodes;
  const uint32_t want_nodes = nf >= 2 ? nf - 1 : (nf == 1 ? 1 : 0);
  if (nn != want_nodes) return fail(RMG_ERR_INVALID_ARG, "rmg_map_load: node count does not match the face count");
  for (uint64_t i = 0; i < 3ull * nf; ++i)
    if (faces[i] >= nv) return fail(RMG_ERR_INVALID_ARG, "rmg_map_load: face vertex index out of range");
  for (uint32_t k = 0; k < nf; ++k) {
    uint32_t fid;
    std::memcpy(&fid, &tris[k].v0.w, 4);
    if (fid >= nf || order[k] >= nf) return fail(RMG_ERR_INVALID_ARG, "rmg_map_load: face id out of range");
    if (leaf_parent[k] < -1 || leaf_parent[k] >= (int)nn)
      return fail(RMG_ERR_INVALID_ARG, "rmg_map_load: leaf parent out of range");
  }
  std::vector<uint32_t> refs_node(nn, 0), refs_leaf(nf, 0);
  for (uint32_t i = 0; i < nn; ++i) {
    const int c[2] = {nodes[i].d.x, nodes[i].d.y};
    for (int k = 0; k < 2; ++k) {
      if (c[k] >= 0) {
        if ((uint32_t)c[k] >= nn || c[k] == 0) return fail(RMG_ERR_INVALID_ARG, "rmg_map_load: child out of range");
        ++refs_node[c[k]];
      } else {
        const uint32_t leaf = (uint32_t)(~c[k]);
        if (leaf >= nf) return fail(RMG_ERR_INVALID_ARG, "rmg_map_load: leaf out of range");
        ++refs_leaf[leaf];
      }
    }
    const int p = nodes[i].d.z;
    if (p < -1 || p >= (int)nn || (i == 0) != (p == -1)) return fail(RMG_ERR_INVALID_ARG, "rmg_map_load: bad parent link");
  }
  for (uint32_t i = 1; i < nn; ++i)
    if (refs_node[i] != 1) return fail(RMG_ERR_INVALID_ARG, "rmg_map_load: node not referenced exactly once");
  if (nf >= 2)
    for (uint32_t k = 0; k < nf; ++k)
      if (refs_leaf[k] != 1) return fail(RMG_ERR_INVALID_ARG, "rmg_map_load: leaf not referenced exactly once");
  // depth (edges) by an explicit walk from the root; every node is reached once
  uint32_t depth = nf ? 1 : 0;
  if (nn > 1) {
    std::vector<std::pair<int, uint32_t>> st;
    st.push_back({0, 0});
    size_t visited = 0;
    while (!st.empty()) {
      const auto [n, dd] = st.back();
      st.pop_back();
      if (++visited > nn) return fail(RMG_ERR_INVALID_ARG, "rmg_map_load: links do not form a tree");
      const int c[2] = {nodes[n].d.x, nodes[n].d.y};
      for (int k = 0; k < 2; ++k) {
        if (c[k] >= 0) st.push_back({c[k], dd + 1});
        else depth = std::max(depth, dd + 1);
      }
    }
    if (visited != nn) return fail(RMG_ERR_INVALID_ARG, "rmg_map_load: unreachable nodes");
  }
  *depth_out = depth;
  return RMG_OK;
}

}  // namespace

extern "C" int rmg_map_save(const rmg_map* m, const char* path) {
  return guarded("rmg_map_save", [&]() -> int {
    if (!m || !path) return fail(RMG_ERR_INVALID_ARG, "rmg_map_save: NULL argument");
    const uint64_t nv = m->n_vertices, nf = m->n_faces, nn = m->n_nodes;
    std::vector<unsigned char> payload(payload_size(nv, nf, nn));
    unsigned char* p = payload.data();
    auto dl = [&](const void* src, size_t bytes) -> int {
      if (bytes) RMG_CUDA_TRY(cudaMemcpy(p, src, bytes, cudaMemcpyDeviceToHost));
      p += bytes;
      return RMG_OK;
    };
    int s = RMG_OK;
    if (s == RMG_OK) s = dl(m->d_vertices, 12 * nv);
    if (s == RMG_OK) s = dl(m->d_faces, 12 * nf);
    if (s == RMG_OK) s = dl(m->d_nodes, sizeof(Node) * nn);
    if (s == RMG_OK) s = dl(m->d_tris, sizeof(Tri) * nf);
    if (s == RMG_OK) s = dl(m->d_leaf_order, 4 * nf);
    if (s == RMG_OK) s = dl(m->d_leaf_parent, 4 * nf);
    if (s != RMG_OK) return s;
    MapFileHeader h;
    std::memset(&h, 0, sizeof(h));
    std::memcpy(h.magic, kMapMagic, 8);
    h.version = 1;
    h.n_vertices = m->n_vertices;
    h.n_faces = m->n_faces;
    h.n_nodes = m->n_nodes;
    h.depth = m->depth;
    h.payload_bytes = payload.size();
    h.checksum = fnv1a64(payload.data(), payload.size());
    FILE* fp = std::fopen(path, "wb");
    if (!fp) return fail(RMG_ERR_INVALID_ARG, std::string("rmg_map_save: cannot write ") + path);
    bool ok = std::fwrite(&h, sizeof(h), 1, fp) == 1;
    ok = ok && (payload.empty() || std::fwrite(payload.data(), 1, payload.size(), fp) == payload.size());
    ok = (std::fclose(fp) == 0) && ok;
    return ok ? RMG_OK : fail(RMG_ERR_INVALID_ARG, "rmg_map_save: write failed");
  });
}

extern "C" int rmg_map_load(const char* path, void* stream, rmg_map** out) {
  return guarded("rmg_map_load", [&]() -> int {
    if (!path || !out) return fail(RMG_ERR_INVALID_ARG, "rmg_map_load: NULL argument");
    *out = nullptr;
    FILE* fp = std::fopen(path, "rb");
    if (!fp) return fail(RMG_ERR_INVALID_ARG, std::string("rmg_map_load: cannot read ") + path);
    MapFileHeader h;
    bool ok = std::fread(&h, sizeof(h), 1, fp) == 1;
    if (!ok || std::memcmp(h.magic, kMapMagic, 8) != 0 || h.version != 1) {
      std::fclose(fp);
      return fail(RMG_ERR_INVALID_ARG, "rmg_map_load: not a map file of this version");
    }
    if (h.n_faces > (1u << 30) || h.payload_bytes != payload_size(h.n_vertices, h.n_faces, h.n_nodes)) {
      std::fclose(fp);
      return fail(RMG_ERR_INVALID_ARG, "rmg_map_load: sizes in the header do not agree");
    }
    std::vector<unsigned char> payload(h.payload_bytes);
    ok = payload.empty() || std::fread(payload.data(), 1, payload.size(), fp) == payload.size();
    const bool trailing = std::fgetc(fp) != EOF;
    std::fclose(fp);
    if (!ok || trailing) return fail(RMG_ERR_INVALID_ARG, "rmg_map_load: file size does not match the header");
    if (fnv1a64(payload.data(), payload.size()) != h.checksum)
      return fail(RMG_ERR_INVALID_ARG, "rmg_map_load: checksum mismatch (damaged file)");
    const uint64_t nv = h.n_vertices, nf = h.n_faces, nn = h.n_nodes;
    const unsigned char* p = payload.data();
    const unsigned char* pv = p;
    const unsigned char* pf = pv + 12 * nv;
    const unsigned char* pn = pf + 12 * nf;
    const unsigned char* pt = pn + sizeof(Node) * nn;
    const unsigned char* po = pt + sizeof(Tri) * nf;
    const unsigned char* pp = po + 4 * nf;
    // aligned host copies for the checks
    std::vector<uint32_t> faces(3 * nf), order(nf);
    std::vector<Node> nodes(nn);
    std::vector<Tri> tris(nf);
    std::vector<int> parents(nf);
    if (nf) std::memcpy(faces.data(), pf, 12 * nf);
    if (nn) std::memcpy(nodes.data(), pn, sizeof(Node) * nn);
    if (nf) {
      std::memcpy(tris.data(), pt, sizeof(Tri) * nf);
      std::memcpy(order.data(), po, 4 * nf);
      std::memcpy(parents.data(), pp, 4 * nf);
    }
    uint32_t depth = 0;
    int s = check_tree(h, faces.data(), nodes.data(), tris.data(), order.data(), parents.data(), &depth);
    if (s != RMG_OK) return s;
    cudaStream_t st = as_stream(stream);
    rmg_map* m = new (std::nothrow) rmg_map;
    if (!m) return fail(RMG_ERR_OOM, "rmg_map_load: host allocation");
    std::memset(m, 0, sizeof(*m));
    cudaGetDevice(&m->device);
    m->n_vertices = h.n_vertices;
    m->n_faces = h.n_faces;
    m->n_nodes = h.n_nodes;
    m->depth = depth;
    auto check = [&](int r) { if (s == RMG_OK) s = r; };
    check(dev_alloc(&m->d_status, 1, "status"));
    check(dev_alloc(&m->d_vertices, 3 * nv, "vertices"));
    check(dev_alloc(&m->d_faces, 3 * nf, "faces"));
    check(dev_alloc(&m->d_nodes, nn, "nodes"));
    check(dev_alloc(&m->d_tris, nf, "tris"));
    check(dev_alloc(&m->d_leaf_order, nf, "leaf order"));
    check(dev_alloc(&m->d_leaf_parent, nf, "leaf parent"));
    check(dev_alloc(&m->d_flags, nn, "flags"));
    auto up = [&](void* dst, const void* src, size_t bytes) {
      if (s == RMG_OK && bytes) s = cuda_status(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, st), "upload");
    };
    if (s == RMG_OK) s = cuda_status(cudaMemsetAsync(m->d_status, 0, 4, st), "memset");
    up(m->d_vertices, pv, 12 * nv);
    up(m->d_faces, faces.data(), 12 * nf);
    up(m->d_nodes, nodes.data(), sizeof(Node) * nn);
    up(m->d_tris, tris.data(), sizeof(Tri) * nf);
    up(m->d_leaf_order, order.data(), 4 * nf);
    up(m->d_leaf_parent, parents.data(), 4 * nf);
    if (s == RMG_OK) s = cuda_status(cudaStreamSynchronize(st), "sync");
    if (s == RMG_OK) s = wide_build(m, st);
    if (s != RMG_OK) { free_map(m); return s; }
    update_info(m, st);
    *out = m;
    return RMG_OK;
  });
}

extern "C" int rmg_map_status(rmg_map* m, int clear) {
  return guarded("rmg_map_status", [&]() -> int {
    if (!m) return fail(RMG_ERR_INVALID_ARG, "rmg_map_status: map is NULL");
    unsigned int word = 0;
    RMG_CUDA_TRY(cudaMemcpy(&word, m->d_status, 4, cudaMemcpyDeviceToHost));
    if (clear) RMG_CUDA_TRY(cudaMemset(m->d_status, 0, 4));
    if (word != 0) {
      set_error("a kernel recorded a device error on this map");
      return (int)word;
    }
    return RMG_OK;
  });
}

extern "C" int rmg_map_debug_set_child(rmg_map* m, uint32_t node, uint32_t which, int32_t child) {
  return guarded("rmg_map_debug_set_child", [&]() -> int {
    if (!m) return fail(RMG_ERR_INVALID_ARG, "rmg_map_debug_set_child: map is NULL");
    if (which >= 2) {  // a slot of the 4-wide tree
      if (!m->d_nodes4 || node >= m->n_nodes4 || which > 5)
        return fail(RMG_ERR_INVALID_ARG, "rmg_map_debug_set_child: wide node/slot out of range");
      if (child >= 0 ? (uint32_t)child >= m->n_nodes4 : (uint32_t)(~child) >= m->n_faces)
        return fail(RMG_ERR_INVALID_ARG, "rmg_map_debug_set_child: child out of range");
      const size_t off = offsetof(Node4, child) + sizeof(int) * (which - 2);
      RMG_CUDA_TRY(cudaMemcpy(reinterpret_cast<char*>(m->d_nodes4 + node) + off, &child, sizeof(int),
                              cudaMemcpyHostToDevice));
      return RMG_OK;
    }
    if (node >= m->n_nodes)
      return fail(RMG_ERR_INVALID_ARG, "rmg_map_debug_set_child: node/which out of range");
    if (child >= 0 ? (uint32_t)child >= m->n_nodes : (uint32_t)(~child) >= m->n_faces)
      return fail(RMG_ERR_INVALID_ARG, "rmg_map_debug_set_child: child out of range");
    const size_t off = offsetof(Node, d) + (which ? sizeof(int) : 0);
    RMG_CUDA_TRY(cudaMemcpy(reinterpret_cast<char*>(m->d_nodes + node) + off, &child, sizeof(int),
                            cudaMemcpyHostToDevice));
    wide_free(m);  // the binary tree is the one damaged: walk it from now on
    return RMG_OK;
  });
}

// ---------------------------------------------------------------------------
// rmg_lbvh_build_noalloc: the LBVH build into caller-owned device memory,
// with no device allocation.  No counterpart in the reference.
//
// Callers that cannot allocate device memory (real-time loops whose allocator
// calls are forbidden, hosts that give the library one fixed device arena and
// own every other byte) still need temporary space for the Morton keys, their
// sorted copy, the sort's own temporary storage and the partial bounds.  That space is the file-scope array below:
// kNoAllocScratchBytes bytes that every GPU which loads this library holds
// until the process exits.  It bounds the mesh to RMG_NOALLOC_MAX_FACES.
//
// The first call on a device resolves the array's device address with
// cudaGetSymbolAddress (the host-side name is only a stand-in and must never
// be handed to a kernel).
// All calls share the one array and it keeps the previous call's contents:
// the words that must start at zero are cleared by each call, and calls whose
// work overlaps on the GPU (different streams, no ordering between them) race
// on the array and produce garbage.  The call synchronises with `stream` once,
// after checking the face indices on the device.
// ---------------------------------------------------------------------------
namespace rmg {
namespace {

constexpr size_t kNoAllocScratchBytes = 4u << 20;  // 4 MiB
static __device__ __align__(256) unsigned char g_lbvh_scratch[kNoAllocScratchBytes];

struct NoAllocSetup {
  bool ready = false;
  unsigned char* base = nullptr;
  size_t sort_temp_bytes = 0;  // CUB temporary storage needed for RMG_NOALLOC_MAX_FACES pairs
};

constexpr int kMaxDevices = 64;
NoAllocSetup g_noalloc[kMaxDevices];
std::mutex g_noalloc_mutex;

__global__ void k_check_faces(const uint32_t* f, uint32_t n_faces, uint32_t n_vertices, unsigned int* bad) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= 3 * n_faces) return;
  if (f[i] >= n_vertices) atomicExch(bad, 1u);
}

// The single-triangle tree of single_node(), on the device: the same min/max
// order (std::min / std::max semantics), leaf 0 under no parent, cleared flag.
__device__ __forceinline__ float min_like_std(float a, float b) { return b < a ? b : a; }
__device__ __forceinline__ float max_like_std(float a, float b) { return a < b ? b : a; }

__global__ void k_single_node(const float* v, const uint32_t* f, Node* node, uint32_t* leaf_order,
                              int32_t* leaf_parent, uint32_t* flags) {
  if (threadIdx.x != 0) return;
  float lo[3], hi[3];
  for (int k = 0; k < 3; ++k) {
    const float a = v[3ull * f[0] + k], b = v[3ull * f[1] + k], c = v[3ull * f[2] + k];
    lo[k] = min_like_std(min_like_std(a, b), c);
    hi[k] = max_like_std(max_like_std(a, b), c);
  }
  const float far = 1e30f;
  node->a = make_float4(lo[0], hi[0], lo[1], hi[1]);
  node->b = make_float4(far, far, far, far);
  node->c = make_float4(lo[2], hi[2], far, far);
  node->d = make_int4(-1, -1, -1, 0);
  leaf_order[0] = 0u;
  leaf_parent[0] = -1;
  flags[0] = 0u;
}

inline size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

int noalloc_setup(int dev, NoAllocSetup** out) {
  std::lock_guard<std::mutex> lock(g_noalloc_mutex);
  if (dev < 0 || dev >= kMaxDevices) return fail(RMG_ERR_NO_DEVICE, "rmg_lbvh_build_noalloc: device id");
  NoAllocSetup& s = g_noalloc[dev];
  if (!s.ready) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_lbvh_scratch);
    if (e != cudaSuccess) return cuda_status(e, "cudaGetSymbolAddress(g_lbvh_scratch)");
    size_t bytes = 0;
    const cudaError_t e2 = cub::DeviceRadixSort::SortPairs(
        nullptr, bytes, (const uint64_t*)nullptr, (uint64_t*)nullptr, (const uint32_t*)nullptr,
        (uint32_t*)nullptr, (int)RMG_NOALLOC_MAX_FACES, 0, 63);
    if (e2 != cudaSuccess) return cuda_status(e2, "sort temp size");
    s.base = static_cast<unsigned char*>(p);
    s.sort_temp_bytes = bytes;
    s.ready = true;
  }
  *out = &s;
  return RMG_OK;
}

}  // namespace
}  // namespace rmg

extern "C" int rmg_lbvh_build_noalloc(const rmg_vec3* vertices, uint32_t n_vertices, const rmg_face* faces,
                                      uint32_t n_faces, const rmg_lbvh_buffers* out, void* stream) {
  return guarded("rmg_lbvh_build_noalloc", [&]() -> int {
    if (!out) return fail(RMG_ERR_INVALID_ARG, "rmg_lbvh_build_noalloc: out is NULL");
    if (n_faces > RMG_NOALLOC_MAX_FACES)
      return fail(RMG_ERR_INVALID_ARG, "rmg_lbvh_build_noalloc: n_faces exceeds RMG_NOALLOC_MAX_FACES (65536)");
    if (n_faces == 0) return RMG_OK;
    if (!vertices || !faces || !out->nodes || !out->tris || !out->leaf_order || !out->leaf_parent || !out->flags)
      return fail(RMG_ERR_INVALID_ARG, "rmg_lbvh_build_noalloc: NULL input or output buffer");
    if ((reinterpret_cast<uintptr_t>(out->nodes) | reinterpret_cast<uintptr_t>(out->tris)) & 15u)
      return fail(RMG_ERR_INVALID_ARG, "rmg_lbvh_build_noalloc: nodes/tris must be 16-byte aligned");
    int dev = 0;
    RMG_CUDA_TRY(cudaGetDevice(&dev));
    NoAllocSetup* su = nullptr;
    int s = noalloc_setup(dev, &su);
    if (s != RMG_OK) return s;
  
    cudaStream_t st = as_stream(stream);
    const uint32_t n = n_faces;
    const int nb = std::min<int>((int)grid_for(n), 4 * device_sm_count());
    // carve the scratch array
    unsigned char* p = su->base;
    size_t off = 0;
    auto take = [&](size_t bytes) { unsigned char* q = p + off; off = align256(off + bytes); return q; };
    uint64_t* keys = reinterpret_cast<uint64_t*>(take(8ull * n));
    uint64_t* keys2 = reinterpret_cast<uint64_t*>(take(8ull * n));
    uint32_t* vals = reinterpret_cast<uint32_t*>(take(4ull * n));
    uint32_t* vals2 = reinterpret_cast<uint32_t*>(take(4ull * n));
    float* partial = reinterpret_cast<float*>(take(24ull * nb));
    float* bounds = reinterpret_cast<float*>(take(24));
    unsigned int* bad = reinterpret_cast<unsigned int*>(take(4));
    void* temp = take(su->sort_temp_bytes);
    size_t temp_bytes = 0;
    RMG_CUDA_TRY(cub::DeviceRadixSort::SortPairs(nullptr, temp_bytes, keys, keys2, vals, vals2, (int)n, 0, 63, st));
    if (off > kNoAllocScratchBytes || temp_bytes > su->sort_temp_bytes)
      return fail(RMG_ERR_INVALID_ARG, "rmg_lbvh_build_noalloc: scratch array too small for this mesh");
  
    const float* v = reinterpret_cast<const float*>(vertices);
    const uint32_t* f = reinterpret_cast<const uint32_t*>(faces);
    Node* nodes = static_cast<Node*>(out->nodes);
    Tri* tris = static_cast<Tri*>(out->tris);
  
    // face indices are checked on the device before any kernel dereferences them
    RMG_CUDA_TRY(cudaMemsetAsync(bad, 0, 4, st));
    k_check_faces<<<grid_for(3ull * n), kBlock, 0, st>>>(f, n, n_vertices, bad);
    RMG_CUDA_TRY(cudaGetLastError());
    unsigned int bad_h = 0;
    RMG_CUDA_TRY(cudaMemcpyAsync(&bad_h, bad, 4, cudaMemcpyDeviceToHost, st));
    RMG_CUDA_TRY(cudaStreamSynchronize(st));
    if (bad_h) return fail(RMG_ERR_INVALID_ARG, "rmg_lbvh_build_noalloc: face index out of range");
  
    if (n == 1) {  // one node with a phantom far-away right child, built on `stream` like the rest
      k_single_node<<<1, 32, 0, st>>>(v, f, nodes, out->leaf_order, out->leaf_parent, out->flags);
      k_pack<<<1, 32, 0, st>>>(v, f, out->leaf_order, 1, tris, nullptr);
      RMG_CUDA_TRY(cudaGetLastError());
      return RMG_OK;
    }
  
    k_centroid_bounds<<<nb, kBlock, 0, st>>>(v, f, n, partial);
    k_bounds_final<<<1, 32, 0, st>>>(partial, nb, bounds);
    k_morton<<<grid_for(n), kBlock, 0, st>>>(v, f, n, bounds, keys, vals);
    RMG_CUDA_TRY(cudaGetLastError());
    RMG_CUDA_TRY(cub::DeviceRadixSort::SortPairs(temp, temp_bytes, keys, keys2, vals, vals2, (int)n, 0, 63, st));
    RMG_CUDA_TRY(cudaMemsetAsync(nodes, 0, sizeof(Node) * (n - 1), st));
    k_karras<<<grid_for(n - 1), kBlock, 0, st>>>(keys2, (int)n, nodes, out->leaf_parent);
    k_pack<<<grid_for(n), kBlock, 0, st>>>(v, f, vals2, n, tris, out->leaf_order);
    RMG_CUDA_TRY(cudaGetLastError());
    RMG_CUDA_TRY(cudaMemsetAsync(out->flags, 0, 4ull * (n - 1), st));
    k_refit<<<grid_for(n), kBlock, 0, st>>>(nodes, tris, out->leaf_parent, out->flags, n);
    RMG_CUDA_TRY(cudaGetLastError());
    return RMG_OK;
  });
}
