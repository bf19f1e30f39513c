// Top-down binned-SAH build of a binary BVH with one triangle per leaf, on the
// GPU, level by level: the binned surface area heuristic of Wald ("On fast
// construction of SAH-based bounding volume hierarchies", IEEE RT 2007),
// breadth-first over all nodes of a level at once.
//
// Every internal node of the current level is a task: a contiguous range of
// the triangle permutation plus the bounds of its triangles' centroids.  Per
// level:
//   1. binning: each triangle of a task falls into one of kNB bins per axis
//      over the task's centroid bounds (centroid: the centre of the
//      triangle's box); a bin accumulates the count, the box
//      and the centroid bounds of its triangles (atomics on order-preserving
//      integer images of the floats, privatised in shared memory when a CTA's
//      triangles all belong to one task);
//   2. split: per task, the split plane between bins of least surface area
//      heuristic cost A_L * N_L + A_R * N_R over the three axes; a task whose
//      centroids coincide, or whose best split would let the tree grow deeper
//      than kMaxDepth, is halved by position instead;
//   3. children: a task's sides of one triangle become leaves, the others
//      internal nodes of the next level, numbered by an exclusive scan over
//      the tasks (so the numbering, like everything else here, does not depend
//      on thread timing);
//   4. partition: a stable partition of every task's range (one exclusive scan
//      over "goes left" flags of all positions) writes the next permutation.
// The leaf of position k holds the k-th triangle of the final permutation.
// Boxes are left to the caller's refit.  The same binning (16 bins over the
// centroid bounds) and cost as the oracle's SAH tree, in binary32.
#include <cub/cub.cuh>

#include <algorithm>
#include <vector>

#include "internal.h"

namespace rmg {
namespace {

#ifndef RMG_SAH_BINS
#define RMG_SAH_BINS 16
#endif
constexpr int kNB = RMG_SAH_BINS;     // bins per axis
constexpr int kBlk = 256;
constexpr uint32_t kBatch = 32768;    // tasks whose bins are held at once
constexpr uint32_t kMaxDepth = 32;    // leaves at most this many edges below the root

struct Task {
  uint32_t first, count;
  int node;        // internal node id
  uint32_t depth;  // edges from the root
  float clo[3], chi[3];  // bounds of the centroids
};

struct Split {
  int axis;          // -1: halved by position
  int bin;           // bins 0..bin go left
  uint32_t left;     // triangles going left
  int ltask, rtask;  // next-level task of each side, -1 for a leaf
  float lclo[3], lchi[3], rclo[3], rchi[3];
};

// count, box lo/hi, centroid lo/hi; floats as order-preserving ints
struct Bin {
  int cnt;
  int blo[3], bhi[3], clo[3], chi[3];
};

__device__ __forceinline__ int f2o(float f) {
  const int b = __float_as_int(f);
  return b >= 0 ? b : b ^ 0x7fffffff;
}
__device__ __forceinline__ float o2f(int o) { return __int_as_float(o >= 0 ? o : o ^ 0x7fffffff); }

__device__ __forceinline__ int ceil_log2(uint32_t x) { return x <= 1 ? 0 : 32 - __clz(x - 1); }

__device__ __forceinline__ float3 tri_v(const float* v, uint32_t i) {
  return make_float3(v[3 * i], v[3 * i + 1], v[3 * i + 2]);
}

// Centroids and boxes of all triangles; identity permutation; one task.
__global__ void k_prep(const float* v, const uint32_t* f, uint32_t n, float4* cen, float4* blo, float4* bhi,
                       uint32_t* idx, int* ptask, int* root_bounds) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  float c[3] = {INFINITY, INFINITY, INFINITY};
  if (i < n) {
    const float3 a = tri_v(v, f[3 * i]), b = tri_v(v, f[3 * i + 1]), d = tri_v(v, f[3 * i + 2]);
    const float4 lo = make_float4(fminf(fminf(a.x, b.x), d.x), fminf(fminf(a.y, b.y), d.y),
                                  fminf(fminf(a.z, b.z), d.z), 0.f);
    const float4 hi = make_float4(fmaxf(fmaxf(a.x, b.x), d.x), fmaxf(fmaxf(a.y, b.y), d.y),
                                  fmaxf(fmaxf(a.z, b.z), d.z), 0.f);
    // the centre of the triangle's box (not the vertex mean: on a box room the
    // vertex mean of a large wall triangle sits a third of the way across the
    // wall, and the tree costs 13% more node visits per ray)
    c[0] = __fmul_rn(__fadd_rn(lo.x, hi.x), 0.5f);
    c[1] = __fmul_rn(__fadd_rn(lo.y, hi.y), 0.5f);
    c[2] = __fmul_rn(__fadd_rn(lo.z, hi.z), 0.5f);
    cen[i] = make_float4(c[0], c[1], c[2], 0.f);
    blo[i] = lo;
    bhi[i] = hi;
    idx[i] = i;
    ptask[i] = 0;
  }
  for (int k = 0; k < 3; ++k) {
    float lo = c[k], hi = i < n ? c[k] : -INFINITY;
    for (int o = 16; o > 0; o >>= 1) {
      lo = fminf(lo, __shfl_xor_sync(0xffffffffu, lo, o));
      hi = fmaxf(hi, __shfl_xor_sync(0xffffffffu, hi, o));
    }
    if ((threadIdx.x & 31) == 0) {
      atomicMin(&root_bounds[k], f2o(lo));
      atomicMax(&root_bounds[3 + k], f2o(hi));
    }
  }
}

__global__ void k_root(const int* root_bounds, uint32_t n, Task* tasks) {
  Task t;
  t.first = 0;
  t.count = n;
  t.node = 0;
  t.depth = 0;
  for (int k = 0; k < 3; ++k) { t.clo[k] = o2f(root_bounds[k]); t.chi[k] = o2f(root_bounds[3 + k]); }
  tasks[0] = t;
}

__global__ void k_bin_clear(Bin* bins, uint32_t nbins) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nbins) return;
  Bin b;
  b.cnt = 0;
  for (int k = 0; k < 3; ++k) {
    b.blo[k] = b.clo[k] = f2o(INFINITY);
    b.bhi[k] = b.chi[k] = f2o(-INFINITY);
  }
  bins[i] = b;
}

// Bin of centroid coordinate c in a task's bounds [lo, hi] (the same float
// operations wherever a bin is computed).
__device__ __forceinline__ int bin_of(float c, float lo, float hi) {
  const float ext = __fsub_rn(hi, lo);
  if (!(ext > 0.f)) return 0;
  const float s = __fdiv_rn((float)kNB, ext);
  const int b = (int)__fmul_rn(__fsub_rn(c, lo), s);
  return min(max(b, 0), kNB - 1);
}

__device__ __forceinline__ void bin_add(Bin* B, const float4& c, const float4& lo, const float4& hi) {
  atomicAdd(&B->cnt, 1);
  const float cc[3] = {c.x, c.y, c.z}, ll[3] = {lo.x, lo.y, lo.z}, hh[3] = {hi.x, hi.y, hi.z};
  for (int k = 0; k < 3; ++k) {
    atomicMin(&B->blo[k], f2o(ll[k]));
    atomicMax(&B->bhi[k], f2o(hh[k]));
    atomicMin(&B->clo[k], f2o(cc[k]));
    atomicMax(&B->chi[k], f2o(cc[k]));
  }
}

// Bins of tasks [t0, t0 + nt) over positions [pos0, pos1).
__global__ void __launch_bounds__(kBlk) k_bin(const int* ptask, const uint32_t* idx, const float4* cen,
                                              const float4* blo, const float4* bhi, const Task* tasks, uint32_t t0,
                                              uint32_t nt, uint32_t pos0, uint32_t pos1, Bin* bins) {
  __shared__ Bin sb[3 * kNB];
  __shared__ int tmin, tmax;
  const uint32_t pos = pos0 + blockIdx.x * blockDim.x + threadIdx.x;
  int t = pos < pos1 ? ptask[pos] : -1;
  if (t >= 0 && ((uint32_t)t < t0 || (uint32_t)t >= t0 + nt)) t = -1;
  if (threadIdx.x == 0) { tmin = 0x7fffffff; tmax = -1; }
  for (int i = threadIdx.x; i < 3 * kNB; i += blockDim.x) {
    sb[i].cnt = 0;
    for (int k = 0; k < 3; ++k) {
      sb[i].blo[k] = sb[i].clo[k] = f2o(INFINITY);
      sb[i].bhi[k] = sb[i].chi[k] = f2o(-INFINITY);
    }
  }
  __syncthreads();
  if (t >= 0) { atomicMin(&tmin, t); atomicMax(&tmax, t); }
  __syncthreads();
  if (tmax < 0) return;  // uniform: no triangle of these tasks here
  const bool shared_bins = tmin == tmax;
  if (t >= 0) {
    const Task& T = tasks[t];
    const uint32_t p = idx[pos];
    const float4 c = cen[p], lo = blo[p], hi = bhi[p];
    const float cc[3] = {c.x, c.y, c.z};
    Bin* base = shared_bins ? sb : bins + (size_t)(t - t0) * 3 * kNB;
    for (int a = 0; a < 3; ++a) bin_add(&base[a * kNB + bin_of(cc[a], T.clo[a], T.chi[a])], c, lo, hi);
  }
  if (!shared_bins) return;
  __syncthreads();
  Bin* g = bins + (size_t)(tmin - t0) * 3 * kNB;
  for (int i = threadIdx.x; i < 3 * kNB; i += blockDim.x) {
    const Bin& s = sb[i];
    if (s.cnt == 0) continue;
    atomicAdd(&g[i].cnt, s.cnt);
    for (int k = 0; k < 3; ++k) {
      atomicMin(&g[i].blo[k], s.blo[k]);
      atomicMax(&g[i].bhi[k], s.bhi[k]);
      atomicMin(&g[i].clo[k], s.clo[k]);
      atomicMax(&g[i].chi[k], s.chi[k]);
    }
  }
}

__device__ __forceinline__ float half_area(const float lo[3], const float hi[3]) {
  const float ex = fmaxf(hi[0] - lo[0], 0.f), ey = fmaxf(hi[1] - lo[1], 0.f), ez = fmaxf(hi[2] - lo[2], 0.f);
  return ex * ey + ey * ez + ez * ex;
}

// One thread per task: the least-cost split (or halving) of tasks [t0, t0 + nt).
__global__ void k_split(const Task* tasks, uint32_t t0, uint32_t nt, const Bin* bins, Split* splits) {
  const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= nt) return;
  const Task T = tasks[t0 + j];
  const Bin* B = bins + (size_t)j * 3 * kNB;
  const uint32_t n = T.count;
  float best = INFINITY;
  int best_axis = -1, best_bin = -1;
  uint32_t best_left = 0;
  for (int a = 0; a < 3; ++a) {
    // suffix areas and counts of bins k..kNB-1
    float rarea[kNB];
    uint32_t rcnt[kNB];
    float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    uint32_t c = 0;
    for (int k = kNB - 1; k >= 0; --k) {
      const Bin& b = B[a * kNB + k];
      c += (uint32_t)b.cnt;
      for (int q = 0; q < 3; ++q) { lo[q] = fminf(lo[q], o2f(b.blo[q])); hi[q] = fmaxf(hi[q], o2f(b.bhi[q])); }
      rarea[k] = half_area(lo, hi);
      rcnt[k] = c;
    }
    for (int q = 0; q < 3; ++q) { lo[q] = INFINITY; hi[q] = -INFINITY; }
    c = 0;
    for (int k = 0; k < kNB - 1; ++k) {
      const Bin& b = B[a * kNB + k];
      c += (uint32_t)b.cnt;
      for (int q = 0; q < 3; ++q) { lo[q] = fminf(lo[q], o2f(b.blo[q])); hi[q] = fmaxf(hi[q], o2f(b.bhi[q])); }
      const uint32_t r = rcnt[k + 1];
      if (c == 0 || r == 0) continue;
      if (T.depth + 1 + ceil_log2(c) > kMaxDepth || T.depth + 1 + ceil_log2(r) > kMaxDepth) continue;
      const float cost = half_area(lo, hi) * (float)c + rarea[k + 1] * (float)r;
      if (cost < best) { best = cost; best_axis = a; best_bin = k; best_left = c; }
    }
  }
  Split s;
  s.axis = best_axis;
  s.bin = best_bin;
  s.ltask = s.rtask = -1;
  if (best_axis < 0) {
    s.left = n / 2;
    for (int q = 0; q < 3; ++q) { s.lclo[q] = s.rclo[q] = T.clo[q]; s.lchi[q] = s.rchi[q] = T.chi[q]; }
  } else {
    s.left = best_left;
    for (int q = 0; q < 3; ++q) { s.lclo[q] = s.rclo[q] = INFINITY; s.lchi[q] = s.rchi[q] = -INFINITY; }
    for (int k = 0; k < kNB; ++k) {
      const Bin& b = B[best_axis * kNB + k];
      if (b.cnt == 0) continue;
      float* clo = k <= best_bin ? s.lclo : s.rclo;
      float* chi = k <= best_bin ? s.lchi : s.rchi;
      for (int q = 0; q < 3; ++q) { clo[q] = fminf(clo[q], o2f(b.clo[q])); chi[q] = fmaxf(chi[q], o2f(b.chi[q])); }
    }
  }
  splits[t0 + j] = s;
}

__global__ void k_child_count(const Task* tasks, const Split* splits, uint32_t nt, uint32_t* cnt) {
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nt) return;
  const uint32_t L = splits[t].left, R = tasks[t].count - L;
  cnt[t] = (L > 1 ? 1u : 0u) + (R > 1 ? 1u : 0u);
}

// Links of the level's nodes, parents of their children, next-level tasks
// (and the first position of every kBatch-th of them).
__global__ void k_create(const Task* tasks, Split* splits, const uint32_t* offs, uint32_t nt, int node_base,
                         Node* nodes, int* leaf_parent, Task* next, uint32_t* batch_first) {
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nt) return;
  const Task T = tasks[t];
  Split& s = splits[t];
  const uint32_t L = s.left, R = T.count - L;
  uint32_t o = offs[t];
  int link[2];
  const uint32_t first[2] = {T.first, T.first + L}, count[2] = {L, R};
  for (int side = 0; side < 2; ++side) {
    if (count[side] == 1) {
      link[side] = ~(int)first[side];
      leaf_parent[first[side]] = T.node;
      if (side == 0) s.ltask = -1; else s.rtask = -1;
    } else {
      const int id = node_base + (int)o;
      link[side] = id;
      nodes[id].d.z = T.node;
      Task c;
      c.first = first[side];
      c.count = count[side];
      c.node = id;
      c.depth = T.depth + 1;
      for (int q = 0; q < 3; ++q) {
        c.clo[q] = side == 0 ? s.lclo[q] : s.rclo[q];
        c.chi[q] = side == 0 ? s.lchi[q] : s.rchi[q];
      }
      next[o] = c;
      if (o % kBatch == 0) batch_first[o / kBatch] = c.first;
      if (side == 0) s.ltask = (int)o; else s.rtask = (int)o;
      ++o;
    }
  }
  nodes[T.node].d.x = link[0];
  nodes[T.node].d.y = link[1];
  nodes[T.node].d.w = 0;
  if (T.node == 0) nodes[0].d.z = -1;
}

__device__ __forceinline__ bool goes_left(const Task& T, const Split& s, uint32_t pos, const float4& c) {
  if (s.axis < 0) return pos - T.first < s.left;
  const float cc[3] = {c.x, c.y, c.z};
  return bin_of(cc[s.axis], T.clo[s.axis], T.chi[s.axis]) <= s.bin;
}

__global__ void k_flags(const int* ptask, const uint32_t* idx, const float4* cen, const Task* tasks,
                        const Split* splits, uint32_t n, uint32_t* fl) {
  const uint32_t pos = blockIdx.x * blockDim.x + threadIdx.x;
  if (pos >= n) return;
  const int t = ptask[pos];
  fl[pos] = (t >= 0 && goes_left(tasks[t], splits[t], pos, cen[idx[pos]])) ? 1u : 0u;
}

// A position that would leave its task's range (flags disagreeing with the
// split's count: never for consistent bins) is not written; it sets *bad.
__global__ void k_scatter(const int* ptask, const uint32_t* idx, const Task* tasks, const Split* splits,
                          const uint32_t* fl, const uint32_t* rk, uint32_t n, uint32_t* idx2, int* ptask2,
                          unsigned int* bad) {
  const uint32_t pos = blockIdx.x * blockDim.x + threadIdx.x;
  if (pos >= n) return;
  const int t = ptask[pos];
  if (t < 0) {
    idx2[pos] = idx[pos];
    ptask2[pos] = -1;
    return;
  }
  const Task T = tasks[t];
  const Split& s = splits[t];
  const uint32_t lrank = rk[pos] - rk[T.first];
  uint32_t np;
  int nt;
  if (fl[pos]) { np = T.first + lrank; nt = s.ltask; }
  else { np = T.first + s.left + (pos - T.first - lrank); nt = s.rtask; }
  if (np - T.first >= T.count) { atomicOr(bad, 1u); return; }
  idx2[np] = idx[pos];
  ptask2[np] = nt;
}

inline unsigned blocks(size_t n) { return (unsigned)((n + kBlk - 1) / kBlk); }

}  // namespace

// Topology of a one-triangle-per-leaf SAH tree over the map's n >= 2 faces:
// child links and parents in m->d_nodes (boxes zero), m->d_leaf_parent, and
// the face of every leaf in d_order.  Synchronises.
int sah_build_topology(rmg_map* m, cudaStream_t st, uint32_t* d_order) {
  const uint32_t n = m->n_faces;
  if (n < 2) return fail(RMG_ERR_INVALID_ARG, "SAH build needs two or more faces");
  float4 *cen = nullptr, *blo = nullptr, *bhi = nullptr;
  uint32_t *idx2 = nullptr, *fl = nullptr, *rk = nullptr, *cnt = nullptr, *offs = nullptr, *batch_first = nullptr;
  int *ptask = nullptr, *ptask2 = nullptr, *root_bounds = nullptr;
  unsigned int* bad = nullptr;
  Task *tasks = nullptr, *next = nullptr;
  Split* splits = nullptr;
  Bin* bins = nullptr;
  void* temp = nullptr;
  size_t temp_bytes = 0, t2 = 0;
  const uint32_t max_tasks = n / 2 + 1;
  const uint32_t max_batches = max_tasks / kBatch + 2;
  int s = RMG_OK;
  auto chk = [&](int r) { if (s == RMG_OK) s = r; };
  chk(dev_alloc(&cen, n, "sah centroids"));
  chk(dev_alloc(&blo, n, "sah boxes"));
  chk(dev_alloc(&bhi, n, "sah boxes"));
  chk(dev_alloc(&idx2, n, "sah permutation"));
  chk(dev_alloc(&fl, n, "sah flags"));
  chk(dev_alloc(&rk, n, "sah ranks"));
  chk(dev_alloc(&ptask, n, "sah tasks of positions"));
  chk(dev_alloc(&ptask2, n, "sah tasks of positions"));
  chk(dev_alloc(&root_bounds, 6, "sah root bounds"));
  chk(dev_alloc(&bad, 1, "sah error word"));
  chk(dev_alloc(&tasks, max_tasks, "sah tasks"));
  chk(dev_alloc(&next, max_tasks, "sah tasks"));
  chk(dev_alloc(&splits, max_tasks, "sah splits"));
  chk(dev_alloc(&cnt, max_tasks, "sah child counts"));
  chk(dev_alloc(&offs, max_tasks, "sah child offsets"));
  chk(dev_alloc(&batch_first, max_batches, "sah batch starts"));
  chk(dev_alloc(&bins, (size_t)std::min<uint32_t>(kBatch, max_tasks) * 3 * kNB, "sah bins"));
  if (s == RMG_OK)
    s = cuda_status(cub::DeviceScan::ExclusiveSum(nullptr, temp_bytes, fl, rk, (int)n, st), "scan size");
  if (s == RMG_OK)
    s = cuda_status(cub::DeviceScan::ExclusiveSum(nullptr, t2, cnt, offs, (int)max_tasks, st), "scan size");
  temp_bytes = std::max(temp_bytes, t2);
  if (s == RMG_OK) {
    char* tmp = nullptr;
    s = dev_alloc(&tmp, temp_bytes, "sah scan temp");
    temp = tmp;
  }
  uint32_t* idx = d_order;
  if (s == RMG_OK) {
    const int init[6] = {0x7f800000, 0x7f800000, 0x7f800000, (int)0x807fffff, (int)0x807fffff, (int)0x807fffff};
    s = cuda_status(cudaMemcpyAsync(root_bounds, init, sizeof(init), cudaMemcpyHostToDevice, st), "sah init");
  }
  if (s == RMG_OK) s = cuda_status(cudaMemsetAsync(m->d_nodes, 0, sizeof(Node) * m->n_nodes, st), "sah init");
  if (s == RMG_OK) s = cuda_status(cudaMemsetAsync(bad, 0, 4, st), "sah init");
  if (s == RMG_OK) {
    k_prep<<<blocks(n), kBlk, 0, st>>>(m->d_vertices, m->d_faces, n, cen, blo, bhi, idx, ptask, root_bounds);
    k_root<<<1, 1, 0, st>>>(root_bounds, n, tasks);
    s = cuda_status(cudaGetLastError(), "sah prep");
  }
  uint32_t T = 1;
  int node_base = 1;
  std::vector<uint32_t> starts{0};
  unsigned levels = 0;
  while (s == RMG_OK && T > 0) {
    if (++levels > 4 * kMaxDepth) { s = fail(RMG_ERR_CUDA, "SAH build: too many levels"); break; }
    // bins and splits, kBatch tasks at a time
    const uint32_t nb = (T + kBatch - 1) / kBatch;
    for (uint32_t b = 0; s == RMG_OK && b < nb; ++b) {
      const uint32_t t0 = b * kBatch, nt = std::min(kBatch, T - t0);
      const uint32_t pos0 = starts[b], pos1 = b + 1 < nb ? starts[b + 1] : n;
      k_bin_clear<<<blocks((size_t)nt * 3 * kNB), kBlk, 0, st>>>(bins, nt * 3 * kNB);
      if (pos1 > pos0) {
        k_bin<<<blocks(pos1 - pos0), kBlk, 0, st>>>(ptask, idx, cen, blo, bhi, tasks, t0, nt, pos0, pos1, bins);
      }
      k_split<<<blocks(nt), kBlk, 0, st>>>(tasks, t0, nt, bins, splits);
      s = cuda_status(cudaGetLastError(), "sah bin/split");
    }
    if (s != RMG_OK) break;
    k_child_count<<<blocks(T), kBlk, 0, st>>>(tasks, splits, T, cnt);
    s = cuda_status(cub::DeviceScan::ExclusiveSum(temp, temp_bytes, cnt, offs, (int)T, st), "sah task scan");
    if (s != RMG_OK) break;
    k_create<<<blocks(T), kBlk, 0, st>>>(tasks, splits, offs, T, node_base, m->d_nodes, m->d_leaf_parent, next,
                                         batch_first);
    k_flags<<<blocks(n), kBlk, 0, st>>>(ptask, idx, cen, tasks, splits, n, fl);
    s = cuda_status(cudaGetLastError(), "sah create/flags");
    if (s == RMG_OK) s = cuda_status(cub::DeviceScan::ExclusiveSum(temp, temp_bytes, fl, rk, (int)n, st), "sah scan");
    if (s != RMG_OK) break;
    k_scatter<<<blocks(n), kBlk, 0, st>>>(ptask, idx, tasks, splits, fl, rk, n, idx2, ptask2, bad);
    s = cuda_status(cudaGetLastError(), "sah scatter");
    if (s != RMG_OK) break;
    // next level's task count (last offset + last count) and batch starts
    uint32_t last[3] = {0, 0, 0};
    s = cuda_status(cudaMemcpyAsync(&last[0], offs + (T - 1), 4, cudaMemcpyDeviceToHost, st), "sah count");
    if (s == RMG_OK) s = cuda_status(cudaMemcpyAsync(&last[1], cnt + (T - 1), 4, cudaMemcpyDeviceToHost, st), "sah count");
    if (s == RMG_OK) s = cuda_status(cudaMemcpyAsync(&last[2], bad, 4, cudaMemcpyDeviceToHost, st), "sah check");
    if (s == RMG_OK) s = cuda_status(cudaStreamSynchronize(st), "sah sync");
    if (s != RMG_OK) break;
    if (last[2]) { s = fail(RMG_ERR_CUDA, "SAH build: partition disagrees with the split counts"); break; }
    const uint32_t Tn = last[0] + last[1];
    if (Tn > max_tasks || node_base + Tn > m->n_nodes) { s = fail(RMG_ERR_CUDA, "SAH build: node count overflow"); break; }
    starts.assign((Tn + kBatch - 1) / kBatch, 0);
    if (!starts.empty()) {
      s = cuda_status(cudaMemcpyAsync(starts.data(), batch_first, 4 * starts.size(), cudaMemcpyDeviceToHost, st),
                      "sah batch starts");
      if (s == RMG_OK) s = cuda_status(cudaStreamSynchronize(st), "sah sync");
    }
    std::swap(idx, idx2);
    std::swap(ptask, ptask2);
    std::swap(tasks, next);
    node_base += (int)Tn;
    T = Tn;
  }
  if (s == RMG_OK && node_base != (int)m->n_nodes) s = fail(RMG_ERR_CUDA, "SAH build: node count mismatch");
  if (s == RMG_OK && idx != d_order)
    s = cuda_status(cudaMemcpyAsync(d_order, idx, 4 * (size_t)n, cudaMemcpyDeviceToDevice, st), "sah order");
  if (s == RMG_OK) s = cuda_status(cudaStreamSynchronize(st), "sah sync");
  // idx2 may now be d_order (swapped): free the scratch permutation only
  cudaFree(idx == d_order ? idx2 : idx);
  cudaFree(cen); cudaFree(blo); cudaFree(bhi); cudaFree(fl); cudaFree(rk);
  cudaFree(ptask); cudaFree(ptask2); cudaFree(root_bounds); cudaFree(bad); cudaFree(tasks); cudaFree(next);
  cudaFree(splits); cudaFree(cnt); cudaFree(offs); cudaFree(batch_first); cudaFree(bins); cudaFree(temp);
  return s;
}

}  // namespace rmg
