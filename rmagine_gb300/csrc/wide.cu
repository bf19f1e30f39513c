// 4-wide tree collapsed from the binary LBVH.
//
// Same leaves (one packed triangle each) and the same boxes as the binary
// tree; a 4-wide node holds up to four children, chosen top-down: start from a
// binary node's two children and repeatedly open the internal child of
// largest surface area until four children are collected or only leaves
// remain (the greedy collapse of Wald, Benthin and Boulos, "Getting rid of
// packets", RT 2008, and of most wide-BVH builders since).  Every slot keeps
// the binary record its box came from (parent node and side), so after a
// binary refit the wide boxes are refreshed by one copy kernel.  Node indices
// are allocated level by level with an atomic counter; their order does not
// affect any result (the traversal's closest hit is order-independent).
#include <vector>

#include "internal.h"

namespace rmg {
namespace {

constexpr int kBlock4 = 256;

struct Cand {
  int id;        // binary child link: >= 0 internal node, < 0 leaf ~k
  int src;       // 2 * binary parent + side
  float lo[3], hi[3];
};

__device__ __forceinline__ Cand cand_of(const Node& n, int parent, int side) {
  Cand c;
  c.src = 2 * parent + side;
  if (side == 0) {
    c.id = n.d.x;
    c.lo[0] = n.a.x; c.hi[0] = n.a.y; c.lo[1] = n.a.z; c.hi[1] = n.a.w; c.lo[2] = n.c.x; c.hi[2] = n.c.y;
  } else {
    c.id = n.d.y;
    c.lo[0] = n.b.x; c.hi[0] = n.b.y; c.lo[1] = n.b.z; c.hi[1] = n.b.w; c.lo[2] = n.c.z; c.hi[2] = n.c.w;
  }
  return c;
}

__device__ __forceinline__ float half_area(const Cand& c) {
  const float ex = fmaxf(c.hi[0] - c.lo[0], 0.f), ey = fmaxf(c.hi[1] - c.lo[1], 0.f),
              ez = fmaxf(c.hi[2] - c.lo[2], 0.f);
  return ex * ey + ey * ez + ez * ex;
}

__device__ __forceinline__ void set_slot(Node4& w, int k, const float lo[3], const float hi[3]) {
  float* lox = &w.lox.x; float* hix = &w.hix.x; float* loy = &w.loy.x;
  float* hiy = &w.hiy.x; float* loz = &w.loz.x; float* hiz = &w.hiz.x;
  lox[k] = lo[0]; hix[k] = hi[0]; loy[k] = lo[1]; hiy[k] = hi[1]; loz[k] = lo[2]; hiz[k] = hi[2];
}

// One level of the collapse: wide nodes [lo4, hi4), whose binary roots are
// bin_of[j], get their children; internal children receive new wide indices.
__global__ void k_collapse(const Node* __restrict__ bn, int* bin_of, int* parent4, uint32_t lo4, uint32_t hi4,
                           Node4* w4, int* src4, unsigned int* count4) {
  const uint32_t j = lo4 + blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= hi4) return;
  const int b = bin_of[j];
  const Node root = bn[b];
  Cand c[4];
  c[0] = cand_of(root, b, 0);
  c[1] = cand_of(root, b, 1);
  int n = 2;
  if (root.d.x == root.d.y) n = 1;  // the one-triangle tree: both links name leaf 0
  while (n < 4) {
    int best = -1;
    float ba = -1.f;
    for (int k = 0; k < n; ++k) {
      if (c[k].id >= 0) {
        const float a = half_area(c[k]);
        if (a > ba) { ba = a; best = k; }
      }
    }
    if (best < 0) break;
    const int id = c[best].id;
    const Node nb = bn[id];
    c[best] = cand_of(nb, id, 0);
    c[n++] = cand_of(nb, id, 1);
  }
  Node4 w;
  const float far[3] = {1e30f, 1e30f, 1e30f};
  int child[4];
  for (int k = 0; k < 4; ++k) {
    if (k < n) {
      set_slot(w, k, c[k].lo, c[k].hi);
      if (c[k].id < 0) {
        child[k] = c[k].id;
      } else {
        const unsigned int k4 = atomicAdd(count4, 1u);
        bin_of[k4] = c[k].id;
        parent4[k4] = (int)j;
        child[k] = (int)k4;
      }
      src4[4 * j + k] = c[k].src;
    } else {
      set_slot(w, k, far, far);
      child[k] = kEmpty4;
      src4[4 * j + k] = -1;
    }
  }
  w.child = make_int4(child[0], child[1], child[2], child[3]);
  w.meta = make_int4(n, parent4[j], 0, 0);
  w4[j] = w;
}

// Boxes of every slot from the (refitted) binary records.
__global__ void k_wide_refit(const Node* __restrict__ bn, const int* __restrict__ src4, uint32_t n4, Node4* w4) {
  const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n4) return;
  Node4 w = w4[j];
  for (int k = 0; k < 4; ++k) {
    const int s = src4[4 * j + k];
    if (s < 0) continue;
    const Cand c = cand_of(bn[s >> 1], s >> 1, s & 1);
    set_slot(w, k, c.lo, c.hi);
  }
  w4[j] = w;
}

}  // namespace

void wide_free(rmg_map* m) {
  wide8_free(m);
  cudaFree(m->d_nodes4);
  cudaFree(m->d_src4);
  m->d_nodes4 = nullptr;
  m->d_src4 = nullptr;
  m->n_nodes4 = 0;
  m->depth4 = 0;
}

// Builds the 4-wide tree of a map whose binary tree is complete.  Synchronises.
int wide_build(rmg_map* m, cudaStream_t st) {
  wide_free(m);
  if (m->n_faces == 0) return RMG_OK;
  const uint32_t cap = std::max<uint32_t>(m->n_nodes, 1u);
  int* bin_of = nullptr;
  int* parent4 = nullptr;
  unsigned int* count4 = nullptr;
  int s = dev_alloc(&m->d_nodes4, cap, "wide nodes");
  if (s == RMG_OK) s = dev_alloc(&m->d_src4, 4 * (size_t)cap, "wide sources");
  if (s == RMG_OK) s = dev_alloc(&bin_of, cap, "wide roots");
  if (s == RMG_OK) s = dev_alloc(&parent4, cap, "wide parents");
  if (s == RMG_OK) s = dev_alloc(&count4, 1, "wide counter");
  const int zero = 0, minus1 = -1;
  const unsigned int one = 1;
  if (s == RMG_OK) s = cuda_status(cudaMemcpyAsync(bin_of, &zero, 4, cudaMemcpyHostToDevice, st), "wide init");
  if (s == RMG_OK) s = cuda_status(cudaMemcpyAsync(parent4, &minus1, 4, cudaMemcpyHostToDevice, st), "wide init");
  if (s == RMG_OK) s = cuda_status(cudaMemcpyAsync(count4, &one, 4, cudaMemcpyHostToDevice, st), "wide init");
  uint32_t lo4 = 0, hi4 = 1, levels = 0;
  while (s == RMG_OK && lo4 < hi4) {
    const uint32_t n = hi4 - lo4;
    k_collapse<<<(n + kBlock4 - 1) / kBlock4, kBlock4, 0, st>>>(m->d_nodes, bin_of, parent4, lo4, hi4, m->d_nodes4,
                                                                m->d_src4, count4);
    s = cuda_status(cudaGetLastError(), "k_collapse");
    unsigned int c = 0;
    if (s == RMG_OK) s = cuda_status(cudaMemcpyAsync(&c, count4, 4, cudaMemcpyDeviceToHost, st), "wide count");
    if (s == RMG_OK) s = cuda_status(cudaStreamSynchronize(st), "wide sync");
    ++levels;
    lo4 = hi4;
    hi4 = c;
    if (hi4 > cap) s = fail(RMG_ERR_CUDA, "wide build: node count exceeds the binary tree");
  }
  cudaFree(bin_of);
  cudaFree(parent4);
  cudaFree(count4);
  if (s != RMG_OK) { wide_free(m); return s; }
  m->n_nodes4 = hi4;
  m->depth4 = levels;
  return RMG_OK;
}

// Refreshes the wide boxes after the binary tree was refitted (asynchronous).
int wide_refit(rmg_map* m, cudaStream_t st) {
  if (!m->d_nodes4 || m->n_nodes4 == 0) return RMG_OK;
  k_wide_refit<<<(m->n_nodes4 + kBlock4 - 1) / kBlock4, kBlock4, 0, st>>>(m->d_nodes, m->d_src4, m->n_nodes4,
                                                                        m->d_nodes4);
  const int s = cuda_status(cudaGetLastError(), "k_wide_refit");
  return s == RMG_OK ? wide8_refit(m, st) : s;
}

}  // namespace rmg
