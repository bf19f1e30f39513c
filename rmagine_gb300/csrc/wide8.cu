// 8-wide tree with quantized child boxes, collapsed from the binary tree.
//
// The layout follows the compressed wide BVH of Ylitie, Karras and Laine,
// "Efficient Incoherent Ray Traversal on GPUs Through Compressed Wide BVHs"
// (HPG 2017): one 80-byte record holds up to eight children, each child box
// stored as six 8-bit offsets on a per-node grid (origin p, power-of-two cell
// 2^e per axis), rounded outward so that every quantized box contains its
// child's exact box.  Children are collected top-down from the binary tree by
// opening the internal candidate of largest surface area until eight are held
// or only leaves remain (as the 4-wide collapse in wide.cu), and placed in
// slots by direction: slot s takes the child whose centroid lies farthest
// towards (+-1, +-1, +-1) with the signs of s's bits, so that for a ray whose
// direction has octant bits o the order s ^ o is roughly nearest first.
// Internal children are stored contiguously from child_base in slot order,
// leaf children (one triangle each) contiguously from tri_base in a copy of
// the packed triangles (tris8).  Every slot keeps the binary record its box
// came from, so a binary refit re-quantizes the 8-wide boxes in one kernel.
// The binary tree's boxes are exact triangle bounds, so the closest hit of a
// walk of this tree is the same as of the binary one (conservative boxes, same
// triangle test and tie rule).
#include <vector>

#include "internal.h"

namespace rmg {
namespace {

constexpr int kBlock8 = 128;
constexpr int kMinExp = -100;  // cell exponent range: keeps 2^e * (1/d) normal and finite for
constexpr int kMaxExp = 60;    // every |1/d| in [1, 1e20] the walk can meet

struct Cand8 {
  int id;   // binary child link: >= 0 internal node, < 0 leaf ~k
  int src;  // 2 * binary parent + side
  float lo[3], hi[3];
};

__device__ __forceinline__ Cand8 cand8_of(const Node& n, int parent, int side) {
  Cand8 c;
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

__device__ __forceinline__ float half_area8(const Cand8& c) {
  const float ex = fmaxf(c.hi[0] - c.lo[0], 0.f), ey = fmaxf(c.hi[1] - c.lo[1], 0.f),
              ez = fmaxf(c.hi[2] - c.lo[2], 0.f);
  return ex * ey + ey * ez + ez * ex;
}

// Grid of one axis: origin p = lo and the smallest exponent e with
// lo + 255 * 2^e >= hi (checked in binary64, where these sums are exact).
// Returns false when the extent needs a cell above 2^kMaxExp.
__device__ __forceinline__ bool axis_grid(float lo, float hi, int& e) {
  const double ext = (double)hi - (double)lo;
  if (!(ext > 0.0)) { e = kMinExp; return true; }
  int k;
  frexp(ext / 255.0, &k);  // ext / 255 < 2^k
  e = k - 1;
  if (e < kMinExp) e = kMinExp;
  while (e <= kMaxExp && (double)lo + 255.0 * ldexp(1.0, e) < (double)hi) ++e;
  return e <= kMaxExp;
}

// Quantized record of one 8-wide node from its slot candidates (slot k empty
// when used[k] is false).  Returns false when a box is too large to quantize.
__device__ bool quantize_node(const Cand8* slot, const bool* used, Node8& w) {
  float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
  for (int k = 0; k < 8; ++k) {
    if (!used[k]) continue;
    for (int a = 0; a < 3; ++a) { lo[a] = fminf(lo[a], slot[k].lo[a]); hi[a] = fmaxf(hi[a], slot[k].hi[a]); }
  }
  int e[3];
  bool ok = true;
  for (int a = 0; a < 3; ++a) {
    if (!(lo[a] <= hi[a])) { lo[a] = 0.f; hi[a] = 0.f; }
    ok = axis_grid(lo[a], hi[a], e[a]) && ok;
  }
  uint32_t qlo[3][2] = {{0, 0}, {0, 0}, {0, 0}}, qhi[3][2] = {{0, 0}, {0, 0}, {0, 0}};
  for (int k = 0; k < 8; ++k) {
    if (!used[k]) continue;
    for (int a = 0; a < 3; ++a) {
      const double cell = ldexp(1.0, e[a]);
      double ql = floor(((double)slot[k].lo[a] - (double)lo[a]) / cell);
      double qh = ceil(((double)slot[k].hi[a] - (double)lo[a]) / cell);
      ql = fmin(fmax(ql, 0.0), 255.0);
      qh = fmin(fmax(qh, 0.0), 255.0);
      qlo[a][k >> 2] |= (uint32_t)ql << (8 * (k & 3));
      qhi[a][k >> 2] |= (uint32_t)qh << (8 * (k & 3));
    }
  }
  const uint32_t eb = (uint32_t)(e[0] + 127) | ((uint32_t)(e[1] + 127) << 8) | ((uint32_t)(e[2] + 127) << 16);
  w.h0 = make_float4(lo[0], lo[1], lo[2], __uint_as_float((__float_as_uint(w.h0.w) & 0xff000000u) | eb));
  w.qx = make_uint4(qlo[0][0], qlo[0][1], qhi[0][0], qhi[0][1]);
  w.qy = make_uint4(qlo[1][0], qlo[1][1], qhi[1][0], qhi[1][1]);
  w.qz = make_uint4(qlo[2][0], qlo[2][1], qhi[2][0], qhi[2][1]);
  return ok;
}

// One level of the collapse: 8-wide nodes [lo8, hi8), whose binary roots are
// bin_of[j], get their children; internal children receive new node indices,
// leaf children new positions in tris8.
__global__ void k_collapse8(const Node* __restrict__ bn, const Tri* __restrict__ tris, int* bin_of, uint32_t lo8,
                            uint32_t hi8, Node8* w8, int* src8, Tri* tris8, int* tri8_src, unsigned int* counters,
                            unsigned int* bad) {
  const uint32_t j = lo8 + blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= hi8) return;
  const int b = bin_of[j];
  const Node root = bn[b];
  Cand8 c[8];
  c[0] = cand8_of(root, b, 0);
  c[1] = cand8_of(root, b, 1);
  int n = 2;
  if (root.d.x == root.d.y) n = 1;  // the one-triangle tree: both links name leaf 0
  while (n < 8) {
    int best = -1;
    float ba = -1.f;
    for (int k = 0; k < n; ++k) {
      if (c[k].id >= 0) {
        const float a = half_area8(c[k]);
        if (a > ba) { ba = a; best = k; }
      }
    }
    if (best < 0) break;
    const int id = c[best].id;
    const Node nb = bn[id];
    c[best] = cand8_of(nb, id, 0);
    c[n++] = cand8_of(nb, id, 1);
  }
  // slots by direction from the node's centre (greedy: the best remaining
  // (child, slot) pair first)
  float nlo[3] = {INFINITY, INFINITY, INFINITY}, nhi[3] = {-INFINITY, -INFINITY, -INFINITY};
  for (int k = 0; k < n; ++k)
    for (int a = 0; a < 3; ++a) { nlo[a] = fminf(nlo[a], c[k].lo[a]); nhi[a] = fmaxf(nhi[a], c[k].hi[a]); }
  int slot_of[8];
  bool slot_used[8] = {false, false, false, false, false, false, false, false};
  bool cand_done[8] = {false, false, false, false, false, false, false, false};
  for (int it = 0; it < n; ++it) {
    float best = -INFINITY;
    int bc = -1, bs = -1;
    for (int k = 0; k < n; ++k) {
      if (cand_done[k]) continue;
      float dc[3];
      for (int a = 0; a < 3; ++a) dc[a] = 0.5f * (c[k].lo[a] + c[k].hi[a]) - 0.5f * (nlo[a] + nhi[a]);
      for (int s = 0; s < 8; ++s) {
        if (slot_used[s]) continue;
        const float v = ((s & 1) ? dc[0] : -dc[0]) + ((s & 2) ? dc[1] : -dc[1]) + ((s & 4) ? dc[2] : -dc[2]);
        if (v > best || bc < 0) { best = v; bc = k; bs = s; }
      }
    }
    cand_done[bc] = true;
    slot_used[bs] = true;
    slot_of[bc] = bs;
  }
  Cand8 slot[8];
  for (int k = 0; k < n; ++k) slot[slot_of[k]] = c[k];
  uint32_t imask = 0, valid = 0, ni = 0, nl = 0;
  for (int s = 0; s < 8; ++s) {
    if (!slot_used[s]) continue;
    valid |= 1u << s;
    if (slot[s].id >= 0) { imask |= 1u << s; ++ni; } else { ++nl; }
  }
  const uint32_t child_base = ni ? atomicAdd(&counters[0], ni) : 0u;
  const uint32_t tri_base = nl ? atomicAdd(&counters[1], nl) : 0u;
  uint32_t ri = 0, rl = 0;
  for (int s = 0; s < 8; ++s) {
    if (!slot_used[s]) { src8[8 * j + s] = -1; continue; }
    src8[8 * j + s] = slot[s].src;
    if (slot[s].id >= 0) bin_of[child_base + ri++] = slot[s].id;
    else {
      tri8_src[tri_base + rl] = ~slot[s].id;
      tris8[tri_base + rl++] = tris[~slot[s].id];
    }
  }
  Node8 w;
  w.h0.w = __uint_as_float(imask << 24);
  if (!quantize_node(slot, slot_used, w)) atomicExch(bad, 1u);
  w.h1 = make_uint4(child_base, tri_base, valid, 0u);
  w8[j] = w;
}

// Boxes of every slot from the (refitted) binary records, re-quantized.
__global__ void k_wide8_refit(const Node* __restrict__ bn, const int* __restrict__ src8, uint32_t n8, Node8* w8,
                              unsigned int* status) {
  const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n8) return;
  Node8 w = w8[j];
  Cand8 slot[8];
  bool used[8];
  for (int s = 0; s < 8; ++s) {
    const int r = src8[8 * j + s];
    used[s] = r >= 0;
    if (used[s]) slot[s] = cand8_of(bn[r >> 1], r >> 1, r & 1);
  }
  if (!quantize_node(slot, used, w)) atomicExch(status, (unsigned)RMG_ERR_UNSUPPORTED);
  w8[j] = w;
}

// The triangle copy after a refit moved the packed triangles.
__global__ void k_tris8_refit(const Tri* __restrict__ tris, const int* __restrict__ tri8_src, uint32_t n, Tri* tris8) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) tris8[i] = tris[tri8_src[i]];
}

}  // namespace

void wide8_free(rmg_map* m) {
  cudaFree(m->d_nodes8);
  cudaFree(m->d_src8);
  cudaFree(m->d_tris8);
  cudaFree(m->d_tri8_src);
  m->d_tri8_src = nullptr;
  m->d_nodes8 = nullptr;
  m->d_src8 = nullptr;
  m->d_tris8 = nullptr;
  m->n_nodes8 = 0;
  m->depth8 = 0;
}

// Builds the 8-wide tree of a map whose binary tree is complete.  Synchronises.
// A scene whose boxes cannot be quantized (extents beyond 255 * 2^60) keeps no
// 8-wide tree; its walks use the binary one.
int wide8_build(rmg_map* m, cudaStream_t st) {
  wide8_free(m);
  if (m->n_faces == 0) return RMG_OK;
  const uint32_t cap = std::max<uint32_t>(m->n_nodes, 1u);
  int* bin_of = nullptr;
  unsigned int* counters = nullptr;  // [0] next node, [1] next triangle slot, [2] quantization failure
  int s = dev_alloc(&m->d_nodes8, cap, "8-wide nodes");
  if (s == RMG_OK) s = dev_alloc(&m->d_src8, 8 * (size_t)cap, "8-wide sources");
  if (s == RMG_OK) s = dev_alloc(&m->d_tris8, m->n_faces, "8-wide triangles");
  if (s == RMG_OK) s = dev_alloc(&m->d_tri8_src, m->n_faces, "8-wide triangle sources");
  if (s == RMG_OK) s = dev_alloc(&bin_of, cap, "8-wide roots");
  if (s == RMG_OK) s = dev_alloc(&counters, 3, "8-wide counters");
  const int zero = 0;
  const unsigned int init[3] = {1u, 0u, 0u};
  if (s == RMG_OK) s = cuda_status(cudaMemcpyAsync(bin_of, &zero, 4, cudaMemcpyHostToDevice, st), "8-wide init");
  if (s == RMG_OK) s = cuda_status(cudaMemcpyAsync(counters, init, 12, cudaMemcpyHostToDevice, st), "8-wide init");
  uint32_t lo8 = 0, hi8 = 1, levels = 0;
  unsigned int c[3] = {0, 0, 0};
  while (s == RMG_OK && lo8 < hi8) {
    const uint32_t n = hi8 - lo8;
    k_collapse8<<<(n + kBlock8 - 1) / kBlock8, kBlock8, 0, st>>>(m->d_nodes, m->d_tris, bin_of, lo8, hi8,
                                                                 m->d_nodes8, m->d_src8, m->d_tris8,
                                                                 m->d_tri8_src, counters, counters + 2);
    s = cuda_status(cudaGetLastError(), "k_collapse8");
    if (s == RMG_OK) s = cuda_status(cudaMemcpyAsync(c, counters, 12, cudaMemcpyDeviceToHost, st), "8-wide count");
    if (s == RMG_OK) s = cuda_status(cudaStreamSynchronize(st), "8-wide sync");
    ++levels;
    lo8 = hi8;
    hi8 = c[0];
    if (hi8 > cap) s = fail(RMG_ERR_CUDA, "8-wide build: node count exceeds the binary tree");
  }
  cudaFree(bin_of);
  cudaFree(counters);
  if (s == RMG_OK && c[1] != m->n_faces) s = fail(RMG_ERR_CUDA, "8-wide build: leaf count differs from the faces");
  if (s != RMG_OK || c[2]) {  // c[2]: a box beyond the quantization range -> no 8-wide tree
    wide8_free(m);
    return s;
  }
  m->n_nodes8 = hi8;
  m->depth8 = levels;
  return RMG_OK;
}

// Re-quantizes the 8-wide boxes and refreshes the triangle copy after the
// binary tree was refitted (asynchronous).  A refit that moves a box beyond the quantization range
// records RMG_ERR_UNSUPPORTED in the map's status word.
int wide8_refit(rmg_map* m, cudaStream_t st) {
  if (!m->d_nodes8 || m->n_nodes8 == 0) return RMG_OK;
  k_wide8_refit<<<(m->n_nodes8 + kBlock8 - 1) / kBlock8, kBlock8, 0, st>>>(m->d_nodes, m->d_src8, m->n_nodes8,
                                                                           m->d_nodes8, m->d_status);
  k_tris8_refit<<<(m->n_faces + kBlock8 - 1) / kBlock8, kBlock8, 0, st>>>(m->d_tris, m->d_tri8_src, m->n_faces,
                                                                          m->d_tris8);
  return cuda_status(cudaGetLastError(), "k_wide8_refit");
}

}  // namespace rmg
