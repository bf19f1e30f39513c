// ORACLE -- test infrastructure only.  CPU restatement of rmagine's Embree
// simulation path, used by tests/, __graft_entry__.smoke() and the CPU
// baseline leg of bench.py as the checker.  Nothing in the product links,
// imports or executes this file.
//
// What it restates (uos/rmagine v2.4.2, paths inside that project):
//   * ray generation    src/rmagine_core/include/rmagine/types/sensor_models.h:169-174 (spherical),
//                       :256-276 (pinhole), :375-384 (O1Dn), :460-468 (OnDn)
//   * pose math         src/rmagine_core/include/rmagine/math/types/Transform.tcc:24-42,
//                       Quaternion.tcc:35-75
//   * ray setup         src/rmagine_embree/include/rmagine/simulation/SphereSimulatorEmbree.tcc:69-99,
//                       O1DnSimulatorEmbree.tcc:84-99, OnDnSimulatorEmbree.tcc:86-101
//   * attributes        SphereSimulatorEmbree.tcc:104-249, O1DnSimulatorEmbree.tcc:132
//   * closest hit       rtcIntersect1 (Embree v4.4.0, third party, not vendored): restated as
//                       the watertight binary32 test of Woop, Benthin and Wald (JCGT 2013) over
//                       every triangle, closest t in (0, range.max], ties to the smaller face id.
// The arithmetic is written operation by operation (build with
// -ffp-contract=off; fmaf() only where the published method fuses) so that a
// ray and a triangle test give the same binary32 results on any IEEE host.
//
// Acceleration: a binned-SAH BVH with a conservative binary64 box test, so the
// tree never changes which triangle is found.  The same tree collapsed to a
// 4-wide tree with SIMD box tests (closest_hit4, orc_simulate4) is the timed
// CPU baseline: an Embree-style single-ray walk with the same outputs.  A
// second, canonical LBVH (Morton codes, Karras radix tree) mirrors the GPU
// library's tree for the tree-equality test and for counting node visits and
// triangle tests.
// FP64 re-intersection (Moeller-Trumbore in binary64) certifies rays whose
// results disagree.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <limits>
#include <numeric>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

struct V3 { float x, y, z; };
struct Qt { float x, y, z, w; };
struct Tf { Qt R; V3 t; };

// Quaternion.tcc:35-42, terms summed left to right.
Qt qmul(const Qt& a, const Qt& b) {
  Qt r;
  r.x = a.w * b.x + a.x * b.w + a.y * b.z - a.z * b.y;
  r.y = a.w * b.y - a.x * b.z + a.y * b.w + a.z * b.x;
  r.z = a.w * b.z + a.x * b.y - a.y * b.x + a.z * b.w;
  r.w = a.w * b.w - a.x * b.x - a.y * b.y - a.z * b.z;
  return r;
}
Qt qinv(const Qt& q) { return Qt{-q.x, -q.y, -q.z, q.w}; }
// Quaternion.tcc:68-75: q * (p, 0) * q^-1.
V3 qrot(const Qt& q, const V3& p) {
  const Qt P{p.x, p.y, p.z, 0.0f};
  const Qt r = qmul(qmul(q, P), qinv(q));
  return V3{r.x, r.y, r.z};
}
// Transform.tcc:34-42.
Tf tmul(const Tf& a, const Tf& b) {
  Tf r;
  const V3 rt = qrot(a.R, b.t);
  r.R = qmul(a.R, b.R);
  r.t = V3{rt.x + a.t.x, rt.y + a.t.y, rt.z + a.t.z};
  return r;
}
Tf load_tf(const float* p) { return Tf{Qt{p[0], p[1], p[2], p[3]}, V3{p[4], p[5], p[6]}}; }

// ---------------------------------------------------------------------------
// Watertight binary32 ray/triangle test.
// ---------------------------------------------------------------------------
struct RayW { float ox, oy, oz; int kx, ky, kz; float Sx, Sy, Sz; };

inline float cmp(const V3& v, int k) { return k == 0 ? v.x : (k == 1 ? v.y : v.z); }

RayW make_rayw(const V3& o, const V3& d) {
  RayW r;
  r.ox = o.x; r.oy = o.y; r.oz = o.z;
  const float ax = std::fabs(d.x), ay = std::fabs(d.y), az = std::fabs(d.z);
  int kz = 0;
  if (ay > ax) kz = 1;
  if (az > std::max(ax, ay)) kz = 2;
  int kx = (kz + 1) % 3, ky = (kx + 1) % 3;
  if (cmp(d, kz) < 0.0f) std::swap(kx, ky);
  r.kx = kx; r.ky = ky; r.kz = kz;
  r.Sx = cmp(d, kx) / cmp(d, kz);
  r.Sy = cmp(d, ky) / cmp(d, kz);
  r.Sz = 1.0f / cmp(d, kz);
  return r;
}

bool tri_hit(const RayW& r, const V3& p0, const V3& p1, const V3& p2, float tfar, float& t_out) {
  const V3 A{p0.x - r.ox, p0.y - r.oy, p0.z - r.oz};
  const V3 B{p1.x - r.ox, p1.y - r.oy, p1.z - r.oz};
  const V3 C{p2.x - r.ox, p2.y - r.oy, p2.z - r.oz};
  const float Akz = cmp(A, r.kz), Bkz = cmp(B, r.kz), Ckz = cmp(C, r.kz);
  const float Ax = std::fmaf(-r.Sx, Akz, cmp(A, r.kx));
  const float Ay = std::fmaf(-r.Sy, Akz, cmp(A, r.ky));
  const float Bx = std::fmaf(-r.Sx, Bkz, cmp(B, r.kx));
  const float By = std::fmaf(-r.Sy, Bkz, cmp(B, r.ky));
  const float Cx = std::fmaf(-r.Sx, Ckz, cmp(C, r.kx));
  const float Cy = std::fmaf(-r.Sy, Ckz, cmp(C, r.ky));
  const float CxBy = Cx * By, CyBx = Cy * Bx;
  const float AxCy = Ax * Cy, AyCx = Ay * Cx;
  const float BxAy = Bx * Ay, ByAx = By * Ax;
  float U = CxBy - CyBx, Vv = AxCy - AyCx, W = BxAy - ByAx;
  if (U == 0.0f || Vv == 0.0f || W == 0.0f) {
    U = (float)((double)Cx * (double)By - (double)Cy * (double)Bx);
    Vv = (float)((double)Ax * (double)Cy - (double)Ay * (double)Cx);
    W = (float)((double)Bx * (double)Ay - (double)By * (double)Ax);
  }
  if ((U < 0.0f || Vv < 0.0f || W < 0.0f) && (U > 0.0f || Vv > 0.0f || W > 0.0f)) return false;
  const float det = (U + Vv) + W;
  if (det == 0.0f) return false;
  const float Az = r.Sz * Akz, Bz = r.Sz * Bkz, Cz = r.Sz * Ckz;
  const float T = std::fmaf(U, Az, std::fmaf(Vv, Bz, W * Cz));
  const float t = T / det;
  if (!(t > 0.0f) || !(t <= tfar)) return false;
  t_out = t;
  return true;
}

struct Mesh {
  std::vector<V3> v;       // vertices
  std::vector<uint32_t> f; // 3 per face
  V3 vert(uint32_t face, int k) const { return v[f[3 * face + k]]; }
};

// ---------------------------------------------------------------------------
// Binned-SAH BVH with conservative binary64 box tests.
// ---------------------------------------------------------------------------
struct BoxD { double lo[3], hi[3]; };

struct SahNode {
  BoxD box;
  int left, right;   // children for internal nodes
  int first, count;  // primitive range for leaves (count > 0)
};

struct SahBvh {
  Mesh mesh;
  std::vector<SahNode> nodes;
  std::vector<uint32_t> prims;
  double pad;  // absolute box padding
};

BoxD empty_box() {
  BoxD b;
  for (int k = 0; k < 3; ++k) { b.lo[k] = INFINITY; b.hi[k] = -INFINITY; }
  return b;
}
void grow(BoxD& b, const V3& p) {
  const double c[3] = {p.x, p.y, p.z};
  for (int k = 0; k < 3; ++k) { b.lo[k] = std::min(b.lo[k], c[k]); b.hi[k] = std::max(b.hi[k], c[k]); }
}
void grow(BoxD& b, const BoxD& o) {
  for (int k = 0; k < 3; ++k) { b.lo[k] = std::min(b.lo[k], o.lo[k]); b.hi[k] = std::max(b.hi[k], o.hi[k]); }
}
double area(const BoxD& b) {
  double e[3];
  for (int k = 0; k < 3; ++k) e[k] = std::max(0.0, b.hi[k] - b.lo[k]);
  return 2.0 * (e[0] * e[1] + e[1] * e[2] + e[2] * e[0]);
}

struct BuildCtx {
  const Mesh* mesh;
  std::vector<BoxD> tb;
  std::vector<double> cen;  // 3 per tri
  std::vector<uint32_t>* prims;
  std::vector<SahNode>* nodes;
  int max_leaf = 4;  // triangles per leaf at most
};

int build_sah(BuildCtx& c, int first, int count) {
  const int idx = (int)c.nodes->size();
  c.nodes->push_back(SahNode{});
  BoxD b = empty_box(), cb = empty_box();
  for (int i = first; i < first + count; ++i) {
    const uint32_t p = (*c.prims)[i];
    grow(b, c.tb[p]);
    const double* q = &c.cen[3 * p];
    for (int k = 0; k < 3; ++k) { cb.lo[k] = std::min(cb.lo[k], q[k]); cb.hi[k] = std::max(cb.hi[k], q[k]); }
  }
  (*c.nodes)[idx].box = b;
  if (count <= c.max_leaf) {
    (*c.nodes)[idx].first = first; (*c.nodes)[idx].count = count;
    (*c.nodes)[idx].left = (*c.nodes)[idx].right = -1;
    return idx;
  }
  const int NB = 16;
  double best_cost = INFINITY;
  int best_axis = -1, best_split = -1;
  for (int ax = 0; ax < 3; ++ax) {
    const double ext = cb.hi[ax] - cb.lo[ax];
    if (!(ext > 0.0)) continue;
    BoxD bins[NB];
    int cnt[NB] = {0};
    for (int k = 0; k < NB; ++k) bins[k] = empty_box();
    for (int i = first; i < first + count; ++i) {
      const uint32_t p = (*c.prims)[i];
      int bi = (int)((c.cen[3 * p + ax] - cb.lo[ax]) / ext * NB);
      bi = std::min(std::max(bi, 0), NB - 1);
      cnt[bi]++;
      grow(bins[bi], c.tb[p]);
    }
    double ra[NB];
    int rc[NB];
    BoxD acc = empty_box();
    int n = 0;
    for (int k = NB - 1; k > 0; --k) { grow(acc, bins[k]); n += cnt[k]; ra[k] = area(acc); rc[k] = n; }
    acc = empty_box(); n = 0;
    for (int k = 0; k < NB - 1; ++k) {
      grow(acc, bins[k]); n += cnt[k];
      if (n == 0 || rc[k + 1] == 0) continue;
      const double cost = area(acc) * n + ra[k + 1] * rc[k + 1];
      if (cost < best_cost) { best_cost = cost; best_axis = ax; best_split = k; }
    }
  }
  int mid;
  if (best_axis < 0) {
    mid = first + count / 2;
  } else {
    const double ext = cb.hi[best_axis] - cb.lo[best_axis];
    auto it = std::partition(c.prims->begin() + first, c.prims->begin() + first + count, [&](uint32_t p) {
      int bi = (int)((c.cen[3 * p + best_axis] - cb.lo[best_axis]) / ext * NB);
      bi = std::min(std::max(bi, 0), NB - 1);
      return bi <= best_split;
    });
    mid = (int)(it - c.prims->begin());
    if (mid == first || mid == first + count) mid = first + count / 2;
  }
  const int l = build_sah(c, first, mid - first);
  const int r = build_sah(c, mid, first + count - mid);
  (*c.nodes)[idx].left = l; (*c.nodes)[idx].right = r;
  (*c.nodes)[idx].count = 0;
  return idx;
}

struct RayD { double o[3], inv[3]; };

bool box_hit(const RayD& r, const BoxD& b, double pad, double tfar, double& tmin_out) {
  double tmin = 0.0, tmax = tfar;
  for (int k = 0; k < 3; ++k) {
    double t0 = (b.lo[k] - pad - r.o[k]) * r.inv[k];
    double t1 = (b.hi[k] + pad - r.o[k]) * r.inv[k];
    if (std::isnan(t0) || std::isnan(t1)) { t0 = -INFINITY; t1 = INFINITY; }
    if (t0 > t1) std::swap(t0, t1);
    tmin = std::max(tmin, t0);
    tmax = std::min(tmax, t1);
  }
  tmin_out = tmin;
  return tmin <= tmax * (1.0 + 1e-9) + 1e-12;
}

struct HitF { float t; uint32_t face; bool hit; };

// Nearest child first with t-culling, like the GPU walk; `node_visits` (when
// non-NULL) counts the internal nodes whose two child boxes were tested.
HitF closest_hit(const SahBvh& bvh, const V3& o, const V3& d, float tfar, uint64_t* tri_tests,
                 uint64_t* node_visits = nullptr) {
  HitF h{tfar, 0xffffffffu, false};
  if (bvh.nodes.empty()) return h;
  const RayW rw = make_rayw(o, d);
  RayD rd;
  const double dd[3] = {d.x, d.y, d.z}, oo[3] = {o.x, o.y, o.z};
  for (int k = 0; k < 3; ++k) { rd.o[k] = oo[k]; rd.inv[k] = 1.0 / dd[k]; }
  int stack[128];
  int sp = 0;
  stack[sp++] = 0;
  while (sp) {
    const SahNode& n = bvh.nodes[stack[--sp]];
    double tmin;
    if (!box_hit(rd, n.box, bvh.pad, (double)h.t, tmin)) continue;
    if (n.count > 0) {
      for (int i = n.first; i < n.first + n.count; ++i) {
        const uint32_t f = bvh.prims[i];
        float t;
        if (tri_hit(rw, bvh.mesh.vert(f, 0), bvh.mesh.vert(f, 1), bvh.mesh.vert(f, 2), h.t, t)) {
          if (t < h.t || f < h.face) { h.t = t; h.face = f; h.hit = true; }
        }
        if (tri_tests) ++*tri_tests;
      }
    } else {
      if (node_visits) ++*node_visits;
      double tl, tr;
      const bool hl = box_hit(rd, bvh.nodes[n.left].box, bvh.pad, (double)h.t, tl);
      const bool hr = box_hit(rd, bvh.nodes[n.right].box, bvh.pad, (double)h.t, tr);
      if (hl && hr) {
        if (tl <= tr) { stack[sp++] = n.right; stack[sp++] = n.left; }
        else { stack[sp++] = n.left; stack[sp++] = n.right; }
      } else if (hl) stack[sp++] = n.left;
      else if (hr) stack[sp++] = n.right;
    }
  }
  return h;
}

// ---------------------------------------------------------------------------
// Embree-class CPU walk: the timed CPU baseline.
//
// The restatement above tests every box twice and in binary64, one ray at a
// time: a correctness yardstick, several times slower than a production CPU
// tracer.  This walk is built the way Embree's single-ray kernels are (Wald,
// Woop, Benthin, Johnson, Ernst, "Embree: A Kernel Framework for Efficient CPU
// Ray Tracing", SIGGRAPH 2014): the binary SAH tree above collapsed into a
// 4-wide tree with the four child boxes of a node stored plane by plane, one
// 4-lane SIMD slab test per node (GCC vector extensions: SSE on x86, NEON on
// Arm), near and far planes picked once per ray from the signs of its
// direction, hit children visited nearest first from a stack of (node, entry
// distance), leaves of up to four triangles.  Triangles go through the same
// watertight tri_hit and the same tie rule (smaller face at equal t), so
// every output equals the restatement's bit for bit (tested).
//
// Boxes: each child box is the binary node's box widened by the tree's
// absolute padding and rounded outward to binary32.  A plane distance
// (c - o) * (1/d) carries at most 3 ulp of relative error (one rounding each
// for c - o, 1/d and the product), so comparing entry <= exit * (1 + 2^-20)
// never rejects a box that the ray meets in [0, t_best].  A direction
// component of magnitude <= 1e-20 is replaced by +-1e20 in 1/d: such a ray
// moves less than 1e-17 along that axis over any sensor range, far inside the
// padding (>= 1e-6), so a box whose unpadded slab holds the origin still
// spans every t of interest on that axis, and a box whose unpadded slab does
// not hold it contains no triangle the ray can meet.
// ---------------------------------------------------------------------------
typedef float f4 __attribute__((vector_size(16)));
typedef int32_t i4 __attribute__((vector_size(16)));

inline f4 splat4(float x) { return f4{x, x, x, x}; }
inline f4 vmin4(f4 a, f4 b) { return a < b ? a : b; }
inline f4 vmax4(f4 a, f4 b) { return a > b ? a : b; }

struct alignas(64) Node4 {
  f4 b[6];          // lo_x, hi_x, lo_y, hi_y, lo_z, hi_z of the four child slots
  i4 ref;           // internal child: node index (>= 0); leaf: ~(first triangle << 4 | count); unused: 0
  uint32_t leaves;  // bit k: slot k is a leaf
};

struct TriF {
  V3 p0, p1, p2;
  uint32_t face;
};

struct Bvh4 {
  const SahBvh* src = nullptr;
  std::vector<Node4> nodes;
  std::vector<TriF> tris;
  int32_t root = 0;  // a node index, or a leaf reference when the whole tree is one leaf
  int depth = 0;
};

constexpr int kStack4Entries = 256;

float round_down(double x) {
  float f = (float)x;
  return (double)f > x ? std::nextafter(f, -INFINITY) : f;
}
float round_up(double x) {
  float f = (float)x;
  return (double)f < x ? std::nextafter(f, INFINITY) : f;
}

int32_t leaf_ref(Bvh4& B, const SahNode& n) {
  const int32_t first = (int32_t)B.tris.size();
  for (int i = n.first; i < n.first + n.count; ++i) {
    const uint32_t f = B.src->prims[i];
    B.tris.push_back(TriF{B.src->mesh.vert(f, 0), B.src->mesh.vert(f, 1), B.src->mesh.vert(f, 2), f});
  }
  return ~(first << 4 | n.count);
}

// Collapses the binary subtree under internal node `bin` into node4 slots:
// the internal slot of largest surface area is opened until four slots.
int collapse4(Bvh4& B, int bin, int depth) {
  const SahBvh& S = *B.src;
  std::vector<int> slot = {S.nodes[bin].left, S.nodes[bin].right};
  while (slot.size() < 4) {
    int best = -1;
    double best_area = -1.0;
    for (size_t k = 0; k < slot.size(); ++k) {
      const SahNode& n = S.nodes[slot[k]];
      if (n.count == 0 && area(n.box) > best_area) { best_area = area(n.box); best = (int)k; }
    }
    if (best < 0) break;
    const SahNode& n = S.nodes[slot[best]];
    slot[best] = n.left;
    slot.push_back(n.right);
  }
  const int idx = (int)B.nodes.size();
  B.nodes.push_back(Node4{});
  B.depth = std::max(B.depth, depth);
  Node4 nd;
  float lo[3][4], hi[3][4];
  nd.leaves = 0;
  for (int k = 0; k < 4; ++k) {  // unused slots: an inverted box, never entered
    nd.ref[k] = 0;
    for (int a = 0; a < 3; ++a) { lo[a][k] = INFINITY; hi[a][k] = -INFINITY; }
  }
  for (size_t k = 0; k < slot.size(); ++k) {
    const SahNode& n = S.nodes[slot[k]];
    for (int a = 0; a < 3; ++a) {
      lo[a][k] = round_down(n.box.lo[a] - S.pad);
      hi[a][k] = round_up(n.box.hi[a] + S.pad);
    }
    nd.ref[k] = n.count > 0 ? leaf_ref(B, n) : collapse4(B, slot[k], depth + 1);
    if (n.count > 0) nd.leaves |= 1u << k;
  }
  for (int a = 0; a < 3; ++a) {
    nd.b[2 * a] = f4{lo[a][0], lo[a][1], lo[a][2], lo[a][3]};
    nd.b[2 * a + 1] = f4{hi[a][0], hi[a][1], hi[a][2], hi[a][3]};
  }
  B.nodes[idx] = nd;
  return idx;
}

Bvh4* build_bvh4(const SahBvh& S) {
  Bvh4* B = new Bvh4;
  B->src = &S;
  if (S.nodes.empty()) return B;
  for (const SahNode& n : S.nodes)  // a leaf reference holds 4 bits of count and 27 of its first triangle
    if (n.count > 15 || S.prims.size() >= (1u << 27)) { delete B; return nullptr; }
  if (S.nodes[0].count > 0) {  // the whole tree is one leaf (its box is not tested, as in the binary walk)
    B->root = leaf_ref(*B, S.nodes[0]);
    return B;
  }
  B->nodes.reserve(S.nodes.size() / 2 + 1);
  B->root = collapse4(*B, 0, 1);
  if (3 * B->depth + 1 > kStack4Entries) { delete B; return nullptr; }  // a stack entry per pending child
  return B;
}

inline void leaf_hits(const Bvh4& B, const RayW& rw, int32_t ref, HitF& h) {
  const int32_t code = ~ref;
  const int first = code >> 4, count = code & 15;
  for (int i = first; i < first + count; ++i) {
    const TriF& tr = B.tris[i];
    float t;
    if (tri_hit(rw, tr.p0, tr.p1, tr.p2, h.t, t) && (t < h.t || tr.face < h.face)) {
      h.t = t; h.face = tr.face; h.hit = true;
    }
  }
}

HitF closest_hit4(const Bvh4& B, const V3& o, const V3& d, float tfar) {
  HitF h{tfar, 0xffffffffu, false};
  if (B.nodes.empty() && B.tris.empty()) return h;
  const RayW rw = make_rayw(o, d);
  if (B.root < 0) {
    leaf_hits(B, rw, B.root, h);
    return h;
  }
  const float dd[3] = {d.x, d.y, d.z};
  float inv[3];
  int neg[3];
  for (int a = 0; a < 3; ++a) {
    inv[a] = std::fabs(dd[a]) > 1e-20f ? 1.0f / dd[a] : std::copysign(1e20f, dd[a]);
    neg[a] = std::signbit(inv[a]) ? 1 : 0;
  }
  const f4 ox = splat4(o.x), oy = splat4(o.y), oz = splat4(o.z);
  const f4 ix = splat4(inv[0]), iy = splat4(inv[1]), iz = splat4(inv[2]);
  const int nx = neg[0], ny = 2 + neg[1], nz = 4 + neg[2];
  const int fx = 1 - neg[0], fy = 3 - neg[1], fz = 5 - neg[2];
  const f4 zero = splat4(0.0f);
  const i4 lane_bit = i4{1, 2, 4, 8};
  const float kW = 1.00000095f;  // 1 + 2^-20
  int32_t st_ref[kStack4Entries];
  float st_t[kStack4Entries];
  int sp = 0;
  int32_t node = B.root;
  for (;;) {
    const Node4& n = B.nodes[node];
    const f4 tn = vmax4(vmax4((n.b[nx] - ox) * ix, (n.b[ny] - oy) * iy), vmax4((n.b[nz] - oz) * iz, zero));
    const f4 tf = vmin4(vmin4((n.b[fx] - ox) * ix, (n.b[fy] - oy) * iy), vmin4((n.b[fz] - oz) * iz, splat4(h.t)));
    i4 bits = (tn <= tf * splat4(kW)) & lane_bit;  // the entered slots as four bits
    bits |= __builtin_shuffle(bits, i4{2, 3, 0, 1});
    bits |= __builtin_shuffle(bits, i4{1, 0, 3, 2});
    const unsigned m = (unsigned)bits[0];
    const unsigned leaves = m & n.leaves;
    unsigned inner = m & ~leaves;
    if (leaves) {  // leaf children are tested on the spot; the closest hit may move: re-cull the others
      for (unsigned l = leaves; l; l &= l - 1) leaf_hits(B, rw, n.ref[__builtin_ctz(l)], h);
      for (unsigned r = inner; r; r &= r - 1) {
        const int k = __builtin_ctz(r);
        if (!(tn[k] <= h.t * kW)) inner &= ~(1u << k);
      }
    }
    if (inner) {
      const int k0 = __builtin_ctz(inner);
      inner &= inner - 1;
      if (inner == 0) { node = n.ref[k0]; continue; }
      const int k1 = __builtin_ctz(inner);
      inner &= inner - 1;
      if (inner == 0) {
        const bool first = tn[k0] <= tn[k1];
        const int kn = first ? k0 : k1, kf = first ? k1 : k0;
        st_ref[sp] = n.ref[kf];
        st_t[sp] = tn[kf];
        ++sp;
        node = n.ref[kn];
        continue;
      }
      int ck[4] = {k0, k1, 0, 0};
      int nc = 2;
      while (inner) { ck[nc++] = __builtin_ctz(inner); inner &= inner - 1; }
      for (int a = 1; a < nc; ++a)  // nearest first
        for (int b = a; b > 0 && tn[ck[b]] < tn[ck[b - 1]]; --b) std::swap(ck[b], ck[b - 1]);
      for (int k = nc - 1; k >= 1; --k) { st_ref[sp] = n.ref[ck[k]]; st_t[sp] = tn[ck[k]]; ++sp; }
      node = n.ref[ck[0]];
      continue;
    }
    for (;;) {
      if (sp == 0) return h;
      --sp;
      if (st_t[sp] <= h.t * kW) break;
    }
    node = st_ref[sp];
  }
}

// ---------------------------------------------------------------------------
// Canonical LBVH (same construction as the GPU library's map builder).
// ---------------------------------------------------------------------------
struct LNode { float a[4], b[4], c[4]; int32_t d[4]; };  // 64 B, same field meaning

struct Lbvh {
  std::vector<LNode> nodes;
  std::vector<float> tris;        // 12 floats per leaf
  std::vector<uint32_t> order;    // face id per leaf
  std::vector<int> leaf_parent;
};

uint64_t spread3(uint64_t x) {
  x &= 0x1fffffull;
  x = (x | (x << 32)) & 0x001f00000000ffffull;
  x = (x | (x << 16)) & 0x001f0000ff0000ffull;
  x = (x | (x << 8)) & 0x100f00f00f00f00full;
  x = (x | (x << 4)) & 0x10c30c30c30c30c3ull;
  x = (x | (x << 2)) & 0x1249249249249249ull;
  return x;
}

int clz64(uint64_t x) { return x ? __builtin_clzll(x) : 64; }
int clz32(uint32_t x) { return x ? __builtin_clz(x) : 32; }

int ldelta(const std::vector<uint64_t>& k, int n, int i, int j) {
  if (j < 0 || j >= n) return -1;
  if (k[i] == k[j]) return 64 + clz32((uint32_t)(i ^ j));
  return clz64(k[i] ^ k[j]);
}

void lbvh_build(const Mesh& m, Lbvh& L) {
  const int n = (int)(m.f.size() / 3);
  L.nodes.clear(); L.tris.clear(); L.order.clear(); L.leaf_parent.clear();
  if (n == 0) return;
  std::vector<V3> cen(n);
  float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
  const float third = 0.333333343f;
  for (int i = 0; i < n; ++i) {
    const V3 a = m.vert(i, 0), b = m.vert(i, 1), c = m.vert(i, 2);
    cen[i] = V3{((a.x + b.x) + c.x) * third, ((a.y + b.y) + c.y) * third, ((a.z + b.z) + c.z) * third};
    const float q[3] = {cen[i].x, cen[i].y, cen[i].z};
    for (int k = 0; k < 3; ++k) { lo[k] = std::min(lo[k], q[k]); hi[k] = std::max(hi[k], q[k]); }
  }
  // one scale for all axes: the centroids' bounding cube
  const float ext = std::max(std::max(hi[0] - lo[0], hi[1] - lo[1]), hi[2] - lo[2]);
  const float s1 = ext > 0.0f ? 2097152.0f / ext : 0.0f;
  const float scale[3] = {s1, s1, s1};
  std::vector<uint64_t> key(n);
  for (int i = 0; i < n; ++i) {
    const float q[3] = {cen[i].x, cen[i].y, cen[i].z};
    uint64_t qq[3];
    for (int k = 0; k < 3; ++k) {
      float v = (q[k] - lo[k]) * scale[k];
      v = std::min(std::max(v, 0.0f), 2097151.0f);
      qq[k] = (uint64_t)(uint32_t)v;
    }
    key[i] = (spread3(qq[0]) << 2) | (spread3(qq[1]) << 1) | spread3(qq[2]);
  }
  std::vector<uint32_t> idx(n);
  std::iota(idx.begin(), idx.end(), 0u);
  std::stable_sort(idx.begin(), idx.end(), [&](uint32_t a, uint32_t b) { return key[a] < key[b]; });
  std::vector<uint64_t> sk(n);
  for (int i = 0; i < n; ++i) sk[i] = key[idx[i]];
  L.order = idx;
  L.tris.resize(12 * (size_t)n);
  for (int k = 0; k < n; ++k) {
    const uint32_t f = idx[k];
    for (int j = 0; j < 3; ++j) {
      const V3 p = m.vert(f, j);
      L.tris[12 * k + 4 * j + 0] = p.x; L.tris[12 * k + 4 * j + 1] = p.y; L.tris[12 * k + 4 * j + 2] = p.z;
      float w = 0.0f;
      if (j == 0) std::memcpy(&w, &f, 4);
      L.tris[12 * k + 4 * j + 3] = w;
    }
  }
  L.leaf_parent.assign(n, -1);
  if (n == 1) {
    LNode nd;
    const float* t = &L.tris[0];
    const float far = 1e30f;
    const float lx = std::min(std::min(t[0], t[4]), t[8]), hx = std::max(std::max(t[0], t[4]), t[8]);
    const float ly = std::min(std::min(t[1], t[5]), t[9]), hy = std::max(std::max(t[1], t[5]), t[9]);
    const float lz = std::min(std::min(t[2], t[6]), t[10]), hz = std::max(std::max(t[2], t[6]), t[10]);
    const float a[4] = {lx, hx, ly, hy}, b[4] = {far, far, far, far}, c[4] = {lz, hz, far, far};
    std::memcpy(nd.a, a, 16); std::memcpy(nd.b, b, 16); std::memcpy(nd.c, c, 16);
    nd.d[0] = -1; nd.d[1] = -1; nd.d[2] = -1; nd.d[3] = 0;
    L.nodes.assign(1, nd);
    return;
  }
  L.nodes.assign(n - 1, LNode{});
  L.nodes[0].d[2] = -1;
  for (int i = 0; i < n - 1; ++i) {
    const int d = (ldelta(sk, n, i, i + 1) - ldelta(sk, n, i, i - 1)) >= 0 ? 1 : -1;
    const int dmin = ldelta(sk, n, i, i - d);
    int lmax = 2;
    while (ldelta(sk, n, i, i + lmax * d) > dmin) lmax <<= 1;
    int l = 0;
    for (int t = lmax >> 1; t >= 1; t >>= 1)
      if (ldelta(sk, n, i, i + (l + t) * d) > dmin) l += t;
    const int j = i + l * d;
    const int dnode = ldelta(sk, n, i, j);
    int s = 0;
    for (int div = 2;; div <<= 1) {
      const int t = (l + div - 1) / div;
      if (ldelta(sk, n, i, i + (s + t) * d) > dnode) s += t;
      if (t <= 1) break;
    }
    const int gamma = i + s * d + std::min(d, 0);
    const int first = std::min(i, j), last = std::max(i, j);
    int left, right;
    if (first == gamma) { left = ~gamma; L.leaf_parent[gamma] = i; }
    else { left = gamma; L.nodes[gamma].d[2] = i; }
    if (last == gamma + 1) { right = ~(gamma + 1); L.leaf_parent[gamma + 1] = i; }
    else { right = gamma + 1; L.nodes[gamma + 1].d[2] = i; }
    L.nodes[i].d[0] = left; L.nodes[i].d[1] = right; L.nodes[i].d[3] = dnode;
  }
  // boxes: post-order (children have larger or smaller indices; recurse iteratively)
  struct FB { float lo[3], hi[3]; };
  std::vector<FB> nb(n - 1);
  std::vector<char> done(n - 1, 0);
  auto tri_box = [&](int k) {
    FB b;
    const float* t = &L.tris[12 * (size_t)k];
    for (int a = 0; a < 3; ++a) {
      b.lo[a] = std::min(std::min(t[a], t[4 + a]), t[8 + a]);
      b.hi[a] = std::max(std::max(t[a], t[4 + a]), t[8 + a]);
    }
    return b;
  };
  std::vector<int> st;
  st.push_back(0);
  while (!st.empty()) {
    const int i = st.back();
    const int l = L.nodes[i].d[0], r = L.nodes[i].d[1];
    bool ready = true;
    if (l >= 0 && !done[l]) { st.push_back(l); ready = false; }
    if (r >= 0 && !done[r]) { st.push_back(r); ready = false; }
    if (!ready) continue;
    st.pop_back();
    const FB bl = l < 0 ? tri_box(~l) : nb[l];
    const FB br = r < 0 ? tri_box(~r) : nb[r];
    LNode& nd = L.nodes[i];
    nd.a[0] = bl.lo[0]; nd.a[1] = bl.hi[0]; nd.a[2] = bl.lo[1]; nd.a[3] = bl.hi[1];
    nd.b[0] = br.lo[0]; nd.b[1] = br.hi[0]; nd.b[2] = br.lo[1]; nd.b[3] = br.hi[1];
    nd.c[0] = bl.lo[2]; nd.c[1] = bl.hi[2]; nd.c[2] = br.lo[2]; nd.c[3] = br.hi[2];
    for (int a = 0; a < 3; ++a) {
      nb[i].lo[a] = std::min(bl.lo[a], br.lo[a]);
      nb[i].hi[a] = std::max(bl.hi[a], br.hi[a]);
    }
    done[i] = 1;
  }
}

// The GPU traversal order on the canonical LBVH (binary32 slab tests in the
// same form), instrumented: counts internal-node visits and triangle tests.
const float kWiden = 1.00000024f;

// cl / ch: the lo / hi plane addends, -o/d widened outward by |o/d| 2^-21.
void slab(const float inv[3], const float cl[3], const float ch[3], const float lo[3], const float hi[3], float& tmin,
          float& tmax) {
  float t0[3], t1[3];
  for (int k = 0; k < 3; ++k) {
    t0[k] = std::fmaf(lo[k], inv[k], cl[k]);
    t1[k] = std::fmaf(hi[k], inv[k], ch[k]);
  }
  tmin = std::max(std::max(std::min(t0[0], t1[0]), std::min(t0[1], t1[1])), std::max(std::min(t0[2], t1[2]), 0.0f));
  tmax = std::min(std::min(std::max(t0[0], t1[0]), std::max(t0[1], t1[1])), std::max(t0[2], t1[2]));
}

HitF lbvh_trace(const Lbvh& L, const V3& o, const V3& d, float tfar, uint64_t& visits, uint64_t& tests) {
  HitF h{tfar, 0xffffffffu, false};
  if (L.nodes.empty()) return h;
  const RayW rw = make_rayw(o, d);
  const float dd[3] = {d.x, d.y, d.z}, oo[3] = {o.x, o.y, o.z};
  float inv[3], cl[3], ch[3];
  for (int k = 0; k < 3; ++k) {
    inv[k] = std::fabs(dd[k]) > 1e-20f ? 1.0f / dd[k] : std::copysign(1e20f, dd[k]);
    const float oi = oo[k] * inv[k];
    const float e = std::copysign(std::fabs(oi) * 4.76837158e-7f, inv[k]);
    cl[k] = -oi - e;
    ch[k] = -oi + e;
  }
  auto test = [&](int k) {
    const float* t = &L.tris[12 * (size_t)k];
    float tt;
    ++tests;
    if (tri_hit(rw, V3{t[0], t[1], t[2]}, V3{t[4], t[5], t[6]}, V3{t[8], t[9], t[10]}, h.t, tt)) {
      uint32_t f;
      std::memcpy(&f, &t[3], 4);
      if (tt < h.t || f < h.face) { h.t = tt; h.face = f; h.hit = true; }
    }
  };
  std::vector<std::pair<int, float>> stack;
  int node = 0;
  for (;;) {
    ++visits;
    const LNode& n = L.nodes[node];
    const float llo[3] = {n.a[0], n.a[2], n.c[0]}, lhi[3] = {n.a[1], n.a[3], n.c[1]};
    const float rlo[3] = {n.b[0], n.b[2], n.c[2]}, rhi[3] = {n.b[1], n.b[3], n.c[3]};
    float tl, tL, tr, tR;
    slab(inv, cl, ch, llo, lhi, tl, tL);
    slab(inv, cl, ch, rlo, rhi, tr, tR);
    bool hl = tl <= std::min(tL, h.t) * kWiden;
    bool hr = tr <= std::min(tR, h.t) * kWiden;
    if (hl && n.d[0] < 0) { test(~n.d[0]); hl = false; }
    if (hr && n.d[1] < 0) { test(~n.d[1]); hr = false; }
    hl = hl && tl <= h.t * kWiden;
    hr = hr && tr <= h.t * kWiden;
    if (hl && hr) {
      const bool lf = tl <= tr;
      stack.push_back({lf ? n.d[1] : n.d[0], lf ? tr : tl});
      node = lf ? n.d[0] : n.d[1];
      continue;
    }
    if (hl || hr) { node = hl ? n.d[0] : n.d[1]; continue; }
    bool found = false;
    while (!stack.empty()) {
      const auto e = stack.back();
      stack.pop_back();
      if (e.second <= h.t * kWiden) { node = e.first; found = true; break; }
    }
    if (!found) break;
  }
  return h;
}

// ---------------------------------------------------------------------------
// Sensor-model rays.
// ---------------------------------------------------------------------------
struct Model {
  int kind;
  uint32_t W, H;
  float rmin, rmax;
  const float* dirs;   // W*H*3 sensor-frame directions
  const float* origs;  // OnDn: W*H*3
  V3 orig;             // O1Dn
};

void make_ray(const Model& m, const Tf& Tsm, uint32_t loc, V3& dir_s, V3& orig_s, V3& o, V3& d) {
  dir_s = V3{m.dirs[3 * loc], m.dirs[3 * loc + 1], m.dirs[3 * loc + 2]};
  d = qrot(Tsm.R, dir_s);
  if (m.kind == 0 || m.kind == 1) {
    orig_s = V3{0.0f, 0.0f, 0.0f};
    o = Tsm.t;
  } else {
    orig_s = m.kind == 2 ? m.orig : V3{m.origs[3 * loc], m.origs[3 * loc + 1], m.origs[3 * loc + 2]};
    const V3 r = qrot(Tsm.R, orig_s);  // Transform::mult(Vector3): R*v + t
    o = V3{r.x + Tsm.t.x, r.y + Tsm.t.y, r.z + Tsm.t.z};
  }
}

int nthreads_or_default(int n) {
#ifdef _OPENMP
  return n > 0 ? n : omp_get_max_threads();
#else
  (void)n;
  return 1;
#endif
}

}  // namespace

extern "C" {

int orc_max_threads(void) { return nthreads_or_default(0); }

// SphericalModel::getDirection: phi/theta from DiscreteInterval::getValue in
// binary32, then the C library's cosf/sinf as in sensor_models.h:169-174.
void orc_dirs_spherical(float phi_min, float phi_inc, uint32_t phi_size, float theta_min, float theta_inc,
                        uint32_t theta_size, float* out) {
  for (uint32_t v = 0; v < phi_size; ++v) {
    const float phi = phi_min + (float)v * phi_inc;
    const float cp = cosf(phi), sp = sinf(phi);
    for (uint32_t h = 0; h < theta_size; ++h) {
      const float th = theta_min + (float)h * theta_inc;
      const float ct = cosf(th), st = sinf(th);
      float* o = out + 3 * ((size_t)v * theta_size + h);
      o[0] = cp * ct; o[1] = cp * st; o[2] = sp;
    }
  }
}

// PinholeModel::getDirection.
void orc_dirs_pinhole(uint32_t W, uint32_t H, float fx, float fy, float cx, float cy, float* out) {
  for (uint32_t v = 0; v < H; ++v) {
    for (uint32_t h = 0; h < W; ++h) {
      const float px = ((float)h - cx) / fx, py = ((float)v - cy) / fy, pz = 1.0f;
      const float n = std::sqrt((px * px + py * py) + pz * pz);
      const float x = px / n, y = py / n, z = pz / n;
      float* o = out + 3 * ((size_t)v * W + h);
      o[0] = z; o[1] = -x; o[2] = -y;
    }
  }
}

void* orc_bvh_build_ex(const float* verts, uint32_t nv, const uint32_t* faces, uint32_t nf, int max_leaf);

void* orc_bvh_build(const float* verts, uint32_t nv, const uint32_t* faces, uint32_t nf) {
  return orc_bvh_build_ex(verts, nv, faces, nf, 4);
}

// Binned-SAH tree with at most max_leaf (>= 1) triangles per leaf.
void* orc_bvh_build_ex(const float* verts, uint32_t nv, const uint32_t* faces, uint32_t nf, int max_leaf) {
  SahBvh* b = new SahBvh;
  b->mesh.v.resize(nv);
  for (uint32_t i = 0; i < nv; ++i) b->mesh.v[i] = V3{verts[3 * i], verts[3 * i + 1], verts[3 * i + 2]};
  b->mesh.f.assign(faces, faces + 3 * (size_t)nf);
  b->prims.resize(nf);
  std::iota(b->prims.begin(), b->prims.end(), 0u);
  double maxabs = 1.0;
  for (const V3& p : b->mesh.v) maxabs = std::max({maxabs, (double)std::fabs(p.x), (double)std::fabs(p.y), (double)std::fabs(p.z)});
  b->pad = maxabs * 1e-6;
  if (nf == 0) return b;
  BuildCtx c;
  c.mesh = &b->mesh;
  c.tb.resize(nf);
  c.cen.resize(3 * (size_t)nf);
  for (uint32_t i = 0; i < nf; ++i) {
    BoxD bb = empty_box();
    for (int k = 0; k < 3; ++k) grow(bb, b->mesh.vert(i, k));
    c.tb[i] = bb;
    for (int k = 0; k < 3; ++k) c.cen[3 * i + k] = 0.5 * (bb.lo[k] + bb.hi[k]);
  }
  c.prims = &b->prims;
  c.nodes = &b->nodes;
  c.max_leaf = std::max(1, max_leaf);
  b->nodes.reserve(2 * (size_t)nf);
  build_sah(c, 0, (int)nf);
  return b;
}

void orc_bvh_free(void* p) { delete static_cast<SahBvh*>(p); }

// Simulate n_poses x H x W rays with Embree-path semantics.  kind: 0 spherical,
// 1 pinhole, 2 O1Dn, 3 OnDn.  dirs (and origs for OnDn) are the model's
// sensor-frame tables; Tsb is one 8-float transform record, Tbm n_poses of them.
// Any output pointer may be NULL.  Counts triangle tests when `tri_tests` != NULL.
}  // extern "C"

namespace {

// The per-ray body of orc_simulate / orc_simulate4 around the closest-hit query
// hit(o, d, tfar, &tests).
template <class HitFn>
int simulate_impl(const Mesh& mesh, HitFn&& hit, int kind, uint32_t W, uint32_t H, float rmin, float rmax,
                  const float* dirs, const float* origs, const float* orig, const float* Tsb, const float* Tbm,
                  uint32_t n_poses, uint8_t* hits, float* ranges, float* points, float* normals, uint32_t* face_ids,
                  uint32_t* geom_ids, uint32_t* object_ids, int nthreads, uint64_t* tri_tests) {
  Model m{kind, W, H, rmin, rmax, dirs, origs, orig ? V3{orig[0], orig[1], orig[2]} : V3{0, 0, 0}};
  const Tf tsb = load_tf(Tsb);
  const int64_t total = (int64_t)n_poses * W * H;
  const float nanf_ = std::numeric_limits<float>::quiet_NaN();
  uint64_t tests_total = 0;
  std::vector<Tf> tsm(n_poses);  // sensor -> map, once per pose as in the reference's pose loop
  for (uint32_t i = 0; i < n_poses; ++i) tsm[i] = tmul(load_tf(Tbm + 8 * (size_t)i), tsb);
#pragma omp parallel for schedule(dynamic, 1024) num_threads(nthreads_or_default(nthreads)) reduction(+ : tests_total)
  for (int64_t gid = 0; gid < total; ++gid) {
    const uint32_t pid = (uint32_t)(gid / ((int64_t)W * H));
    const uint32_t loc = (uint32_t)(gid - (int64_t)pid * W * H);
    const Tf& Tsm = tsm[pid];
    V3 dir_s, orig_s, o, d;
    make_ray(m, Tsm, loc, dir_s, orig_s, o, d);
    uint64_t tt = 0;
    const HitF h = hit(o, d, rmax, tri_tests ? &tt : nullptr);
    tests_total += tt;
    if (h.hit) {
      const float t = h.t;
      if (hits) hits[gid] = t >= rmin ? 1 : 0;
      if (ranges) ranges[gid] = t;
      if (points) {
        float p[3] = {dir_s.x * t, dir_s.y * t, dir_s.z * t};
        if (kind >= 2) { p[0] = p[0] + orig_s.x; p[1] = p[1] + orig_s.y; p[2] = p[2] + orig_s.z; }
        std::memcpy(points + 3 * gid, p, 12);
      }
      if (normals) {
        const V3 p0 = mesh.vert(h.face, 0), p1 = mesh.vert(h.face, 1), p2 = mesh.vert(h.face, 2);
        const V3 e1{p1.x - p0.x, p1.y - p0.y, p1.z - p0.z}, e2{p2.x - p0.x, p2.y - p0.y, p2.z - p0.z};
        V3 n{e1.y * e2.z - e1.z * e2.y, e1.z * e2.x - e1.x * e2.z, e1.x * e2.y - e1.y * e2.x};
        float len = std::sqrt((n.x * n.x + n.y * n.y) + n.z * n.z);
        n = V3{n.x / len, n.y / len, n.z / len};
        n = qrot(qinv(Tsm.R), n);
        const float dp = (dir_s.x * n.x + dir_s.y * n.y) + dir_s.z * n.z;
        if (dp > 0.0f) n = V3{-n.x, -n.y, -n.z};
        len = std::sqrt((n.x * n.x + n.y * n.y) + n.z * n.z);
        const float q[3] = {n.x / len, n.y / len, n.z / len};
        std::memcpy(normals + 3 * gid, q, 12);
      }
      if (face_ids) face_ids[gid] = h.face;
      if (geom_ids) geom_ids[gid] = 0;
      if (object_ids) object_ids[gid] = 0;
    } else {
      if (hits) hits[gid] = 0;
      if (ranges) ranges[gid] = rmax + 1.0f;
      if (points) { points[3 * gid] = nanf_; points[3 * gid + 1] = nanf_; points[3 * gid + 2] = nanf_; }
      if (normals) { normals[3 * gid] = nanf_; normals[3 * gid + 1] = nanf_; normals[3 * gid + 2] = nanf_; }
      if (face_ids) face_ids[gid] = 0xffffffffu;
      if (geom_ids) geom_ids[gid] = 0xffffffffu;
      if (object_ids) object_ids[gid] = 0xffffffffu;
    }
  }
  if (tri_tests) *tri_tests = tests_total;
  return 0;
}

}  // namespace

extern "C" {

int orc_simulate(void* bvhp, int kind, uint32_t W, uint32_t H, float rmin, float rmax, const float* dirs,
                 const float* origs, const float* orig, const float* Tsb, const float* Tbm, uint32_t n_poses,
                 uint8_t* hits, float* ranges, float* points, float* normals, uint32_t* face_ids,
                 uint32_t* geom_ids, uint32_t* object_ids, int nthreads, uint64_t* tri_tests) {
  const SahBvh& bvh = *static_cast<SahBvh*>(bvhp);
  return simulate_impl(
      bvh.mesh, [&](const V3& o, const V3& d, float tfar, uint64_t* tests) { return closest_hit(bvh, o, d, tfar, tests); },
      kind, W, H, rmin, rmax, dirs, origs, orig, Tsb, Tbm, n_poses, hits, ranges, points, normals, face_ids, geom_ids,
      object_ids, nthreads, tri_tests);
}

// The Embree-class 4-wide walk over a binned-SAH tree of orc_bvh_build*; NULL
// when the tree is deeper than the walk's stack allows.  The SAH tree must
// outlive it.
void* orc_bvh4_build(void* bvhp) { return build_bvh4(*static_cast<SahBvh*>(bvhp)); }

void orc_bvh4_free(void* p) { delete static_cast<Bvh4*>(p); }

// orc_simulate through the 4-wide walk (the same outputs; no triangle counts).
int orc_simulate4(void* bvh4, int kind, uint32_t W, uint32_t H, float rmin, float rmax, const float* dirs,
                  const float* origs, const float* orig, const float* Tsb, const float* Tbm, uint32_t n_poses,
                  uint8_t* hits, float* ranges, float* points, float* normals, uint32_t* face_ids,
                  uint32_t* geom_ids, uint32_t* object_ids, int nthreads) {
  const Bvh4& B = *static_cast<Bvh4*>(bvh4);
  return simulate_impl(
      B.src->mesh, [&](const V3& o, const V3& d, float tfar, uint64_t*) { return closest_hit4(B, o, d, tfar); },
      kind, W, H, rmin, rmax, dirs, origs, orig, Tsb, Tbm, n_poses, hits, ranges, points, normals, face_ids, geom_ids,
      object_ids, nthreads, nullptr);
}

// Rays of the same workload (origins and map-frame directions), for
// re-intersection by the certifier.  out_o / out_d: 3 floats per requested ray.
int orc_rays(int kind, uint32_t W, uint32_t H, const float* dirs, const float* origs, const float* orig,
             const float* Tsb, const float* Tbm, const uint64_t* gids, uint64_t n, float* out_o, float* out_d) {
  Model m{kind, W, H, 0, 0, dirs, origs, orig ? V3{orig[0], orig[1], orig[2]} : V3{0, 0, 0}};
  const Tf tsb = load_tf(Tsb);
  for (uint64_t i = 0; i < n; ++i) {
    const uint64_t gid = gids[i];
    const uint32_t pid = (uint32_t)(gid / ((uint64_t)W * H));
    const uint32_t loc = (uint32_t)(gid - (uint64_t)pid * W * H);
    const Tf Tsm = tmul(load_tf(Tbm + 8 * (size_t)pid), tsb);
    V3 dir_s, orig_s, o, d;
    make_ray(m, Tsm, loc, dir_s, orig_s, o, d);
    out_o[3 * i] = o.x; out_o[3 * i + 1] = o.y; out_o[3 * i + 2] = o.z;
    out_d[3 * i] = d.x; out_d[3 * i + 1] = d.y; out_d[3 * i + 2] = d.z;
  }
  return 0;
}

// Batched correspondence statistics (statistics.cpp:19-126) on all host
// threads, the CPU baseline of the statistics kernels: B batches of N
// correspondences, filters in binary32 exactly as oracle/stats.py's
// correspondences() (dmask / mmask > 0; point-to-point: |M - D|^2 < md^2;
// point-to-plane when normals are given: |(M - D).n| < md, M := D + n sd), then
// binary64 means and covariance in two passes.  out: 16 doubles per batch --
// dataset mean, model mean, covariance row-major (row = model axis), count.
int orc_stats_batched(const float* D, const float* M, const float* Nrm, const uint8_t* dmask, const uint8_t* mmask,
                      uint32_t B, uint32_t N, float max_dist, int nthreads, double* out) {
  const float md = max_dist, md2 = md * md;
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads_or_default(nthreads))
  for (int64_t b = 0; b < (int64_t)B; ++b) {
    const size_t base = (size_t)b * N;
    double sd[3] = {0, 0, 0}, sm[3] = {0, 0, 0}, n = 0;
    auto pair = [&](size_t i, float* dd, float* mm) -> bool {
      if (dmask && !(dmask[base + i] > 0)) return false;
      if (mmask && !(mmask[base + i] > 0)) return false;
      const float* d = D + 3 * (base + i);
      const float* m = M + 3 * (base + i);
      const float dx = m[0] - d[0], dy = m[1] - d[1], dz = m[2] - d[2];
      if (Nrm) {
        const float* nn = Nrm + 3 * (base + i);
        const float s = (dx * nn[0] + dy * nn[1]) + dz * nn[2];
        if (!(std::fabs(s) < md)) return false;
        for (int k = 0; k < 3; ++k) { dd[k] = d[k]; mm[k] = d[k] + nn[k] * s; }
      } else {
        const float d2 = (dx * dx + dy * dy) + dz * dz;
        if (!(d2 < md2)) return false;
        for (int k = 0; k < 3; ++k) { dd[k] = d[k]; mm[k] = m[k]; }
      }
      return true;
    };
    float dd[3], mm[3];
    for (uint32_t i = 0; i < N; ++i) {
      if (!pair(i, dd, mm)) continue;
      for (int k = 0; k < 3; ++k) { sd[k] += dd[k]; sm[k] += mm[k]; }
      n += 1.0;
    }
    double* o = out + 16 * (size_t)b;
    for (int k = 0; k < 16; ++k) o[k] = 0.0;
    if (n == 0.0) continue;
    double dm[3], mmean[3], C[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    for (int k = 0; k < 3; ++k) { dm[k] = sd[k] / n; mmean[k] = sm[k] / n; }
    for (uint32_t i = 0; i < N; ++i) {
      if (!pair(i, dd, mm)) continue;
      const double dc[3] = {dd[0] - dm[0], dd[1] - dm[1], dd[2] - dm[2]};
      const double mc[3] = {mm[0] - mmean[0], mm[1] - mmean[1], mm[2] - mmean[2]};
      for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) C[3 * r + c] += mc[r] * dc[c];
    }
    for (int k = 0; k < 3; ++k) { o[k] = dm[k]; o[3 + k] = mmean[k]; }
    for (int k = 0; k < 9; ++k) o[6 + k] = C[k] / n;
    o[15] = n;
  }
  return 0;
}

// The range adjoint's analytic gradient on all host threads, the CPU baseline
// of the pose-gradient kernel: the restatement of oracle/grad.py's
// RayFaceSet.analytic in binary64 for every ray of n_poses x (W x H) whose
// simulated hit (face, range) and observation are valid (face set, range >=
// rmin, rmin <= r_obs <= rmax).  Per ray: r = n.(p0 - o)/(n.d) for the pose's
// ray, psi = clamp(r - r_obs, -delta, delta), dr/drho = -n_b/(n_b.d_b), dr/domega
// = -(p_b x n_b)/(n_b.d_b); grad (6 per pose) sums psi dr/dxi, loss the Huber terms.
int orc_pose_grad(void* bvhp, int kind, uint32_t W, uint32_t H, float rmin, float rmax, const float* dirs,
                  const float* origs, const float* orig, const float* Tsb, const float* Tbm, uint32_t n_poses,
                  const uint32_t* face_ids, const float* ranges, const float* r_obs, double delta, int nthreads,
                  double* grad, double* loss) {
  const Mesh& mesh = static_cast<SahBvh*>(bvhp)->mesh;
  auto rot = [](const float* q, double R[9]) {
    const double x = q[0], y = q[1], z = q[2], w = q[3];
    const double v[9] = {1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w),
                         2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w),
                         2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)};
    for (int k = 0; k < 9; ++k) R[k] = v[k];
  };
  double Rsb[9];
  rot(Tsb, Rsb);
  const size_t WH = (size_t)W * H;
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads_or_default(nthreads))
  for (int64_t p = 0; p < (int64_t)n_poses; ++p) {
    double Rbm[9];
    rot(Tbm + 8 * (size_t)p, Rbm);
    const double tbm[3] = {Tbm[8 * p + 4], Tbm[8 * p + 5], Tbm[8 * p + 6]};
    double g[6] = {0, 0, 0, 0, 0, 0}, L = 0.0;
    for (size_t loc = 0; loc < WH; ++loc) {
      const size_t gid = (size_t)p * WH + loc;
      const uint32_t f = face_ids[gid];
      const double obs = r_obs[gid];
      if (f == 0xffffffffu || !(ranges[gid] >= rmin) || !(obs >= rmin) || !(obs <= rmax)) continue;
      const double ds[3] = {dirs[3 * loc], dirs[3 * loc + 1], dirs[3 * loc + 2]};
      double os[3] = {0, 0, 0};
      if (kind == 2) { os[0] = orig[0]; os[1] = orig[1]; os[2] = orig[2]; }
      if (kind == 3) { os[0] = origs[3 * loc]; os[1] = origs[3 * loc + 1]; os[2] = origs[3 * loc + 2]; }
      double db[3], ob[3];
      for (int r = 0; r < 3; ++r) {
        db[r] = Rsb[3 * r] * ds[0] + Rsb[3 * r + 1] * ds[1] + Rsb[3 * r + 2] * ds[2];
        ob[r] = Tsb[4 + r] + (Rsb[3 * r] * os[0] + Rsb[3 * r + 1] * os[1] + Rsb[3 * r + 2] * os[2]);
      }
      double o[3], d[3];
      for (int r = 0; r < 3; ++r) {
        o[r] = Rbm[3 * r] * ob[0] + Rbm[3 * r + 1] * ob[1] + Rbm[3 * r + 2] * ob[2] + tbm[r];
        d[r] = Rbm[3 * r] * db[0] + Rbm[3 * r + 1] * db[1] + Rbm[3 * r + 2] * db[2];
      }
      const V3 a = mesh.vert(f, 0), b1 = mesh.vert(f, 1), c = mesh.vert(f, 2);
      const double p0[3] = {a.x, a.y, a.z};
      const double e1[3] = {b1.x - p0[0], b1.y - p0[1], b1.z - p0[2]};
      const double e2[3] = {c.x - p0[0], c.y - p0[1], c.z - p0[2]};
      const double n[3] = {e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2], e1[0] * e2[1] - e1[1] * e2[0]};
      const double r = (n[0] * (p0[0] - o[0]) + n[1] * (p0[1] - o[1]) + n[2] * (p0[2] - o[2])) /
                       (n[0] * d[0] + n[1] * d[1] + n[2] * d[2]);
      const double e = r - obs;
      const double psi = std::min(std::max(e, -delta), delta);
      double nb[3];
      for (int k = 0; k < 3; ++k) nb[k] = Rbm[k] * n[0] + Rbm[3 + k] * n[1] + Rbm[6 + k] * n[2];  // R_bm^T n
      const double bb = nb[0] * db[0] + nb[1] * db[1] + nb[2] * db[2];
      const double pb[3] = {ob[0] + r * db[0], ob[1] + r * db[1], ob[2] + r * db[2]};
      const double cx[3] = {pb[1] * nb[2] - pb[2] * nb[1], pb[2] * nb[0] - pb[0] * nb[2], pb[0] * nb[1] - pb[1] * nb[0]};
      for (int k = 0; k < 3; ++k) { g[k] += -nb[k] / bb * psi; g[3 + k] += -cx[k] / bb * psi; }
      const double ae = std::fabs(e);
      L += ae <= delta ? 0.5 * e * e : delta * (ae - 0.5 * delta);
    }
    for (int k = 0; k < 6; ++k) grad[6 * p + k] = g[k];
    loss[p] = L;
  }
  return 0;
}

}  // extern "C"

// Range noise on all host threads, the CPU baseline of rmg_noise_apply: the
// restatement of oracle/noise.py's apply() in C++ -- Philox4x32-10 (Salmon,
// Moraes, Dror, Shaw, SC 2011; counter (i, call), key = seed), uniforms as odd
// multiples of 2^-24, Box-Muller in binary64 -- for kind 0 (Gaussian), 1
// (range-relative Gaussian) and 2 (uniform dust).  out: n binary64 ranges.
namespace {
struct Philox4 { uint32_t v[4]; };
Philox4 philox4x32_10(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3, uint32_t k0, uint32_t k1) {
  uint32_t c[4] = {c0, c1, c2, c3};
  for (int r = 0; r < 10; ++r) {
    if (r > 0) { k0 += 0x9E3779B9u; k1 += 0xBB67AE85u; }
    const uint64_t p0 = (uint64_t)0xD2511F53u * c[0], p1 = (uint64_t)0xCD9E8D57u * c[2];
    const uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0, hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
    const uint32_t n0 = hi1 ^ c[1] ^ k0, n2 = hi0 ^ c[3] ^ k1;
    c[0] = n0; c[1] = lo1; c[2] = n2; c[3] = lo0;
  }
  return Philox4{{c[0], c[1], c[2], c[3]}};
}
inline double uniform01(uint32_t x) { return (double)((x >> 8) | 1u) * 0x1p-24; }
}  // namespace

extern "C" int orc_noise_apply(int kind, const float* ranges, double* out, uint64_t n, uint64_t seed, uint64_t call,
                               double mean, double stddev, double range_exp, double hit_p, double ret_p,
                               double max_range, int nthreads) {
  const uint32_t k0 = (uint32_t)seed, k1 = (uint32_t)(seed >> 32), c2 = (uint32_t)call, c3 = (uint32_t)(call >> 32);
  const double two_pi = 2.0 * M_PI;
  if (kind == 0 || kind == 1) {
    const int64_t nb = (int64_t)((n + 3) / 4);
#pragma omp parallel for schedule(static, 4096) num_threads(nthreads_or_default(nthreads))
    for (int64_t i = 0; i < nb; ++i) {
      const Philox4 b = philox4x32_10((uint32_t)i, (uint32_t)((uint64_t)i >> 32), c2, c3, k0, k1);
      double u[4];
      for (int k = 0; k < 4; ++k) u[k] = uniform01(b.v[k]);
      const double r0 = std::sqrt(-2.0 * std::log(u[0])), r1 = std::sqrt(-2.0 * std::log(u[2]));
      const double z[4] = {r0 * std::cos(two_pi * u[1]), r0 * std::sin(two_pi * u[1]),
                           r1 * std::cos(two_pi * u[3]), r1 * std::sin(two_pi * u[3])};
      for (int k = 0; k < 4; ++k) {
        const uint64_t e = 4 * (uint64_t)i + k;
        if (e >= n) break;
        const double r = ranges[e];
        const double sd = kind == 0 ? stddev : stddev * std::pow(std::max(r, 0.0), range_exp);
        out[e] = r <= max_range ? r + (z[k] * sd + mean) : r;
      }
    }
    return 0;
  }
  if (kind != 2) return 1;
#pragma omp parallel for schedule(static, 4096) num_threads(nthreads_or_default(nthreads))
  for (int64_t i = 0; i < (int64_t)n; ++i) {
    const Philox4 b = philox4x32_10((uint32_t)i, (uint32_t)((uint64_t)i >> 32), c2, c3, k0, k1);
    const double u0 = uniform01(b.v[0]), u1 = uniform01(b.v[1]), u2 = uniform01(b.v[2]);
    const double r = ranges[i];
    const double rr = std::min(r, max_range);
    const double p_hit = 1.0 - std::pow(1.0 - hit_p, rr);
    const double nr = (double)((float)u1 * (float)rr);
    const double p_ret = std::pow(ret_p, nr);
    out[i] = (u0 < p_hit && u2 < p_ret) ? nr : r;
  }
  return 0;
}

extern "C" {

// Binary64 Moeller-Trumbore of one ray against one face.  Writes t and the
// smallest barycentric coordinate (negative = outside).  Returns 1 when the
// plane is hit in front of the origin (t > 0), -1 for a face index outside the
// mesh.
int orc_intersect_f64(void* bvhp, const float* o, const float* d, uint32_t face, double* t_out,
                      double* minbary_out) {
  const SahBvh& bvh = *static_cast<SahBvh*>(bvhp);
  if ((size_t)face >= bvh.mesh.f.size() / 3) { *t_out = INFINITY; *minbary_out = -INFINITY; return -1; }
  const V3 a = bvh.mesh.vert(face, 0), b = bvh.mesh.vert(face, 1), c = bvh.mesh.vert(face, 2);
  const double p0[3] = {a.x, a.y, a.z}, p1[3] = {b.x, b.y, b.z}, p2[3] = {c.x, c.y, c.z};
  const double O[3] = {o[0], o[1], o[2]}, D[3] = {d[0], d[1], d[2]};
  double e1[3], e2[3], s[3];
  for (int k = 0; k < 3; ++k) { e1[k] = p1[k] - p0[k]; e2[k] = p2[k] - p0[k]; s[k] = O[k] - p0[k]; }
  const double pv[3] = {D[1] * e2[2] - D[2] * e2[1], D[2] * e2[0] - D[0] * e2[2], D[0] * e2[1] - D[1] * e2[0]};
  const double det = e1[0] * pv[0] + e1[1] * pv[1] + e1[2] * pv[2];
  if (det == 0.0) { *t_out = INFINITY; *minbary_out = -INFINITY; return 0; }
  const double u = (s[0] * pv[0] + s[1] * pv[1] + s[2] * pv[2]) / det;
  const double qv[3] = {s[1] * e1[2] - s[2] * e1[1], s[2] * e1[0] - s[0] * e1[2], s[0] * e1[1] - s[1] * e1[0]};
  const double v = (D[0] * qv[0] + D[1] * qv[1] + D[2] * qv[2]) / det;
  const double t = (e2[0] * qv[0] + e2[1] * qv[1] + e2[2] * qv[2]) / det;
  *t_out = t;
  *minbary_out = std::min(std::min(u, v), 1.0 - u - v);
  return t > 0.0 ? 1 : 0;
}

// Closest binary32 hit of explicit rays (origins/directions), any tree.
int orc_trace_rays(void* bvhp, const float* o, const float* d, uint64_t n, float tfar, float* t_out,
                   uint32_t* face_out, int nthreads) {
  const SahBvh& bvh = *static_cast<SahBvh*>(bvhp);
#pragma omp parallel for schedule(dynamic, 256) num_threads(nthreads_or_default(nthreads))
  for (int64_t i = 0; i < (int64_t)n; ++i) {
    const HitF h = closest_hit(bvh, V3{o[3 * i], o[3 * i + 1], o[3 * i + 2]},
                               V3{d[3 * i], d[3 * i + 1], d[3 * i + 2]}, tfar, nullptr);
    t_out[i] = h.hit ? h.t : INFINITY;
    face_out[i] = h.face;
  }
  return 0;
}

// ---- canonical LBVH ----------------------------------------------------------
void* orc_lbvh_build(const float* verts, uint32_t nv, const uint32_t* faces, uint32_t nf) {
  Mesh m;
  m.v.resize(nv);
  for (uint32_t i = 0; i < nv; ++i) m.v[i] = V3{verts[3 * i], verts[3 * i + 1], verts[3 * i + 2]};
  m.f.assign(faces, faces + 3 * (size_t)nf);
  Lbvh* L = new Lbvh;
  lbvh_build(m, *L);
  return L;
}

void orc_lbvh_free(void* p) { delete static_cast<Lbvh*>(p); }

uint32_t orc_lbvh_num_nodes(void* p) { return (uint32_t)static_cast<Lbvh*>(p)->nodes.size(); }

// nodes: n_nodes * 16 words (64-byte records), tris: n_faces * 12 floats, order: n_faces.
void orc_lbvh_export(void* p, void* nodes, float* tris, uint32_t* order) {
  const Lbvh& L = *static_cast<Lbvh*>(p);
  if (nodes && !L.nodes.empty()) std::memcpy(nodes, L.nodes.data(), L.nodes.size() * sizeof(LNode));
  if (tris && !L.tris.empty()) std::memcpy(tris, L.tris.data(), L.tris.size() * 4);
  if (order && !L.order.empty()) std::memcpy(order, L.order.data(), L.order.size() * 4);
}

// Traverses explicit rays through the canonical LBVH in the GPU kernel's
// order and returns per-ray node visits and triangle tests plus the hit.
int orc_lbvh_count(void* p, const float* o, const float* d, uint64_t n, float tfar, uint32_t* visits,
                   uint32_t* tests, float* t_out, uint32_t* face_out, int nthreads) {
  const Lbvh& L = *static_cast<Lbvh*>(p);
#pragma omp parallel for schedule(dynamic, 256) num_threads(nthreads_or_default(nthreads))
  for (int64_t i = 0; i < (int64_t)n; ++i) {
    uint64_t v = 0, t = 0;
    const HitF h = lbvh_trace(L, V3{o[3 * i], o[3 * i + 1], o[3 * i + 2]}, V3{d[3 * i], d[3 * i + 1], d[3 * i + 2]},
                              tfar, v, t);
    visits[i] = (uint32_t)v;
    tests[i] = (uint32_t)t;
    if (t_out) t_out[i] = h.hit ? h.t : INFINITY;
    if (face_out) face_out[i] = h.face;
  }
  return 0;
}

// Node visits, triangle tests and hits of explicit rays through any tree in
// the GPU library's layout (nodes: n_faces - 1 records of 16 words, tris:
// n_faces records of 12 floats, as rmg_map_export writes them), walked like
// orc_lbvh_count walks the canonical LBVH.
int orc_tree_count(const void* nodes, const float* tris, uint32_t n_faces, const float* o, const float* d, uint64_t n,
                   float tfar, uint32_t* visits, uint32_t* tests, float* t_out, uint32_t* face_out, int nthreads) {
  Lbvh L;
  if (n_faces >= 2) {
    L.nodes.resize(n_faces - 1);
    std::memcpy(L.nodes.data(), nodes, sizeof(LNode) * L.nodes.size());
    L.tris.assign(tris, tris + 12 * (size_t)n_faces);
  }
#pragma omp parallel for schedule(dynamic, 256) num_threads(nthreads_or_default(nthreads))
  for (int64_t i = 0; i < (int64_t)n; ++i) {
    uint64_t v = 0, t = 0;
    const HitF h = lbvh_trace(L, V3{o[3 * i], o[3 * i + 1], o[3 * i + 2]}, V3{d[3 * i], d[3 * i + 1], d[3 * i + 2]},
                              tfar, v, t);
    visits[i] = (uint32_t)v;
    tests[i] = (uint32_t)t;
    if (t_out) t_out[i] = h.hit ? h.t : INFINITY;
    if (face_out) face_out[i] = h.face;
  }
  return 0;
}

// SAH-tree node count (the tree-quality yardstick).
uint32_t orc_bvh_num_nodes(void* p) { return (uint32_t)static_cast<SahBvh*>(p)->nodes.size(); }

// Writes a one-triangle-per-leaf SAH tree (max_leaf 1) as a GPU map file
// (the RMGLBVH1 layout of rmg_map_save: 48-byte header, then vertices, faces,
// 64-byte nodes, 48-byte packed triangles, leaf order, leaf parents, with an
// FNV-1a 64 checksum of the payload).  Internal nodes are numbered in depth-
// first preorder from the root (0), leaf k holds prims[k]; child boxes are the
// exact binary32 bounds of their triangles.  Returns the tree depth (edges to
// the deepest leaf), or -1 when the tree has a leaf of more than one triangle
// or the file cannot be written.  Used by tests to load a second topology of
// the same mesh into the GPU library.
int orc_bvh_save_map(void* p, const char* path) {
  const SahBvh& b = *static_cast<SahBvh*>(p);
  const uint32_t nv = (uint32_t)b.mesh.v.size(), nf = (uint32_t)(b.mesh.f.size() / 3);
  if (nf < 2) return -1;
  for (const SahNode& n : b.nodes)
    if (n.count > 1) return -1;
  struct FBox { float lo[3], hi[3]; };
  const uint32_t nn = nf - 1;
  std::vector<int32_t> id(b.nodes.size(), 0);  // SAH node -> internal id, or ~leaf
  {
    int32_t next = 0;
    std::vector<int> st{0};
    while (!st.empty()) {
      const int k = st.back();
      st.pop_back();
      const SahNode& n = b.nodes[k];
      if (n.count == 1) { id[k] = ~n.first; continue; }
      id[k] = next++;
      st.push_back(n.right);
      st.push_back(n.left);
    }
  }
  std::vector<uint32_t> words(16 * (size_t)nn, 0);
  std::vector<float> tris(12 * (size_t)nf);
  std::vector<uint32_t> order(nf);
  std::vector<int32_t> leaf_parent(nf, -1);
  std::vector<FBox> box(b.nodes.size());
  int depth = 0;
  // post-order: boxes bottom-up; pre-order ids already assigned
  std::vector<std::pair<int, int>> st{{0, 0}};
  std::vector<int> post;
  std::vector<int> level(b.nodes.size(), 0);
  while (!st.empty()) {
    const auto [k, lv] = st.back();
    st.pop_back();
    level[k] = lv;
    post.push_back(k);
    const SahNode& n = b.nodes[k];
    if (n.count == 1) { depth = std::max(depth, lv); continue; }
    st.push_back({n.left, lv + 1});
    st.push_back({n.right, lv + 1});
  }
  for (auto it = post.rbegin(); it != post.rend(); ++it) {
    const int k = *it;
    const SahNode& n = b.nodes[k];
    FBox fb;
    if (n.count == 1) {
      const uint32_t f = b.prims[n.first];
      for (int a = 0; a < 3; ++a) { fb.lo[a] = INFINITY; fb.hi[a] = -INFINITY; }
      for (int v = 0; v < 3; ++v) {
        const V3 q = b.mesh.vert(f, v);
        const float c[3] = {q.x, q.y, q.z};
        for (int a = 0; a < 3; ++a) { fb.lo[a] = std::min(fb.lo[a], c[a]); fb.hi[a] = std::max(fb.hi[a], c[a]); }
        tris[12 * (size_t)n.first + 4 * v + 0] = q.x;
        tris[12 * (size_t)n.first + 4 * v + 1] = q.y;
        tris[12 * (size_t)n.first + 4 * v + 2] = q.z;
        tris[12 * (size_t)n.first + 4 * v + 3] = 0.0f;
      }
      std::memcpy(&tris[12 * (size_t)n.first + 3], &f, 4);
      order[n.first] = f;
    } else {
      const FBox& L = box[n.left];
      const FBox& R = box[n.right];
      for (int a = 0; a < 3; ++a) { fb.lo[a] = std::min(L.lo[a], R.lo[a]); fb.hi[a] = std::max(L.hi[a], R.hi[a]); }
      uint32_t* w = &words[16 * (size_t)id[k]];
      const float fa[12] = {L.lo[0], L.hi[0], L.lo[1], L.hi[1], R.lo[0], R.hi[0], R.lo[1], R.hi[1],
                            L.lo[2], L.hi[2], R.lo[2], R.hi[2]};
      std::memcpy(w, fa, 48);
      const int32_t links[4] = {id[n.left], id[n.right], -1, 0};
      std::memcpy(w + 12, links, 16);
      for (int c : {n.left, n.right}) {
        if (id[c] >= 0) std::memcpy(&words[16 * (size_t)id[c] + 14], &id[k], 4);
        else leaf_parent[~id[c]] = id[k];
      }
    }
    box[k] = fb;
  }
  std::vector<unsigned char> payload;
  auto put = [&](const void* src, size_t bytes) {
    const unsigned char* q = static_cast<const unsigned char*>(src);
    payload.insert(payload.end(), q, q + bytes);
  };
  for (const V3& v : b.mesh.v) { const float q[3] = {v.x, v.y, v.z}; put(q, 12); }
  put(b.mesh.f.data(), 4 * b.mesh.f.size());
  put(words.data(), 4 * words.size());
  put(tris.data(), 4 * tris.size());
  put(order.data(), 4 * order.size());
  put(leaf_parent.data(), 4 * leaf_parent.size());
  uint64_t h = 1469598103934665603ull;
  for (unsigned char c : payload) { h ^= c; h *= 1099511628211ull; }
  unsigned char hdr[48] = {'R', 'M', 'G', 'L', 'B', 'V', 'H', '1'};
  const uint32_t hw[6] = {1u, nv, nf, nn, (uint32_t)depth, 0u};
  std::memcpy(hdr + 8, hw, 24);
  const uint64_t tail[2] = {(uint64_t)payload.size(), h};
  std::memcpy(hdr + 32, tail, 16);
  FILE* fp = std::fopen(path, "wb");
  if (!fp) return -1;
  bool ok = std::fwrite(hdr, 48, 1, fp) == 1 && std::fwrite(payload.data(), 1, payload.size(), fp) == payload.size();
  ok = (std::fclose(fp) == 0) && ok;
  return ok ? depth : -1;
}

// Per-ray internal-node visits and triangle tests of explicit rays through the
// SAH tree (the tree-quality yardstick beside orc_lbvh_count), plus the hit.
int orc_bvh_count(void* p, const float* o, const float* d, uint64_t n, float tfar, uint32_t* visits,
                  uint32_t* tests, float* t_out, uint32_t* face_out, int nthreads) {
  const SahBvh& bvh = *static_cast<SahBvh*>(p);
#pragma omp parallel for schedule(dynamic, 256) num_threads(nthreads_or_default(nthreads))
  for (int64_t i = 0; i < (int64_t)n; ++i) {
    uint64_t v = 0, t = 0;
    const HitF h = closest_hit(bvh, V3{o[3 * i], o[3 * i + 1], o[3 * i + 2]}, V3{d[3 * i], d[3 * i + 1], d[3 * i + 2]},
                               tfar, &t, &v);
    visits[i] = (uint32_t)v;
    tests[i] = (uint32_t)t;
    if (t_out) t_out[i] = h.hit ? h.t : INFINITY;
    if (face_out) face_out[i] = h.face;
  }
  return 0;
}

}  // extern "C"
