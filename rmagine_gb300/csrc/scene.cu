// Scenes: instances of several meshes under a top-level LBVH (two-level BVH).
//
// Replaces the instance hierarchy of rmagine's Embree / OptiX maps
// (EmbreeScene.cpp:246-406, EmbreeInstance.cpp:33-60, OptixScene.cpp:396-481)
// for the simulators.  Bottom level: each geometry is an ordinary rmg_map (its
// LBVH and packed triangles), shared by every instance that places it.  Top
// level: an LBVH over the instances' map-frame boxes, built by the same device
// builder as a mesh -- instance i is handed to it as the degenerate triangle
// (lo_i, hi_i, centre_i), whose bounds are exactly the box and whose centroid
// is the box centre -- so rmg_map_refit of that tree is the dynamic-scene
// update.  Leaf k of the top tree is the k-th live instance (face id k).
//
// Partial re-braiding (Benthin, Woop, Wald, Afra, "Improved Two-Level BVHs
// using Partial Re-Braiding", HPG 2017): the tree of a large geometry (at
// least 2 x RMG_SCENE_PIECE_TRIS triangles) is opened at scene creation into
// pieces -- subtrees of about RMG_SCENE_PIECE_TRIS triangles, found by opening
// the piece with the largest box first -- and every instance of it enters the
// top tree once per piece, with that piece's box in the map frame.  A top-level
// leaf is then (instance, start node): a ray enters only the pieces of a big
// mesh that lie along it, and the top tree sorts them among the small
// instances as a single tree of the baked geometry would.  Every triangle lies
// under exactly one piece and the ray transform does not depend on the piece,
// so the hits and the result are those of the unopened tree.
//
// Identity instances (rotation (0,0,0,1), no translation, unit scale) leave the
// top tree: the geometry of the first such instance of each geometry (up to
// kMaxDirect geometries) is walked by every ray directly, in the map frame,
// before the top tree, which then holds only the other instances and starts
// with the closest hit found so far as its far limit.  Identity instances
// after the first of the same geometry are dropped: their hits coincide with
// the first's in range and face and lose the tie to its smaller index.
//
// Traversal (k_trace_scene): the top tree is walked with a full stack; at an
// instance leaf the ray is taken into the instance's mesh frame,
//     o_l = s^-1 (.) R^T (o - t),   d_l = s^-1 (.) R^T d   (R^T as conj(q) sandwich),
// which keeps the ray parameter t, and the geometry's tree is walked by the
// plain kernel's RayTrav from the leaf's start node with tfar = the best range
// so far.  A hit replaces the best when its range is smaller, or equal with a
// smaller instance index, or equal in both with a smaller face index (two
// pieces of one instance), so the result is the lexicographic minimum
// (t, instance, face) over all hits, independent of the visiting order.  Both trees must be at most 32 levels deep
// (checked at creation; the stack guards turn a corrupt tree into
// RMG_ERR_TRAVERSAL_BUDGET in the scene's status word).
#include <cmath>
#include <cstring>
#include <vector>

#include "internal.h"
#include "trace.cuh"

struct rmg_scene;

namespace rmg {
namespace {

struct InstDev {
  float4 qinv;   // conj(q): map -> mesh rotation
  float4 t;      // translation (w unused)
  float4 inv_s;  // 1 / scale per axis (w unused)
  float4 q;      // mesh -> map rotation (normals)
  uint4 ids;     // geometry, geom_id, object_id, instance index
};

struct GeomDev {
  const Node* nodes;
  const Tri* tris;
  int root;
  unsigned budget;
};

constexpr uint32_t kMaxDirect = 4;

struct SceneParams {
  TraceParams T;  // T.map: the top-level tree, status = the scene's word
  const InstDev* inst;
  const GeomDev* geoms;
  const uint2* leaves;  // top-level leaf -> (instance record, start node in its geometry's tree)
  uint2 direct[kMaxDirect];  // (geometry, instance record) walked in the map frame before the top tree
  uint32_t n_direct;
};

struct Best {
  float t;
  int tri;        // packed triangle index in the hit geometry, -1 = none
  uint32_t face;
  int inst;       // live-instance slot
  uint32_t order; // instance index (tie-break)
};

__device__ __forceinline__ void instance_hit(const SceneParams& S, int k, const V& o, const V& d, Best& best,
                                             bool& over) {
  const uint2 leaf = __ldg(&S.leaves[__float_as_uint(__ldg(&S.T.map.tris[k].v0.w))]);
  const uint32_t slot = leaf.x;
  const InstDev* ip = S.inst + slot;
  const float4 qi = __ldg(&ip->qinv), tt = __ldg(&ip->t), is = __ldg(&ip->inv_s);
  const uint4 ids = __ldg(&ip->ids);
  const Q qinv{qi.x, qi.y, qi.z, qi.w};
  const V rl = qrot(qinv, V{sub(o.x, tt.x), sub(o.y, tt.y), sub(o.z, tt.z)});
  const V ol{mul(rl.x, is.x), mul(rl.y, is.y), mul(rl.z, is.z)};
  const V rd = qrot(qinv, d);
  const V dl{mul(rd.x, is.x), mul(rd.y, is.y), mul(rd.z, is.z)};
  const GeomDev* gp = S.geoms + ids.x;
  DeviceMap bm;
  bm.nodes = reinterpret_cast<const Node*>(__ldg(reinterpret_cast<const unsigned long long*>(&gp->nodes)));
  bm.tris = reinterpret_cast<const Tri*>(__ldg(reinterpret_cast<const unsigned long long*>(&gp->tris)));
  bm.root = (int)leaf.y;
  bm.n_nodes = 0;
  bm.n_tris = 0;
  bm.status = S.T.map.status;
  const unsigned budget = __ldg(&gp->budget);
  RayTrav<kFullStack, 0> r;
  ShortStack<kFullStack> stack;
  if (!r.init(bm, ol, dl, best.t)) return;
  while (!r.step(bm, budget, stack)) {
  }
  if (r.over) { over = true; return; }
  if (r.h.tri < 0) return;
  // r.h.t <= best.t here (the walk's tfar); at equal range the smaller instance,
  // then the smaller face (another piece of the same instance) wins
  if (r.h.t < best.t || best.inst < 0 || ids.w < best.order || (ids.w == best.order && r.h.face < best.face)) {
    best.t = r.h.t;
    best.tri = r.h.tri;
    best.face = r.h.face;
    best.inst = (int)slot;
    best.order = ids.w;
  }
}

// The geometry of an identity instance, walked in the map frame (its mesh frame
// is the map frame); the same tie rule as instance_hit.
__device__ __forceinline__ void direct_hit(const SceneParams& S, uint2 entry, const V& o, const V& d, Best& best,
                                           bool& over) {
  const GeomDev* gp = S.geoms + entry.x;
  DeviceMap bm;
  bm.nodes = reinterpret_cast<const Node*>(__ldg(reinterpret_cast<const unsigned long long*>(&gp->nodes)));
  bm.tris = reinterpret_cast<const Tri*>(__ldg(reinterpret_cast<const unsigned long long*>(&gp->tris)));
  bm.root = __ldg(&gp->root);
  bm.n_nodes = 0;
  bm.n_tris = 0;
  bm.status = S.T.map.status;
  const unsigned budget = __ldg(&gp->budget);
  RayTrav<kFullStack, 0> r;
  ShortStack<kFullStack> stack;
  if (!r.init(bm, o, d, best.t)) return;
  while (!r.step(bm, budget, stack)) {
  }
  if (r.over) { over = true; return; }
  if (r.h.tri < 0) return;
  const uint32_t order = __ldg(&S.inst[entry.y].ids.w);
  if (r.h.t < best.t || best.inst < 0 || order < best.order || (order == best.order && r.h.face < best.face)) {
    best.t = r.h.t;
    best.tri = r.h.tri;
    best.face = r.h.face;
    best.inst = (int)entry.y;
    best.order = order;
  }
}

// Top-level walk with a full stack (depth <= 32 checked at creation; the guard
// below only fires on a corrupt tree).
__device__ __forceinline__ void trace_scene(const SceneParams& S, const V& o, const V& d, float tfar, Best& best,
                                            bool& over) {
  best.t = tfar;
  best.tri = -1;
  best.face = 0xffffffffu;
  best.inst = -1;
  best.order = 0xffffffffu;
  for (uint32_t i = 0; i < S.n_direct && !over; ++i) direct_hit(S, S.direct[i], o, d, best, over);
  const DeviceMap& tl = S.T.map;
  if (tl.root < 0 || over) {
    if (over) {
      best.tri = -1;
      best.t = tfar;
      best.face = 0xffffffffu;
      best.inst = -1;
    }
    return;
  }
  const RayBox rb = make_raybox(o, d);
  int stk_node[kFullStack];
  float stk_t[kFullStack];
  int sp = 0;
  int node = tl.root;
  unsigned steps = 0;
  while (true) {
    if (++steps > S.T.budget) { over = true; break; }
    const Node* np = tl.nodes + node;
    const float4 a = __ldg(&np->a), b = __ldg(&np->b), c = __ldg(&np->c);
    const int4 ln = __ldg(&np->d);
    float tminL, tmaxL, tminR, tmaxR;
    slab(rb, a.x, a.y, a.z, a.w, c.x, c.y, tminL, tmaxL);
    slab(rb, b.x, b.y, b.z, b.w, c.z, c.w, tminR, tmaxR);
    bool hitL = visit(tminL, tmaxL, best.t);
    bool hitR = visit(tminR, tmaxR, best.t);
    const bool leafL = hitL && ln.x < 0, leafR = hitR && ln.y < 0;
    if (leafL || leafR) {  // only an instance walk can move the closest hit: re-cull on this path
      if (leafL) instance_hit(S, ~ln.x, o, d, best, over);
      if (leafR) instance_hit(S, ~ln.y, o, d, best, over);
      if (over) break;
      hitL = hitL && !leafL && tminL <= best.t * kWiden;
      hitR = hitR && !leafR && tminR <= best.t * kWiden;
    }
    if (hitL && hitR) {
      if (sp >= kFullStack) { over = true; break; }
      const bool lf = tminL <= tminR;
      stk_node[sp] = lf ? ln.y : ln.x;
      stk_t[sp] = lf ? tminR : tminL;
      ++sp;
      node = lf ? ln.x : ln.y;
      continue;
    }
    if (hitL || hitR) {
      node = hitL ? ln.x : ln.y;
      continue;
    }
    bool found = false;
    while (sp > 0) {
      --sp;
      node = stk_node[sp];
      if (stk_t[sp] <= best.t * kWiden) { found = true; break; }
    }
    if (!found) break;
  }
  if (over) {
    best.tri = -1;
    best.t = tfar;
    best.face = 0xffffffffu;
    best.inst = -1;
  }
}

#ifndef RMG_SCENE_MIN_BLOCKS
#define RMG_SCENE_MIN_BLOCKS 4
#endif

template <int OK>
__global__ void __launch_bounds__(256, RMG_SCENE_MIN_BLOCKS) k_trace_scene(const SceneParams S) {
  const TraceParams& P = S.T;
  const uint64_t warp = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (warp >= P.n_tiles) return;
  const uint32_t lane = threadIdx.x & 31;
  const uint32_t pose = (uint32_t)(warp / P.tiles_per_pose);
  const uint32_t r = (uint32_t)(warp - (uint64_t)pose * P.tiles_per_pose);
  const uint32_t ty = r / P.tiles_x, tx = r - ty * P.tiles_x;
  const uint32_t tile_w = 1u << P.tile_w_log2;
  const uint32_t vid = ty * P.tile_h + (lane >> P.tile_w_log2);
  const uint32_t hid = tx * tile_w + (lane & (tile_w - 1));
  const uint32_t W = P.sen.width, H = P.sen.height;
  if (vid >= H || hid >= W) return;
  const uint32_t loc = visit_loc(P.sen, vid * W + hid);
  const uint64_t gid = (uint64_t)pose * W * H + loc;

  const Tf Tsm = tmul(load_tf(P.Tbm[pose]), P.Tsb);
  V dir_s, orig_s, o, d;
  setup_ray<OK>(P.sen, Tsm, loc, dir_s, orig_s, o, d);
  Best best;
  bool over = false;
  trace_scene(S, o, d, P.sen.range_max, best, over);
  if (over) atomicExch(P.map.status, (unsigned)RMG_ERR_TRAVERSAL_BUDGET);

  const rmg_outputs& out = P.out;
  if (best.tri >= 0) {
    const float t = best.t;
    if (out.hits) out.hits[gid] = t >= P.sen.range_min ? 1 : 0;
    if (out.ranges) out.ranges[gid] = t;
    if (out.points) {
      const V p = hit_point<OK>(dir_s, orig_s, t);
      float* po = reinterpret_cast<float*>(out.points) + 3 * gid;
      po[0] = p.x; po[1] = p.y; po[2] = p.z;
    }
    const InstDev* ip = S.inst + best.inst;
    if (out.normals) {
      const uint4 ids = __ldg(&ip->ids);
      const Tri* tris = reinterpret_cast<const Tri*>(
          __ldg(reinterpret_cast<const unsigned long long*>(&S.geoms[ids.x].tris)));
      const V nl = face_normal_unit(tris + best.tri);
      const float4 is = __ldg(&ip->inv_s), q = __ldg(&ip->q);
      const V nm = qrot(Q{q.x, q.y, q.z, q.w}, V{mul(nl.x, is.x), mul(nl.y, is.y), mul(nl.z, is.z)});
      const V n = normal_to_sensor(nm, dir_s, Tsm);
      float* no = reinterpret_cast<float*>(out.normals) + 3 * gid;
      no[0] = n.x; no[1] = n.y; no[2] = n.z;
    }
    if (out.face_ids) out.face_ids[gid] = best.face;
    if (out.geom_ids || out.object_ids) {
      const uint4 ids = __ldg(&ip->ids);
      if (out.geom_ids) out.geom_ids[gid] = ids.y;
      if (out.object_ids) out.object_ids[gid] = ids.z;
    }
  } else {
    const float nanf_ = __int_as_float(0x7fc00000);
    if (out.hits) out.hits[gid] = 0;
    if (out.ranges) out.ranges[gid] = add(P.sen.range_max, 1.0f);
    if (out.points) {
      float* po = reinterpret_cast<float*>(out.points) + 3 * gid;
      po[0] = nanf_; po[1] = nanf_; po[2] = nanf_;
    }
    if (out.normals) {
      float* no = reinterpret_cast<float*>(out.normals) + 3 * gid;
      no[0] = nanf_; no[1] = nanf_; no[2] = nanf_;
    }
    if (out.face_ids) out.face_ids[gid] = 0xffffffffu;
    if (out.geom_ids) out.geom_ids[gid] = 0xffffffffu;
    if (out.object_ids) out.object_ids[gid] = 0xffffffffu;
  }
}

// Request of k_piece_boxes: the box of one piece, read from its parent node.
struct PieceReq {
  const Node* nodes;
  int parent, side;
};

// Current boxes of the pieces (after any refit of their geometries).
__global__ void k_piece_boxes(const PieceReq* req, uint32_t n, float* out) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const PieceReq q = req[i];
  const Node* p = q.nodes + q.parent;
  const float4 a = p->a, b = p->b, c = p->c;
  float* o = out + 6 * (size_t)i;
  if (q.side == 0) {
    o[0] = a.x; o[1] = a.z; o[2] = c.x; o[3] = a.y; o[4] = a.w; o[5] = c.y;
  } else {
    o[0] = b.x; o[1] = b.z; o[2] = c.z; o[3] = b.y; o[4] = b.w; o[5] = c.w;
  }
}

}  // namespace

int default_config(const rmg_sensor* s, rmg_launch_config* cfg);
int make_trace_params(const rmg_map* map, const rmg_sensor* sensor, const rmg_transform* Tsb,
                      const rmg_transform* Tbm, uint32_t n_poses, const rmg_outputs* out,
                      const rmg_launch_config& cfg, TraceParams& P);
DeviceMap device_view(const rmg_map* m);

}  // namespace rmg

using namespace rmg;

// A piece of an opened geometry tree: subtree root `node`, the box of which
// sits in child slot `side` of node `parent`.
struct ScenePiece {
  int node, parent, side;
};

struct rmg_scene {
  int device = 0;
  std::vector<const rmg_map*> geoms;
  std::vector<std::vector<ScenePiece>> pieces;  // per geometry; empty = not opened
  std::vector<uint32_t> piece_base;             // per geometry: first request in d_piece_req
  uint32_t n_pieces = 0;
  uint32_t n_instances = 0;
  std::vector<uint32_t> live;   // instance index of each live instance record
  uint32_t n_leaves = 0;        // top-level leaves: (instance, piece) pairs
  std::vector<uint2> direct;    // (geometry, instance record) of the geometries walked without the top tree
  rmg_map* tlas = nullptr;      // NULL when no instance is in the top tree
  InstDev* d_inst = nullptr;
  uint2* d_leaves = nullptr;
  GeomDev* d_geoms = nullptr;
  PieceReq* d_piece_req = nullptr;
  float* d_piece_box = nullptr;  // 6 per piece: lo, hi
  unsigned int* d_status = nullptr;
};

namespace {

void free_scene(rmg_scene* s) {
  if (s->tlas) rmg_map_destroy(s->tlas);
  cudaFree(s->d_inst);
  cudaFree(s->d_leaves);
  cudaFree(s->d_geoms);
  cudaFree(s->d_piece_req);
  cudaFree(s->d_piece_box);
  cudaFree(s->d_status);
  delete s;
}

// Triangles per piece of an opened geometry tree; 0 opens none.  Measured on
// the 1M-triangle terrain under 2,000 box instances (the terrain cut into
// K x K separate meshes as a stand-in): 3,864 Mrays/s unopened, 4,525 / 4,620 /
// 4,613 / 4,548 for 16 / 64 / 256 / 1,024 pieces of 62k / 16k / 4k / 1k.
#ifndef RMG_SCENE_PIECE_TRIS
#define RMG_SCENE_PIECE_TRIS 16384
#endif
constexpr uint32_t kMaxPieces = 256;

double box_area(const float lo[3], const float hi[3]) {
  const double dx = (double)hi[0] - lo[0], dy = (double)hi[1] - lo[1], dz = (double)hi[2] - lo[2];
  return dx * dy + dy * dz + dz * dx;
}

// Opens the tree of a geometry with at least 2 x RMG_SCENE_PIECE_TRIS
// triangles into about n_faces / RMG_SCENE_PIECE_TRIS pieces (at most
// kMaxPieces): the piece with the largest box surface is replaced by its two
// children until there are enough, or until every piece has a leaf child.
int open_geometry(const rmg_map* g, cudaStream_t st, std::vector<ScenePiece>& out) {
  out.clear();
  const uint32_t per = RMG_SCENE_PIECE_TRIS;
  if (per == 0 || g->n_faces < 2u * per) return RMG_OK;
  const uint32_t want = std::min<uint32_t>(kMaxPieces, g->n_faces / per);
  struct Cand {
    ScenePiece p;
    float lo[3], hi[3];
    bool closed;  // has a leaf child: stays whole
  };
  std::vector<Cand> c;
  c.push_back(Cand{ScenePiece{0, -1, 0}, {g->lo[0], g->lo[1], g->lo[2]}, {g->hi[0], g->hi[1], g->hi[2]}, false});
  RMG_CUDA_TRY(cudaStreamSynchronize(st));
  while (c.size() < want) {
    int pick = -1;
    double area = -1.0;
    for (size_t i = 0; i < c.size(); ++i)
      if (!c[i].closed && box_area(c[i].lo, c[i].hi) > area) { area = box_area(c[i].lo, c[i].hi); pick = (int)i; }
    if (pick < 0) break;
    Node nd;
    RMG_CUDA_TRY(cudaMemcpyAsync(&nd, g->d_nodes + c[pick].p.node, sizeof nd, cudaMemcpyDeviceToHost, st));
    RMG_CUDA_TRY(cudaStreamSynchronize(st));
    if (nd.d.x < 0 || nd.d.y < 0) { c[pick].closed = true; continue; }
    const int parent = c[pick].p.node;
    c[pick] = Cand{ScenePiece{nd.d.x, parent, 0}, {nd.a.x, nd.a.z, nd.c.x}, {nd.a.y, nd.a.w, nd.c.y}, false};
    c.push_back(Cand{ScenePiece{nd.d.y, parent, 1}, {nd.b.x, nd.b.z, nd.c.z}, {nd.b.y, nd.b.w, nd.c.w}, false});
  }
  if (c.size() < 2) return RMG_OK;
  for (const Cand& x : c) out.push_back(x.p);
  return RMG_OK;
}


// q (x) p (x) conj(q) in binary64 with the binary32 q as given.
void qrot_d(const rmg_quat& q, const double p[3], double out[3]) {
  const double qx = q.x, qy = q.y, qz = q.z, qw = q.w;
  // a = q * (p, 0)
  const double ax = qw * p[0] + qy * p[2] - qz * p[1];
  const double ay = qw * p[1] - qx * p[2] + qz * p[0];
  const double az = qw * p[2] + qx * p[1] - qy * p[0];
  const double aw = -qx * p[0] - qy * p[1] - qz * p[2];
  // a * conj(q)
  out[0] = -aw * qx + ax * qw - ay * qz + az * qy;
  out[1] = -aw * qy + ax * qz + ay * qw - az * qx;
  out[2] = -aw * qz - ax * qy + ay * qx + az * qw;
}

int check_instances(const rmg_scene* s, const rmg_instance_desc* inst, uint32_t n) {
  if (n > 0 && !inst) return fail(RMG_ERR_INVALID_ARG, "scene: instances is NULL");
  if (n > (1u << 24)) return fail(RMG_ERR_INVALID_ARG, "scene: too many instances");
  for (uint32_t i = 0; i < n; ++i) {
    const rmg_instance_desc& I = inst[i];
    if (I.geometry >= s->geoms.size()) return fail(RMG_ERR_INVALID_ARG, "scene: instance geometry index out of range");
    const float sc[3] = {I.scale.x, I.scale.y, I.scale.z};
    for (float v : sc)
      if (!(std::isfinite(v) && v != 0.0f)) return fail(RMG_ERR_INVALID_ARG, "scene: instance scale must be finite and non-zero");
    const double qn = std::sqrt((double)I.T.R.x * I.T.R.x + (double)I.T.R.y * I.T.R.y + (double)I.T.R.z * I.T.R.z +
                                (double)I.T.R.w * I.T.R.w);
    if (!(std::fabs(qn - 1.0) < 1e-3)) return fail(RMG_ERR_INVALID_ARG, "scene: instance rotation is not a unit quaternion");
    if (!(std::isfinite(I.T.t.x) && std::isfinite(I.T.t.y) && std::isfinite(I.T.t.z)))
      return fail(RMG_ERR_INVALID_ARG, "scene: instance translation is not finite");
  }
  return RMG_OK;
}

// Map-frame box of a mesh-frame box [lo, hi] under an instance, padded by 1e-5
// of the coordinates' magnitude so that the binary32 ray transform of a hit
// near the box's faces can never fall outside: the top-level "triangle"
// (lo, hi, centre).
void world_box(const rmg_instance_desc& I, const float lo_m[3], const float hi_m[3], std::vector<rmg_vec3>& verts,
               std::vector<rmg_face>& faces) {
  double lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
  double mag = 1.0;
  for (int c = 0; c < 8; ++c) {
    const double p[3] = {(double)I.scale.x * ((c & 1) ? hi_m[0] : lo_m[0]),
                         (double)I.scale.y * ((c & 2) ? hi_m[1] : lo_m[1]),
                         (double)I.scale.z * ((c & 4) ? hi_m[2] : lo_m[2])};
    double w[3];
    qrot_d(I.T.R, p, w);
    w[0] += I.T.t.x; w[1] += I.T.t.y; w[2] += I.T.t.z;
    for (int k = 0; k < 3; ++k) {
      lo[k] = std::min(lo[k], w[k]);
      hi[k] = std::max(hi[k], w[k]);
      mag = std::max(mag, std::fabs(w[k]));
    }
  }
  const double pad = 1e-5 * mag;
  rmg_vec3 vlo, vhi, vc;
  float* fl = &vlo.x;
  float* fh = &vhi.x;
  float* fc = &vc.x;
  for (int k = 0; k < 3; ++k) {
    fl[k] = std::nextafter((float)(lo[k] - pad), -INFINITY);
    fh[k] = std::nextafter((float)(hi[k] + pad), INFINITY);
    fc[k] = (float)(0.5 * ((double)fl[k] + (double)fh[k]));
  }
  const uint32_t b = (uint32_t)verts.size();
  verts.push_back(vlo);
  verts.push_back(vhi);
  verts.push_back(vc);
  faces.push_back(rmg_face{b, b + 1, b + 2});
}

// The top-level leaves: one per (live instance, piece of its geometry's tree),
// or per live instance where the tree is not opened, with their boxes, and the
// record of every live instance.
int instance_leaves(const rmg_scene* s, const rmg_instance_desc* inst, uint32_t n, cudaStream_t st,
                    std::vector<uint32_t>& live, std::vector<rmg_vec3>& verts, std::vector<rmg_face>& faces,
                    std::vector<InstDev>& rec, std::vector<uint2>& leaves, std::vector<uint2>& direct) {
  live.clear();
  verts.clear();
  faces.clear();
  rec.clear();
  leaves.clear();
  direct.clear();
  std::vector<char> walked(s->geoms.size(), 0);  // geometry walked directly
  std::vector<float> pbox;
  if (s->n_pieces > 0) {
    const unsigned grid = (s->n_pieces + 127) / 128;
    k_piece_boxes<<<grid, 128, 0, st>>>(s->d_piece_req, s->n_pieces, s->d_piece_box);
    RMG_CUDA_TRY(cudaGetLastError());
    pbox.resize(6 * (size_t)s->n_pieces);
    RMG_CUDA_TRY(cudaMemcpyAsync(pbox.data(), s->d_piece_box, sizeof(float) * pbox.size(), cudaMemcpyDeviceToHost, st));
    RMG_CUDA_TRY(cudaStreamSynchronize(st));
  }
  for (uint32_t i = 0; i < n; ++i) {
    const rmg_instance_desc& I = inst[i];
    const rmg_map* g = s->geoms[I.geometry];
    if (g->n_faces == 0) continue;
    const bool identity = I.T.R.x == 0.0f && I.T.R.y == 0.0f && I.T.R.z == 0.0f && I.T.R.w == 1.0f &&
                          I.T.t.x == 0.0f && I.T.t.y == 0.0f && I.T.t.z == 0.0f && I.scale.x == 1.0f &&
                          I.scale.y == 1.0f && I.scale.z == 1.0f;
    if (identity && walked[I.geometry]) continue;  // never wins against the first identity instance
    const uint32_t slot = (uint32_t)rec.size();
    const std::vector<ScenePiece>& pc = s->pieces[I.geometry];
    if (identity && direct.size() < kMaxDirect) {
      walked[I.geometry] = 1;
      direct.push_back(make_uint2(I.geometry, slot));
    } else if (pc.empty()) {
      world_box(I, g->lo, g->hi, verts, faces);
      leaves.push_back(make_uint2(slot, 0u));
    } else {
      for (size_t j = 0; j < pc.size(); ++j) {
        const float* b = &pbox[6 * ((size_t)s->piece_base[I.geometry] + j)];
        world_box(I, b, b + 3, verts, faces);
        leaves.push_back(make_uint2(slot, (uint32_t)pc[j].node));
      }
    }
    InstDev r;
    r.qinv = make_float4(-I.T.R.x, -I.T.R.y, -I.T.R.z, I.T.R.w);
    r.t = make_float4(I.T.t.x, I.T.t.y, I.T.t.z, 0.0f);
    r.inv_s = make_float4(1.0f / I.scale.x, 1.0f / I.scale.y, 1.0f / I.scale.z, 0.0f);
    r.q = make_float4(I.T.R.x, I.T.R.y, I.T.R.z, I.T.R.w);
    r.ids = make_uint4(I.geometry, I.geom_id, I.object_id, i);
    rec.push_back(r);
    live.push_back(i);
  }
  return RMG_OK;
}

int upload_instances(rmg_scene* s, const std::vector<InstDev>& rec, const std::vector<uint2>& leaves,
                     cudaStream_t st) {
  cudaFree(s->d_inst);
  s->d_inst = nullptr;
  cudaFree(s->d_leaves);
  s->d_leaves = nullptr;
  if (rec.empty()) return RMG_OK;
  int r = dev_alloc(&s->d_inst, rec.size(), "scene instances");
  if (r == RMG_OK) r = dev_alloc(&s->d_leaves, std::max<size_t>(1, leaves.size()), "scene leaves");
  if (r != RMG_OK) return r;
  RMG_CUDA_TRY(cudaMemcpyAsync(s->d_inst, rec.data(), sizeof(InstDev) * rec.size(), cudaMemcpyHostToDevice, st));
  if (!leaves.empty())
    RMG_CUDA_TRY(cudaMemcpyAsync(s->d_leaves, leaves.data(), sizeof(uint2) * leaves.size(), cudaMemcpyHostToDevice, st));
  return RMG_OK;
}

int build_top(rmg_scene* s, const rmg_instance_desc* inst, uint32_t n, bool rebuild, cudaStream_t st) {
  std::vector<uint32_t> live;
  std::vector<rmg_vec3> verts;
  std::vector<rmg_face> faces;
  std::vector<InstDev> rec;
  std::vector<uint2> leaves;
  std::vector<uint2> direct;
  int r = instance_leaves(s, inst, n, st, live, verts, faces, rec, leaves, direct);
  if (r != RMG_OK) return r;
  bool same_direct = direct.size() == s->direct.size();
  for (size_t i = 0; same_direct && i < direct.size(); ++i)
    same_direct = direct[i].x == s->direct[i].x && direct[i].y == s->direct[i].y;
  const bool same = s->tlas && same_direct && live.size() == s->live.size() && leaves.size() == s->n_leaves &&
                    !leaves.empty();
  if (!rebuild && same) {
    r = rmg_map_refit(s->tlas, verts.data(), (uint32_t)verts.size(), st);
  } else {
    if (s->tlas) { rmg_map_destroy(s->tlas); s->tlas = nullptr; }
    if (!faces.empty()) {
      r = rmg_map_build(verts.data(), (uint32_t)verts.size(), faces.data(), (uint32_t)faces.size(), st, &s->tlas);
      if (r == RMG_OK && s->tlas->depth > (unsigned)kFullStack)
        r = fail(RMG_ERR_UNSUPPORTED, "scene: top-level tree deeper than 32 levels");
    }
  }
  if (r != RMG_OK) return r;
  r = upload_instances(s, rec, leaves, st);
  if (r != RMG_OK) return r;
  RMG_CUDA_TRY(cudaStreamSynchronize(st));
  s->live = live;
  s->n_leaves = (uint32_t)leaves.size();
  s->direct = direct;
  s->n_instances = n;
  return RMG_OK;
}

}  // namespace

extern "C" int rmg_scene_create(const rmg_map* const* geometries, uint32_t n_geometries,
                                const rmg_instance_desc* instances, uint32_t n_instances, void* stream,
                                rmg_scene** out) {
  return guarded("rmg_scene_create", [&]() -> int {
    if (!out) return fail(RMG_ERR_INVALID_ARG, "rmg_scene_create: out is NULL");
    *out = nullptr;
    if (n_geometries > 0 && !geometries) return fail(RMG_ERR_INVALID_ARG, "rmg_scene_create: geometries is NULL");
    rmg_scene* s = new (std::nothrow) rmg_scene;
    if (!s) return fail(RMG_ERR_OOM, "rmg_scene_create: host allocation");
    cudaGetDevice(&s->device);
    for (uint32_t g = 0; g < n_geometries; ++g) {
      if (!geometries[g]) { delete s; return fail(RMG_ERR_INVALID_ARG, "rmg_scene_create: NULL geometry"); }
      if (geometries[g]->n_faces > 0 && geometries[g]->depth > (unsigned)kFullStack) {
        delete s;
        return fail(RMG_ERR_UNSUPPORTED, "rmg_scene_create: a geometry's tree is deeper than 32 levels");
      }
      s->geoms.push_back(geometries[g]);
    }
    int r = check_instances(s, instances, n_instances);
    if (r != RMG_OK) { delete s; return r; }
    cudaStream_t st = as_stream(stream);
    r = dev_alloc(&s->d_status, 1, "scene status");
    if (r == RMG_OK) r = cuda_status(cudaMemsetAsync(s->d_status, 0, 4, st), "memset");
    if (r == RMG_OK && n_geometries > 0) {
      std::vector<GeomDev> g(n_geometries);
      for (uint32_t i = 0; i < n_geometries; ++i) {
        const DeviceMap dm = device_view(geometries[i]);
        g[i] = GeomDev{dm.nodes, dm.tris, dm.root, 2u * geometries[i]->n_nodes + 64u};
      }
      r = dev_alloc(&s->d_geoms, n_geometries, "scene geometries");
      if (r == RMG_OK)
        r = cuda_status(cudaMemcpyAsync(s->d_geoms, g.data(), sizeof(GeomDev) * n_geometries, cudaMemcpyHostToDevice, st),
                        "copy geometries");
    }
    // Open the trees of large geometries into pieces (only those some instance places).
    s->pieces.assign(n_geometries, {});
    s->piece_base.assign(n_geometries, 0);
    std::vector<bool> used(n_geometries, false);
    for (uint32_t i = 0; i < n_instances; ++i) used[instances[i].geometry] = true;
    std::vector<PieceReq> req;
    for (uint32_t gi = 0; r == RMG_OK && gi < n_geometries; ++gi) {
      if (!used[gi]) continue;
      r = open_geometry(geometries[gi], st, s->pieces[gi]);
      s->piece_base[gi] = (uint32_t)req.size();
      for (const ScenePiece& p : s->pieces[gi]) req.push_back(PieceReq{geometries[gi]->d_nodes, p.parent, p.side});
    }
    // Bound the top tree: with more than 2^22 leaves from opened trees, open none.
    uint64_t n_leaves = 0;
    for (uint32_t i = 0; i < n_instances; ++i) n_leaves += std::max<size_t>(1, s->pieces[instances[i].geometry].size());
    if (n_leaves > (1ull << 22)) {
      for (auto& pc : s->pieces) pc.clear();
      req.clear();
    }
    s->n_pieces = (uint32_t)req.size();
    if (r == RMG_OK && !req.empty()) {
      r = dev_alloc(&s->d_piece_req, req.size(), "scene pieces");
      if (r == RMG_OK) r = dev_alloc(&s->d_piece_box, 6 * req.size(), "scene piece boxes");
      if (r == RMG_OK)
        r = cuda_status(cudaMemcpyAsync(s->d_piece_req, req.data(), sizeof(PieceReq) * req.size(), cudaMemcpyHostToDevice,
                                        st), "copy pieces");
    }
    if (r == RMG_OK) r = build_top(s, instances, n_instances, true, st);
    if (r != RMG_OK) { free_scene(s); return r; }
    *out = s;
    return RMG_OK;
  });
}

extern "C" int rmg_scene_update(rmg_scene* s, const rmg_instance_desc* instances, uint32_t n_instances, int rebuild,
                                void* stream) {
  return guarded("rmg_scene_update", [&]() -> int {
    if (!s) return fail(RMG_ERR_INVALID_ARG, "rmg_scene_update: scene is NULL");
    if (n_instances != s->n_instances) return fail(RMG_ERR_INVALID_ARG, "rmg_scene_update: instance count differs");
    int r = check_instances(s, instances, n_instances);
    if (r != RMG_OK) return r;
    return build_top(s, instances, n_instances, rebuild != 0, as_stream(stream));
  });
}

extern "C" int rmg_scene_destroy(rmg_scene* s) {
  return guarded("rmg_scene_destroy", [&]() -> int {
    if (!s) return RMG_OK;
    free_scene(s);
    return RMG_OK;
  });
}

extern "C" int rmg_scene_status(rmg_scene* s, int clear) {
  return guarded("rmg_scene_status", [&]() -> int {
    if (!s) return fail(RMG_ERR_INVALID_ARG, "rmg_scene_status: scene is NULL");
    unsigned int word = 0;
    RMG_CUDA_TRY(cudaMemcpy(&word, s->d_status, 4, cudaMemcpyDeviceToHost));
    if (clear) RMG_CUDA_TRY(cudaMemset(s->d_status, 0, 4));
    if (word != 0) {
      set_error("a kernel recorded a device error on this scene");
      return (int)word;
    }
    return RMG_OK;
  });
}

extern "C" int rmg_simulate_scene(const rmg_scene* s, const rmg_sensor* sensor, const rmg_transform* Tsb,
                                  const rmg_transform* Tbm, uint32_t n_poses, const rmg_outputs* out, void* stream) {
  return guarded("rmg_simulate_scene", [&]() -> int {
    if (!s || !sensor || !Tsb || !out)
      return fail(RMG_ERR_INVALID_ARG, "rmg_simulate_scene: NULL scene, sensor, Tsb or outputs");
    if (n_poses == 0) return RMG_OK;
    if (!Tbm) return fail(RMG_ERR_INVALID_ARG, "rmg_simulate_scene: Tbm is NULL");
    if (!out->hits && !out->ranges && !out->points && !out->normals && !out->face_ids && !out->geom_ids &&
        !out->object_ids)
      return RMG_OK;
    rmg_launch_config cfg;
    default_config(sensor, &cfg);
    SceneParams S;
    // the top-level tree's launch geometry; an empty scene uses a zero-face stand-in view
    rmg_map empty;
    std::memset(&empty, 0, sizeof(empty));
    const rmg_map* top = s->tlas ? s->tlas : &empty;
    make_trace_params(top, sensor, Tsb, Tbm, n_poses, out, cfg, S.T);
    S.T.map.status = s->d_status;
    S.inst = s->d_inst;
    S.geoms = s->d_geoms;
    S.leaves = s->d_leaves;
    S.n_direct = (uint32_t)s->direct.size();
    for (uint32_t i = 0; i < kMaxDirect; ++i) S.direct[i] = i < S.n_direct ? s->direct[i] : make_uint2(0u, 0u);
    const uint64_t blocks = (S.T.n_tiles + cfg.block_warps - 1) / cfg.block_warps;
    if (blocks > 0x7fffffffull) return fail(RMG_ERR_INVALID_ARG, "rmg_simulate_scene: too many rays for one launch");
    const unsigned block = 32u * cfg.block_warps;
    cudaStream_t st = as_stream(stream);
    switch (sensor->model.kind) {
      case RMG_MODEL_SPHERICAL:
      case RMG_MODEL_PINHOLE: k_trace_scene<ORIGIN_POSE><<<(unsigned)blocks, block, 0, st>>>(S); break;
      case RMG_MODEL_O1DN: k_trace_scene<ORIGIN_SINGLE><<<(unsigned)blocks, block, 0, st>>>(S); break;
      default: k_trace_scene<ORIGIN_TABLE><<<(unsigned)blocks, block, 0, st>>>(S); break;
    }
    return cuda_status(cudaGetLastError(), "k_trace_scene");
  });
}
