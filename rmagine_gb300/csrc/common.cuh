// Internal definitions shared by the CUDA translation units of librmg_gb300.
//
// Arithmetic that decides WHICH triangle a ray hits, and the ray itself, is
// written with explicit rounding intrinsics (__fmul_rn / __fadd_rn / __fsub_rn
// / __fmaf_rn) so that nvcc cannot contract or reorder it.  That makes every
// ray and every triangle test a fixed sequence of IEEE-754 binary32
// operations, the same sequence a host implementation produces with
// -ffp-contract=off and explicit fmaf() in the same places.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <math.h>

#include "../../include/rmg.h"

namespace rmg {

// ----------------------------------------------------------------------------
// Device data layout of a map.
//
// Internal BVH node, 64 B, both children's boxes in the parent so that one
// node visit tests two boxes with three 16-byte loads plus one for the links:
//   a = (L.lo.x, L.hi.x, L.lo.y, L.hi.y)
//   b = (R.lo.x, R.hi.x, R.lo.y, R.hi.y)
//   c = (L.lo.z, L.hi.z, R.lo.z, R.hi.z)
//   d = (left, right, parent, split_bit)     ints
// Children >= 0 are internal node indices; a child < 0 is the leaf holding
// packed triangle ~child.  parent of the root is -1.
//
// Packed triangle, 48 B, in Morton (leaf) order:
//   v0 = (x, y, z, face id as int bits), v1 = (x, y, z, 0), v2 = (x, y, z, 0)
// ----------------------------------------------------------------------------
struct __align__(16) Node {
  float4 a, b, c;
  int4 d;
};

struct __align__(16) Tri {
  float4 v0, v1, v2;
};

// 4-wide node, 128 B (one cache line), collapsed from the binary tree:
// the four child boxes as structure of arrays (component k = child k), the
// child links (>= 0 wide node, < 0 leaf ~packed triangle, kEmpty4 = no child,
// whose box is a point at 1e30 that no ray reaches), and meta = (children,
// parent wide node or -1, 0, 0).
constexpr int kEmpty4 = (int)0x80000000;

struct __align__(16) Node4 {
  float4 lox, hix, loy, hiy, loz, hiz;
  int4 child;
  int4 meta;
};

// 8-wide node with quantized child boxes, 80 B (wide8.cu):
//   h0 = (p.x, p.y, p.z, e.x + 127 | (e.y + 127) << 8 | (e.z + 127) << 16 | imask << 24 as bits)
//   h1 = (child_base, tri_base, valid, 0)
//   qx = (lo.x slots 0-3, lo.x slots 4-7, hi.x slots 0-3, hi.x slots 4-7), one byte per slot; qy, qz alike
// Slot k's box is [p + 2^e * q_lo, p + 2^e * q_hi] per axis, containing the
// child's exact box.  valid / imask: bit k set when slot k holds a child / an
// internal child.  Internal children are nodes child_base + (internal slots
// below k), leaf children triangles tri_base + (leaf slots below k) of tris8.
struct __align__(16) Node8 {
  float4 h0;
  uint4 h1;
  uint4 qx, qy, qz;
};

static_assert(sizeof(Node) == 64, "node record is 64 B");
static_assert(sizeof(Node8) == 80, "8-wide node record is 80 B");
static_assert(sizeof(Node4) == 128, "wide node record is 128 B");
static_assert(sizeof(Tri) == 48, "triangle record is 48 B");

// Device error word values are rmg_status codes.
struct DeviceMap {
  const Node4* nodes4;  // the 4-wide tree, or NULL
  const Node8* nodes8;  // the 8-wide tree, or NULL
  const Tri* tris8;     // its triangles (a permutation of tris), or NULL
  const Node* nodes;
  const Tri* tris;
  int n_nodes;
  int n_tris;
  int root;            // 0, or -1 when the map is empty
  unsigned int* status;  // device error word
};

struct SensorDev {
  uint32_t kind;
  uint32_t width, height;
  float range_min, range_max;
  const float* dirs;    // 3*width*height floats (sensor frame)
  const float* origs;   // OnDn: 3*width*height floats, else NULL
  float3 orig;          // O1Dn origin
  const uint32_t* order;  // visiting order of the table's rays (O1Dn / OnDn), NULL = the table's own
};

// The table entry (and output element) of launch slot i: a sensor whose table
// of scattered directions was sorted for coherence visits its rays in that
// order; every per-ray input and output stays at the table's own index.
__device__ __forceinline__ uint32_t visit_loc(const SensorDev& sen, uint32_t i) {
  return sen.order ? __ldg(sen.order + i) : i;
}

// ----------------------------------------------------------------------------
// Exact-order small math (no contraction).
// ----------------------------------------------------------------------------
struct Q { float x, y, z, w; };
struct V { float x, y, z; };

__device__ __forceinline__ float mul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float add(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float sub(float a, float b) { return __fsub_rn(a, b); }

// Hamilton product in the term order of rmagine's Quaternion::mult
// (math/types/Quaternion.tcc:35-42), each term rounded, summed left to right.
__device__ __forceinline__ Q qmul(const Q& a, const Q& b) {
  Q r;
  r.x = sub(add(add(mul(a.w, b.x), mul(a.x, b.w)), mul(a.y, b.z)), mul(a.z, b.y));
  r.y = add(add(sub(mul(a.w, b.y), mul(a.x, b.z)), mul(a.y, b.w)), mul(a.z, b.x));
  r.z = add(sub(add(mul(a.w, b.z), mul(a.x, b.y)), mul(a.y, b.x)), mul(a.z, b.w));
  r.w = sub(sub(sub(mul(a.w, b.w), mul(a.x, b.x)), mul(a.y, b.y)), mul(a.z, b.z));
  return r;
}

__device__ __forceinline__ Q qconj(const Q& q) { return Q{-q.x, -q.y, -q.z, q.w}; }

// Rotation as the full sandwich q * (p, 0) * conj(q) (Quaternion.tcc:68-75).
__device__ __forceinline__ V qrot(const Q& q, const V& p) {
  const Q P{p.x, p.y, p.z, 0.0f};
  const Q r = qmul(qmul(q, P), qconj(q));
  return V{r.x, r.y, r.z};
}

struct Tf { Q R; V t; };

// Transform composition T1 * T2 (Transform.tcc:34-42): t = R1*t2 + t1, R = R1*R2.
__device__ __forceinline__ Tf tmul(const Tf& a, const Tf& b) {
  Tf r;
  const V rt = qrot(a.R, b.t);
  r.R = qmul(a.R, b.R);
  r.t = V{add(rt.x, a.t.x), add(rt.y, a.t.y), add(rt.z, a.t.z)};
  return r;
}

__device__ __forceinline__ Tf load_tf(const rmg_transform& T) {
  return Tf{Q{T.R.x, T.R.y, T.R.z, T.R.w}, V{T.t.x, T.t.y, T.t.z}};
}

// ----------------------------------------------------------------------------
// Watertight ray/triangle test (Woop, Benthin, Wald, "Watertight
// Ray/Triangle Intersection", JCGT 2(1), 2013).
//
// Per-ray constants: kz = axis of largest |dir|, kx/ky the other two in
// cyclic order, swapped when dir[kz] < 0 to keep the winding; shear
// Sx = d[kx]/d[kz], Sy = d[ky]/d[kz], Sz = 1/d[kz].
// The edge functions U, V, W are computed without fused multiply-add so that
// the shared edge of two neighbouring triangles yields exactly opposite
// values (the watertightness argument of the paper); when any of them is
// exactly zero they are recomputed in binary64 from the same binary32
// inputs, as the paper prescribes.
// Accepts 0 < t <= tfar, both windings.
// ----------------------------------------------------------------------------
struct RayW {
  float ox, oy, oz;
  int kx, ky, kz;
  float Sx, Sy, Sz;
};

__device__ __forceinline__ float comp(const float3& v, int k) {
  return k == 0 ? v.x : (k == 1 ? v.y : v.z);
}

__device__ __forceinline__ RayW make_rayw(V o, V d) {
  RayW r;
  r.ox = o.x; r.oy = o.y; r.oz = o.z;
  const float ax = fabsf(d.x), ay = fabsf(d.y), az = fabsf(d.z);
  int kz = 0;
  if (ay > ax) kz = 1;
  if (az > fmaxf(ax, ay)) kz = 2;
  int kx = kz + 1; if (kx == 3) kx = 0;
  int ky = kx + 1; if (ky == 3) ky = 0;
  const float dz = kz == 0 ? d.x : (kz == 1 ? d.y : d.z);
  if (dz < 0.0f) { const int t = kx; kx = ky; ky = t; }
  const float dx = kx == 0 ? d.x : (kx == 1 ? d.y : d.z);
  const float dy = ky == 0 ? d.x : (ky == 1 ? d.y : d.z);
  r.kx = kx; r.ky = ky; r.kz = kz;
  r.Sx = __fdiv_rn(dx, dz);
  r.Sy = __fdiv_rn(dy, dz);
  r.Sz = __fdiv_rn(1.0f, dz);
  return r;
}

// Returns true and sets t when the ray hits the triangle with 0 < t <= tfar.
__device__ __forceinline__ bool tri_hit(const RayW& r, const float4& p0, const float4& p1,
                                        const float4& p2, float tfar, float& t_out) {
  const float3 A = make_float3(sub(p0.x, r.ox), sub(p0.y, r.oy), sub(p0.z, r.oz));
  const float3 B = make_float3(sub(p1.x, r.ox), sub(p1.y, r.oy), sub(p1.z, r.oz));
  const float3 C = make_float3(sub(p2.x, r.ox), sub(p2.y, r.oy), sub(p2.z, r.oz));
  const float Akz = comp(A, r.kz), Bkz = comp(B, r.kz), Ckz = comp(C, r.kz);
  const float Ax = __fmaf_rn(-r.Sx, Akz, comp(A, r.kx));
  const float Ay = __fmaf_rn(-r.Sy, Akz, comp(A, r.ky));
  const float Bx = __fmaf_rn(-r.Sx, Bkz, comp(B, r.kx));
  const float By = __fmaf_rn(-r.Sy, Bkz, comp(B, r.ky));
  const float Cx = __fmaf_rn(-r.Sx, Ckz, comp(C, r.kx));
  const float Cy = __fmaf_rn(-r.Sy, Ckz, comp(C, r.ky));
  float U = sub(mul(Cx, By), mul(Cy, Bx));
  float Vv = sub(mul(Ax, Cy), mul(Ay, Cx));
  float W = sub(mul(Bx, Ay), mul(By, Ax));
  if (U == 0.0f || Vv == 0.0f || W == 0.0f) {
    const double CxBy = (double)Cx * (double)By, CyBx = (double)Cy * (double)Bx;
    U = (float)(CxBy - CyBx);
    const double AxCy = (double)Ax * (double)Cy, AyCx = (double)Ay * (double)Cx;
    Vv = (float)(AxCy - AyCx);
    const double BxAy = (double)Bx * (double)Ay, ByAx = (double)By * (double)Ax;
    W = (float)(BxAy - ByAx);
  }
  if ((U < 0.0f || Vv < 0.0f || W < 0.0f) && (U > 0.0f || Vv > 0.0f || W > 0.0f)) return false;
  const float det = add(add(U, Vv), W);
  if (det == 0.0f) return false;
  const float Az = mul(r.Sz, Akz), Bz = mul(r.Sz, Bkz), Cz = mul(r.Sz, Ckz);
  const float T = __fmaf_rn(U, Az, __fmaf_rn(Vv, Bz, mul(W, Cz)));
  // Cheap reject before the division: T/det <= 0, or T/det certainly beyond
  // tfar (the 1+1e-6 margin covers the rounding of the two products, so this
  // never rejects a triangle that the exact test below would accept).
  const float Ts = det < 0.0f ? -T : T;
  if (!(Ts > 0.0f)) return false;
  if (Ts > mul(mul(tfar, fabsf(det)), 1.000001f)) return false;
  // The decision itself: 0 < t <= tfar on the correctly rounded quotient.
  const float t = __fdiv_rn(T, det);
  if (!(t > 0.0f) || !(t <= tfar)) return false;
  t_out = t;
  return true;
}

}  // namespace rmg
