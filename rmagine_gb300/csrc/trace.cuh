// Per-ray closest-hit traversal of the LBVH and the attribute epilogue.
//
// This is the GPU restatement of the per-ray body of rmagine's simulators:
//   SphereSimulatorEmbree.tcc:69-249 (ray setup, rtcIntersect1, attributes)
//   O1DnSimulatorEmbree.tcc:84-132, OnDnSimulatorEmbree.tcc:86-134 (origins)
// with the BVH query done by this file instead of Embree/OptiX.
//
// Traversal ("short stack + parent pointers"):
//   * Every internal node carries both child boxes; a visit tests the two
//     boxes, intersects leaf children (one triangle each) on the spot and
//     descends into the nearer hit internal child.
//   * A trail of 32, 64 or 128 bits (chosen from the tree depth) records, one
//     bit per level, whether the other child of that level is still pending.  The pending children themselves are kept
//     in a circular short stack of SS entries (SS = 0: none).  When the stack
//     has run dry but the trail still has pending levels, the ray climbs the
//     parent links to the pending level and takes the sibling: stackless
//     backtracking in the manner of Hapala et al. 2011 / Afra and
//     Szirmay-Kalos 2014, so any SS gives the same visits and results.
//   * Box tests widen every plane distance outward by |o/d| 2^-21 and the
//     interval by 2^-22 relative (RayBox); triangle tests are the
//     watertight test of common.cuh.  Closest-hit ties are broken by the
//     smaller face id, so the result does not depend on traversal order.
//   * Every ray has a step budget (2 * internal nodes + 64 node visits and
//     parent climbs, more than any valid tree needs).  Exceeding it records
//     RMG_ERR_TRAVERSAL_BUDGET in the map's device status word and ends the
//     ray as a miss: a corrupt tree cannot hang the kernel.
#pragma once

#include "common.cuh"

namespace rmg {

constexpr float kWiden = 1.00000024f;  // 1 + 2^-22

// Slab arithmetic in packed pairs (fma.rn.f32x2, two IEEE single FMAs per
// instruction on sm_100 and later) when set; the results are the same either
// way.  Measured 2% faster on the 1M-triangle terrain (6,296 vs 6,173 Mrays/s).
#ifndef RMG_SLAB_F32X2
#define RMG_SLAB_F32X2 1
#endif

enum OriginKind { ORIGIN_POSE = 0, ORIGIN_SINGLE = 1, ORIGIN_TABLE = 2 };

struct Hit {
  float t;
  int tri;          // packed (leaf-order) triangle index, -1 = none
  uint32_t face;    // original face id
};

// Slab constants of one ray.  A plane at coordinate c is crossed at
// t = fma(c, 1/d, -o/d).  Rounding o/d leaves an absolute error of up to
// |o/d| * 2^-24 in every such t -- far more than a relative widening covers
// when the origin is far from the coordinate origin and d is small in that
// axis -- so each plane's addend carries an outward offset e = |o/d| * 2^-21
// (the near plane earlier, the far plane later).  The remaining error of a
// plane distance is below 2 ulp of t plus 2 |o/d| 2^-24 (rounded 1/d and
// o/d, rounded addend, one rounding of the fma), inside e plus the relative
// widening kWiden, so a box that the ray truly meets within (0, tfar] is never
// culled and the closest hit does not depend on the tree.
struct RayBox {
  float ix, iy, iz;     // 1/d (zero components replaced by +-1e20)
  float clx, cly, clz;  // addend of the lo plane: -o/d -+ e (minus when 1/d > 0)
  float chx, chy, chz;  // addend of the hi plane: -o/d +- e
#if RMG_SLAB_F32X2
  unsigned long long pix, piy, piz;     // (1/d, 1/d) per axis, packed for fma.rn.f32x2
  unsigned long long cx, cy, cz;        // (lo addend, hi addend) per axis
#endif
};

#if RMG_SLAB_F32X2
__device__ __forceinline__ unsigned long long pack2(float lo, float hi) {
  unsigned long long r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(lo), "f"(hi));
  return r;
}
#endif

__device__ __forceinline__ RayBox make_raybox(const V& o, const V& d) {
  RayBox r;
  r.ix = fabsf(d.x) > 1e-20f ? __frcp_rn(d.x) : copysignf(1e20f, d.x);
  r.iy = fabsf(d.y) > 1e-20f ? __frcp_rn(d.y) : copysignf(1e20f, d.y);
  r.iz = fabsf(d.z) > 1e-20f ? __frcp_rn(d.z) : copysignf(1e20f, d.z);
  // explicit roundings: the 8-wide walk's leaf test (leaf_exact) repeats these operations
  const float oix = __fmul_rn(o.x, r.ix), oiy = __fmul_rn(o.y, r.iy), oiz = __fmul_rn(o.z, r.iz);
  const float kE = 4.76837158e-7f;  // 2^-21
  const float ex = copysignf(fabsf(oix) * kE, r.ix), ey = copysignf(fabsf(oiy) * kE, r.iy),
              ez = copysignf(fabsf(oiz) * kE, r.iz);
  r.clx = __fsub_rn(-oix, ex); r.chx = __fadd_rn(-oix, ex);
  r.cly = __fsub_rn(-oiy, ey); r.chy = __fadd_rn(-oiy, ey);
  r.clz = __fsub_rn(-oiz, ez); r.chz = __fadd_rn(-oiz, ez);
#if RMG_SLAB_F32X2
  r.pix = pack2(r.ix, r.ix);
  r.piy = pack2(r.iy, r.iy);
  r.piz = pack2(r.iz, r.iz);
  r.cx = pack2(r.clx, r.chx);
  r.cy = pack2(r.cly, r.chy);
  r.cz = pack2(r.clz, r.chz);
#endif
  return r;
}

// Three-input float min/max (PTX ISA 8.8, sm_100 and later); same NaN rules as
// the two-input forms.
__device__ __forceinline__ float fmin3f(float a, float b, float c) {
  float d;
  asm("min.f32 %0, %1, %2, %3;" : "=f"(d) : "f"(a), "f"(b), "f"(c));
  return d;
}
__device__ __forceinline__ float fmax3f(float a, float b, float c) {
  float d;
  asm("max.f32 %0, %1, %2, %3;" : "=f"(d) : "f"(a), "f"(b), "f"(c));
  return d;
}

#if RMG_SLAB_F32X2
// (lo, hi) * (1/d, 1/d) + (lo addend, hi addend) for one axis in one packed
// FMA (fma.rn.f32x2, sm_100 and later: two IEEE single-precision FMAs).
__device__ __forceinline__ void slab_axis(float lo, float hi, unsigned long long inv, unsigned long long add,
                                          float& t0, float& t1) {
  unsigned long long r;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r) : "l"(pack2(lo, hi)), "l"(inv), "l"(add));
  asm("mov.b64 {%0, %1}, %2;" : "=f"(t0), "=f"(t1) : "l"(r));
}
#endif

// Slab test of one box; tmin includes the ray's tnear = 0.
__device__ __forceinline__ void slab(const RayBox& r, float lox, float hix, float loy, float hiy,
                                     float loz, float hiz, float& tmin, float& tmax) {
#if RMG_SLAB_F32X2
  float x0, x1, y0, y1, z0, z1;
  slab_axis(lox, hix, r.pix, r.cx, x0, x1);
  slab_axis(loy, hiy, r.piy, r.cy, y0, y1);
  slab_axis(loz, hiz, r.piz, r.cz, z0, z1);
#else
  const float x0 = fmaf(lox, r.ix, r.clx), x1 = fmaf(hix, r.ix, r.chx);
  const float y0 = fmaf(loy, r.iy, r.cly), y1 = fmaf(hiy, r.iy, r.chy);
  const float z0 = fmaf(loz, r.iz, r.clz), z1 = fmaf(hiz, r.iz, r.chz);
#endif
  tmin = fmax3f(fminf(x0, x1), fminf(y0, y1), fmaxf(fminf(z0, z1), 0.0f));
  tmax = fmin3f(fmaxf(x0, x1), fmaxf(y0, y1), fmaxf(z0, z1));
}

__device__ __forceinline__ bool visit(float tmin, float tmax, float best) {
  return tmin <= fminf(tmax, best) * kWiden;
}

__device__ __forceinline__ void test_tri(const DeviceMap& map, const RayW& rw, int k, Hit& h) {
  const Tri* tp = map.tris + k;
  const float4 p0 = __ldg(&tp->v0), p1 = __ldg(&tp->v1), p2 = __ldg(&tp->v2);
  float t;
  if (tri_hit(rw, p0, p1, p2, h.t, t)) {
    const uint32_t f = __float_as_uint(p0.w);
    if (t < h.t || f < h.face) { h.t = t; h.tri = k; h.face = f; }
  }
}

// The trail: one bit per internal level of the current path ("the other child
// of this level is still pending").  TB bits must exceed the tree's internal
// depth; the launcher picks 32, 64 or 128 from the depth the build measured.
template <int TB> struct Trail;

template <> struct Trail<32> {
  uint32_t v = 0;
  __device__ __forceinline__ void push(uint32_t bit) { v = (v << 1) | bit; }
  __device__ __forceinline__ bool empty() const { return v == 0; }
  __device__ __forceinline__ int ctz() const { return __ffs((int)v) - 1; }
  __device__ __forceinline__ void shr(int k) { v >>= k; }
  __device__ __forceinline__ void clear_low() { v ^= 1u; }
};

template <> struct Trail<64> {
  uint64_t v = 0;
  __device__ __forceinline__ void push(uint32_t bit) { v = (v << 1) | bit; }
  __device__ __forceinline__ bool empty() const { return v == 0; }
  __device__ __forceinline__ int ctz() const { return __ffsll((long long)v) - 1; }
  __device__ __forceinline__ void shr(int k) { v >>= k; }
  __device__ __forceinline__ void clear_low() { v ^= 1ull; }
};

// TB == 0: no trail at all; the traversal keeps every pending far child on a
// full stack (used when the tree's internal depth is below the stack size).
template <> struct Trail<0> {
  __device__ __forceinline__ void push(uint32_t) {}
};

template <> struct Trail<128> {
  uint64_t lo = 0, hi = 0;
  __device__ __forceinline__ void push(uint32_t bit) {
    hi = (hi << 1) | (lo >> 63);
    lo = (lo << 1) | bit;
  }
  __device__ __forceinline__ bool empty() const { return (lo | hi) == 0; }
  __device__ __forceinline__ int ctz() const {
    return lo ? (__ffsll((long long)lo) - 1) : (64 + __ffsll((long long)hi) - 1);
  }
  __device__ __forceinline__ void shr(int k) {
    if (k >= 64) { lo = hi >> (k - 64); hi = 0; }
    else if (k > 0) { lo = (lo >> k) | (hi << (64 - k)); hi >>= k; }
  }
  __device__ __forceinline__ void clear_low() { lo ^= 1ull; }
};

inline int trail_bits_for_depth(unsigned depth) { return depth <= 32 ? 32 : (depth <= 64 ? 64 : 128); }

// One ray's traversal state.  step() performs one node visit and, when the
// visit does not descend, the backtrack to the next pending node; it returns
// true once the ray is finished (or out of budget, which sets `over`).  The
// classic kernel loops step() to completion; the refill kernel interleaves the
// steps of rays that start at different times.  Both run this same code, so
// their results are identical.
// The circular short stack lives in its own object (dynamically indexed arrays
// go to local memory; keeping them apart lets the scalar state stay in registers).
template <int SS>
struct ShortStack {
  int node[SS > 0 ? SS : 1];
  float t[SS > 0 ? SS : 1];
};

template <int SS, int TB>
struct RayTrav {
  RayW rw;
  RayBox rb;
  Hit h;
  float tfar;
  int node;
  Trail<TB> trail;
  int sp, top;
  unsigned steps;
  bool over;

  // Returns false when there is nothing to traverse (empty map).
  __device__ __forceinline__ bool init(const DeviceMap& map, const V& o, const V& d, float tfar_) {
    tfar = tfar_;
    h.t = tfar_;
    h.tri = -1;
    h.face = 0xffffffffu;
    over = false;
    steps = 0;
    sp = 0;
    top = 0;
    trail = Trail<TB>();
    node = map.root;
    if (map.root < 0) return false;
    rw = make_rayw(o, d);
    rb = make_raybox(o, d);
    return true;
  }

  __device__ __forceinline__ bool fail_budget() {
    over = true;
    h.tri = -1;
    h.t = tfar;
    h.face = 0xffffffffu;
    return true;
  }

  __device__ __forceinline__ bool step(const DeviceMap& map, unsigned budget, ShortStack<SS>& stack) {
    if (++steps > budget) return fail_budget();
    const Node* np = map.nodes + node;
    const float4 a = __ldg(&np->a);
    const float4 b = __ldg(&np->b);
    const float4 c = __ldg(&np->c);
    const int4 ln = __ldg(&np->d);
    float tminL, tmaxL, tminR, tmaxR;
    slab(rb, a.x, a.y, a.z, a.w, c.x, c.y, tminL, tmaxL);
    slab(rb, b.x, b.y, b.z, b.w, c.z, c.w, tminR, tmaxR);
    bool hitL = visit(tminL, tmaxL, h.t);
    bool hitR = visit(tminR, tmaxR, h.t);
    // Leaf children are tested on the spot; only then can the closest hit have
    // moved, so the internal children are re-culled only on that path (+2-3%
    // against re-culling after every visit).
    const bool leafL = hitL && ln.x < 0, leafR = hitR && ln.y < 0;
    if (leafL || leafR) {
      if (leafL) test_tri(map, rw, ~ln.x, h);
      if (leafR) test_tri(map, rw, ~ln.y, h);
      hitL = hitL && !leafL && tminL <= h.t * kWiden;
      hitR = hitR && !leafR && tminR <= h.t * kWiden;
    }
    if (hitL && hitR) {
      const bool lf = tminL <= tminR;
      if constexpr (TB == 0) {
        if (sp >= SS) return fail_budget();  // only a corrupt tree gets this deep
        stack.node[sp] = lf ? ln.y : ln.x;
        stack.t[sp] = lf ? tminR : tminL;
        ++sp;
      } else if (SS > 0) {
        top = (top + 1) & (SS - 1);
        stack.node[top] = lf ? ln.y : ln.x;
        stack.t[top] = lf ? tminR : tminL;
        sp = sp < SS ? sp + 1 : SS;
      }
      trail.push(1u);
      node = lf ? ln.x : ln.y;
      return false;
    }
    if (hitL || hitR) {
      trail.push(0u);
      node = hitL ? ln.x : ln.y;
      return false;
    }
    if constexpr (TB == 0) {
      // ---- full stack: pop the nearest pending child that survives the cull ----
      while (sp > 0) {
        --sp;
        node = stack.node[sp];
        if (stack.t[sp] <= h.t * kWiden) return false;
      }
      return true;
    }
    // ---- backtrack to the nearest pending level ----
    if constexpr (TB != 0) {
    while (!trail.empty()) {
      const int k = trail.ctz();
      trail.shr(k);
      trail.clear_low();
      if (SS > 0 && sp > 0) {
        const int cand = stack.node[top];
        const float ct = stack.t[top];
        top = (top - 1) & (SS > 0 ? SS - 1 : 0);
        --sp;
        node = cand;
        if (ct <= h.t * kWiden) return false;
      } else {
        // The trail never holds more levels than the path below the root, so
        // a climb that reaches the root's parent (-1) means a corrupt tree.
        for (int j = 0; j < k && node >= 0; ++j) node = __ldg(&map.nodes[node].d.z);
        steps += (unsigned)k;
        const int p = node >= 0 ? __ldg(&map.nodes[node].d.z) : -1;
        if (steps > budget || p < 0) return fail_budget();
        const Node* pp = map.nodes + p;
        const int4 pl = __ldg(&pp->d);
        float tmin, tmax;
        int sib;
        if (pl.x == node) {
          sib = pl.y;
          const float4 bb = __ldg(&pp->b);
          const float4 cc = __ldg(&pp->c);
          slab(rb, bb.x, bb.y, bb.z, bb.w, cc.z, cc.w, tmin, tmax);
        } else {
          sib = pl.x;
          const float4 aa = __ldg(&pp->a);
          const float4 cc = __ldg(&pp->c);
          slab(rb, aa.x, aa.y, aa.z, aa.w, cc.x, cc.y, tmin, tmax);
        }
        node = sib;
        if (visit(tmin, tmax, h.t)) return false;
      }
    }
    }
    return true;
  }
};

// Full-stack size of the binary walks (tree depth <= 32).
constexpr int kFullStack = 32;

// Trail tag of the 4-wide traversal (trace_ray4); the other tags are trail widths.
constexpr int kWideTB = 4;
// Stack of the 4-wide traversal: a visit pushes at most three children, so a
// wide tree of at most 21 levels (the launcher checks the built depth) never
// holds more than 63 pending entries; a deeper push (a corrupt tree) ends in
// the budget error.
constexpr int kStack4 = 64;

__device__ __forceinline__ void cswap(float& ta, int& ca, float& tb, int& cb) {
  const bool s = tb < ta;
  const float t = s ? tb : ta;
  const int c = s ? cb : ca;
  tb = s ? ta : tb;
  cb = s ? ca : cb;
  ta = t;
  ca = c;
}

// Closest hit through the 4-wide tree.  Same boxes, same culling rule
// (tmin <= min(tmax, best) * (1 + 2^-22)) and the same triangle test and tie
// rule as the binary walk, so the hit (t, face) is identical; only the order
// of visits differs.  Leaf children are tested as soon as their box is hit;
// internal children are visited nearest first (a 4-element sorting network on
// the entry distances), the others pushed far to near.
__device__ __forceinline__ void trace_ray4(const DeviceMap& map, const V& o, const V& d, float tfar,
                                           unsigned budget, Hit& h, bool& over_budget) {
  h.t = tfar;
  h.tri = -1;
  h.face = 0xffffffffu;
  if (map.root < 0) return;
  const RayW rw = make_rayw(o, d);
  const RayBox rb = make_raybox(o, d);
  int stk_node[kStack4];
  float stk_t[kStack4];
  int sp = 0;
  int node = 0;
  unsigned steps = 0;
  while (true) {
    if (++steps > budget) { over_budget = true; break; }
    const Node4* np = map.nodes4 + node;
    const float4 lox = __ldg(&np->lox), hix = __ldg(&np->hix), loy = __ldg(&np->loy), hiy = __ldg(&np->hiy);
    const float4 loz = __ldg(&np->loz), hiz = __ldg(&np->hiz);
    const int4 ch = __ldg(&np->child);
    float t0, t1, t2, t3, m0, m1, m2, m3;
    slab(rb, lox.x, hix.x, loy.x, hiy.x, loz.x, hiz.x, t0, m0);
    slab(rb, lox.y, hix.y, loy.y, hiy.y, loz.y, hiz.y, t1, m1);
    slab(rb, lox.z, hix.z, loy.z, hiy.z, loz.z, hiz.z, t2, m2);
    slab(rb, lox.w, hix.w, loy.w, hiy.w, loz.w, hiz.w, t3, m3);
    bool v0 = visit(t0, m0, h.t), v1 = visit(t1, m1, h.t), v2 = visit(t2, m2, h.t), v3 = visit(t3, m3, h.t);
    if (v0 && ch.x < 0) { if (ch.x != kEmpty4) test_tri(map, rw, ~ch.x, h); v0 = false; }
    if (v1 && ch.y < 0) { if (ch.y != kEmpty4) test_tri(map, rw, ~ch.y, h); v1 = false; }
    if (v2 && ch.z < 0) { if (ch.z != kEmpty4) test_tri(map, rw, ~ch.z, h); v2 = false; }
    if (v3 && ch.w < 0) { if (ch.w != kEmpty4) test_tri(map, rw, ~ch.w, h); v3 = false; }
    const float cull = h.t * kWiden;
    const float inf = __int_as_float(0x7f800000);
    float k0 = v0 && t0 <= cull ? t0 : inf, k1 = v1 && t1 <= cull ? t1 : inf;
    float k2 = v2 && t2 <= cull ? t2 : inf, k3 = v3 && t3 <= cull ? t3 : inf;
    int c0 = ch.x, c1 = ch.y, c2 = ch.z, c3 = ch.w;
    cswap(k0, c0, k1, c1);
    cswap(k2, c2, k3, c3);
    cswap(k0, c0, k2, c2);
    cswap(k1, c1, k3, c3);
    cswap(k1, c1, k2, c2);
    if (k0 < inf) {
      if (sp + 3 > kStack4) { over_budget = true; break; }  // only a corrupt tree gets this deep
      if (k3 < inf) { stk_node[sp] = c3; stk_t[sp] = k3; ++sp; }
      if (k2 < inf) { stk_node[sp] = c2; stk_t[sp] = k2; ++sp; }
      if (k1 < inf) { stk_node[sp] = c1; stk_t[sp] = k1; ++sp; }
      node = c0;
      continue;
    }
    bool found = false;
    while (sp > 0) {
      --sp;
      if (stk_t[sp] <= h.t * kWiden) { node = stk_node[sp]; found = true; break; }
    }
    if (!found) break;
  }
  if (over_budget) {
    h.tri = -1;
    h.t = tfar;
    h.face = 0xffffffffu;
  }
}

// Trail tag of the 8-wide walk (trace_ray8).
constexpr int kWide8TB = 8;
// Stack of the 8-wide walk: one entry (a node's pending children) per level,
// so trees of up to kStack8 + 1 levels (the launcher checks the built depth);
// a deeper push (a corrupt tree) ends in the budget error.
constexpr int kStack8 = 24;

// One quantized plane offset as a float: 2^23 + q exactly (the byte q = byte
// k of w in the mantissa of 2^23), one byte permute instead of a conversion.
__device__ __forceinline__ float q_magic(uint32_t w, uint32_t k) {
  return __uint_as_float(__byte_perm(w, 0x4B000000u, 0x7440u | k));
}

// Slot order -> key order: bit s of m moves to bit s ^ oct.
__device__ __forceinline__ uint32_t octant_order(uint32_t m, uint32_t oct) {
  if (oct & 1u) m = ((m & 0x55u) << 1) | ((m >> 1) & 0x55u);
  if (oct & 2u) m = ((m & 0x33u) << 2) | ((m >> 2) & 0x33u);
  if (oct & 4u) m = ((m & 0x0Fu) << 4) | ((m >> 4) & 0x0Fu);
  return m;
}

// Near and far plane addends of one axis of an 8-wide node, for the plane
// distance t = fma(2^23 + q, s, addend) with s = 2^e / d:
//   c = fma(p, 1/d, -o/d) is the distance of the grid origin plane, and the
//   addend is c -+ eps - 2^23 s.  eps bounds every rounding outward: -o/d and
//   c carry |o/d| 2^-24 and |c| 2^-24, forming the addend another |c| 2^-24 +
//   |s| / 2 (the 2^23 s term), the fma one relative rounding of t; eps =
//   (|o/d| + 3|c|) 2^-21 + 2.0625 |s| covers them with the relative widening
//   kWiden of the far plane (|t| <= |c| + 256 |s|) folded in.
__device__ __forceinline__ void wide8_axis(float p, uint32_t ebyte, float inv, float noi, float eo,
                                           float& s, float& an, float& af) {
  s = __int_as_float(__float_as_int(inv) + (((int)ebyte - 127) << 23));  // inv * 2^e, exact
  const float c = fmaf(p, inv, noi);
  const float as = fabsf(s);
  const float eps = fmaf(as, 2.0625f, fmaf(fabsf(c), 1.430511474609375e-6f, eo));  // 3 * 2^-21
  an = fmaf(-8388608.0f, s, c - eps);
  af = fmaf(-8388608.0f, s, c + eps);
}

// A leaf of the 8-wide tree: the triangle's exact box (the min / max of its
// vertices, as the binary builders store it) tested with the binary walk's
// slab arithmetic (make_raybox / slab / visit, operation for operation), then
// the triangle.  The quantized boxes alone would be conservative, but the
// binary walk is not conservative everywhere: a ray lying exactly in a box
// face (a zero direction component with the origin on that plane) enters the
// box or not by the sign of the zero (1/d = +-1e20), as in Embree.  Testing a
// leaf only when the binary walk's own test admits it keeps the closest hit of
// both walks identical in that case too.
__device__ __forceinline__ void leaf_exact(const DeviceMap& map, const RayW& rw, int k, float ix, float iy, float iz,
                                           float nx, float ny, float nz, float ex, float ey, float ez, Hit& h) {
  const Tri* tp = map.tris + k;
  const float4 p0 = __ldg(&tp->v0), p1 = __ldg(&tp->v1), p2 = __ldg(&tp->v2);
  const float sx = copysignf(ex, ix), sy = copysignf(ey, iy), sz = copysignf(ez, iz);
  const float x0 = __fmaf_rn(fminf(fminf(p0.x, p1.x), p2.x), ix, __fsub_rn(nx, sx));
  const float x1 = __fmaf_rn(fmaxf(fmaxf(p0.x, p1.x), p2.x), ix, __fadd_rn(nx, sx));
  const float y0 = __fmaf_rn(fminf(fminf(p0.y, p1.y), p2.y), iy, __fsub_rn(ny, sy));
  const float y1 = __fmaf_rn(fmaxf(fmaxf(p0.y, p1.y), p2.y), iy, __fadd_rn(ny, sy));
  const float z0 = __fmaf_rn(fminf(fminf(p0.z, p1.z), p2.z), iz, __fsub_rn(nz, sz));
  const float z1 = __fmaf_rn(fmaxf(fmaxf(p0.z, p1.z), p2.z), iz, __fadd_rn(nz, sz));
  const float tmin = fmax3f(fminf(x0, x1), fminf(y0, y1), fmaxf(fminf(z0, z1), 0.0f));
  const float tmax = fmin3f(fmaxf(x0, x1), fmaxf(y0, y1), fmaxf(z0, z1));
  if (!visit(tmin, tmax, h.t)) return;
  float t;
  if (tri_hit(rw, p0, p1, p2, h.t, t)) {
    const uint32_t f = __float_as_uint(p0.w);
    if (t < h.t || f < h.face) { h.t = t; h.tri = k; h.face = f; }
  }
}

// Closest hit through the 8-wide quantized tree (wide8.cu).  Every child box
// of a visited node is tested (uniform work for the warp), leaf children's
// triangles are intersected at once, and the internal children that the ray
// enters are visited in the order of the ray's octant (nearest slots first);
// a node's pending children wait on the stack as one entry (node base,
// remaining children, internal-slot mask).  The boxes are conservative and
// the triangle test and tie rule are those of the binary walk, so the hit
// (t, face) is identical; h.tri indexes map.tris, which the launcher points
// at the 8-wide tree's triangle copy.
__device__ __forceinline__ void trace_ray8(const DeviceMap& map, const V& o, const V& d, float tfar,
                                           unsigned budget, Hit& h, bool& over_budget) {
  h.t = tfar;
  h.tri = -1;
  h.face = 0xffffffffu;
  if (map.root < 0) return;
  const RayW rw = make_rayw(o, d);
  const float ix = fabsf(d.x) > 1e-20f ? __frcp_rn(d.x) : copysignf(1e20f, d.x);
  const float iy = fabsf(d.y) > 1e-20f ? __frcp_rn(d.y) : copysignf(1e20f, d.y);
  const float iz = fabsf(d.z) > 1e-20f ? __frcp_rn(d.z) : copysignf(1e20f, d.z);
  const float nx = -__fmul_rn(o.x, ix), ny = -__fmul_rn(o.y, iy), nz = -__fmul_rn(o.z, iz);
  const float kE = 4.76837158e-7f;  // 2^-21
  const float ex = fabsf(nx) * kE, ey = fabsf(ny) * kE, ez = fabsf(nz) * kE;
  const uint32_t oct = (ix < 0.f ? 1u : 0u) | (iy < 0.f ? 2u : 0u) | (iz < 0.f ? 4u : 0u);
  uint2 stack[kStack8];
  int sp = 0;
  uint32_t cur_base = 0, cur_bits = 0;  // pending children in key order (bits 0-7) | internal slots << 8
  int node = 0;
  unsigned steps = 0;
  for (;;) {
    if (++steps > budget) { over_budget = true; break; }
    const Node8* np = map.nodes8 + node;
    const float4 h0 = __ldg(&np->h0);
    const uint4 h1 = __ldg(&np->h1);
    const uint4 qx = __ldg(&np->qx), qy = __ldg(&np->qy), qz = __ldg(&np->qz);
    const uint32_t meta = __float_as_uint(h0.w);
    float sx, sy, sz, anx, afx, any, afy, anz, afz;
    wide8_axis(h0.x, meta & 0xffu, ix, nx, ex, sx, anx, afx);
    wide8_axis(h0.y, (meta >> 8) & 0xffu, iy, ny, ey, sy, any, afy);
    wide8_axis(h0.z, (meta >> 16) & 0xffu, iz, nz, ez, sz, anz, afz);
    // near / far plane bytes of each axis by the ray's direction
    const uint32_t nx0 = ix >= 0.f ? qx.x : qx.z, nx1 = ix >= 0.f ? qx.y : qx.w;
    const uint32_t fx0 = ix >= 0.f ? qx.z : qx.x, fx1 = ix >= 0.f ? qx.w : qx.y;
    const uint32_t ny0 = iy >= 0.f ? qy.x : qy.z, ny1 = iy >= 0.f ? qy.y : qy.w;
    const uint32_t fy0 = iy >= 0.f ? qy.z : qy.x, fy1 = iy >= 0.f ? qy.w : qy.y;
    const uint32_t nz0 = iz >= 0.f ? qz.x : qz.z, nz1 = iz >= 0.f ? qz.y : qz.w;
    const uint32_t fz0 = iz >= 0.f ? qz.z : qz.x, fz1 = iz >= 0.f ? qz.w : qz.y;
    const float cull = h.t * kWiden;
    uint32_t hit = 0;
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      const uint32_t b = (uint32_t)(k & 3);
      const float tnx = fmaf(q_magic(k < 4 ? nx0 : nx1, b), sx, anx);
      const float tfx = fmaf(q_magic(k < 4 ? fx0 : fx1, b), sx, afx);
      const float tny = fmaf(q_magic(k < 4 ? ny0 : ny1, b), sy, any);
      const float tfy = fmaf(q_magic(k < 4 ? fy0 : fy1, b), sy, afy);
      const float tnz = fmaf(q_magic(k < 4 ? nz0 : nz1, b), sz, anz);
      const float tfz = fmaf(q_magic(k < 4 ? fz0 : fz1, b), sz, afz);
      const float tmin = fmax3f(tnx, tny, fmaxf(tnz, 0.0f));
      const float tmax = fmin3f(tfx, tfy, fminf(tfz, cull));
      if (tmin <= tmax) hit |= 1u << k;
    }
    const uint32_t valid = h1.z, imask = meta >> 24;
    hit &= valid;
    // leaf children: the binary walk's own box test on the triangle's exact
    // bounds, then the triangle (see leaf_exact)
    const uint32_t leaves = valid & ~imask;
    uint32_t lh = hit & ~imask;
    while (lh) {
      const uint32_t s = (uint32_t)(__ffs((int)lh) - 1);
      lh &= lh - 1u;
      leaf_exact(map, rw, (int)(h1.y + __popc(leaves & ((1u << s) - 1u))), ix, iy, iz, nx, ny, nz, ex, ey, ez, h);
    }
    // internal children: nearest-octant slots first
    const uint32_t km = octant_order(hit & imask, oct);
    if (km) {
      if (cur_bits & 0xffu) {
        if (sp >= kStack8) { over_budget = true; break; }  // only a corrupt tree gets this deep
        stack[sp++] = make_uint2(cur_base, cur_bits);
      }
      cur_base = h1.x;
      cur_bits = km | (imask << 8);
    }
    while (!(cur_bits & 0xffu) && sp > 0) {
      const uint2 e = stack[--sp];
      cur_base = e.x;
      cur_bits = e.y;
    }
    if (!(cur_bits & 0xffu)) break;
    const uint32_t k = (uint32_t)(__ffs((int)(cur_bits & 0xffu)) - 1);
    cur_bits &= ~(1u << k);
    const uint32_t s = k ^ oct;
    node = (int)(cur_base + __popc((cur_bits >> 8) & ((1u << s) - 1u)));
  }
  if (over_budget) {
    h.tri = -1;
    h.t = tfar;
    h.face = 0xffffffffu;
  }
}

// Trail tag of the warp-synchronous packet walk (trace_ray_packet).
constexpr int kPacketTB = 1;

// Warp-synchronous walk of the binary tree for the 32 rays of one tile: the
// warp moves through the tree together and visits a node when any lane's ray
// needs it (__any_sync), so every node is loaded once per warp (a broadcast)
// and all branching is uniform; each lane keeps its own culling distance and
// closest hit, so every ray's result is the same as in its own walk.  The
// nearer child goes first when more lanes enter it first.  Lanes without a
// ray (ragged tiles) take part with no culling distance at all.  All 32 lanes
// must call this together.  Pending nodes: one index per level for the warp
// (held by every lane), each lane's own entry distance (+inf where its ray did
// not enter the node).  It pays when a tile's rays share most of their paths
// (measured: 2,412-triangle room with VLP-16 +33%, 1M-triangle terrain with a
// 640 x 480 camera +6%) and loses where they part early (the terrain with the
// 128 x 1024 spherical sensor, whose near-horizon rows reach very different
// ranges: -9%).  A variant that let the lanes go their own ways once few of
// them shared the path was slower everywhere (lanes never regroup).
__device__ __forceinline__ void trace_ray_packet(const DeviceMap& map, const V& o, const V& d, float tfar,
                                                 bool active, unsigned budget, Hit& h, bool& over_budget) {
  h.t = active ? tfar : -1.0f;
  h.tri = -1;
  h.face = 0xffffffffu;
  if (map.root < 0) {
    h.t = tfar;
    return;
  }
  const RayW rw = make_rayw(o, d);
  const RayBox rb = make_raybox(o, d);
  int stk_node[kFullStack];
  float stk_t[kFullStack];
  int sp = 0;
  int node = map.root;
  unsigned steps = 0;
  const float inf = __int_as_float(0x7f800000);
  while (true) {
    if (++steps > budget) { over_budget = true; break; }
    const Node* np = map.nodes + node;
    const float4 a = __ldg(&np->a);
    const float4 b = __ldg(&np->b);
    const float4 c = __ldg(&np->c);
    const int4 ln = __ldg(&np->d);
    float tminL, tmaxL, tminR, tmaxR;
    slab(rb, a.x, a.y, a.z, a.w, c.x, c.y, tminL, tmaxL);
    slab(rb, b.x, b.y, b.z, b.w, c.z, c.w, tminR, tmaxR);
    bool hitL = visit(tminL, tmaxL, h.t);
    bool hitR = visit(tminR, tmaxR, h.t);
    if (ln.x < 0 || ln.y < 0) {  // uniform: the node is the same for the whole warp
      if (ln.x < 0) {
        if (hitL) test_tri(map, rw, ~ln.x, h);
        hitL = false;
      }
      if (ln.y < 0) {
        if (hitR) test_tri(map, rw, ~ln.y, h);
        hitR = false;
      }
      const float cull = h.t * kWiden;  // only a triangle test can have moved the closest hit
      hitL = hitL && tminL <= cull;
      hitR = hitR && tminR <= cull;
    }
    const bool anyL = __any_sync(0xffffffffu, hitL), anyR = __any_sync(0xffffffffu, hitR);
    if (anyL && anyR) {
      if (sp >= kFullStack) { over_budget = true; break; }  // only a corrupt tree gets this deep
      const bool prefL = hitL && (!hitR || tminL <= tminR);
      const bool prefR = hitR && !prefL;
      const bool leftFirst = __popc(__ballot_sync(0xffffffffu, prefL)) >= __popc(__ballot_sync(0xffffffffu, prefR));
      stk_node[sp] = leftFirst ? ln.y : ln.x;
      stk_t[sp] = leftFirst ? (hitR ? tminR : inf) : (hitL ? tminL : inf);
      ++sp;
      node = leftFirst ? ln.x : ln.y;
      continue;
    }
    if (anyL || anyR) {
      node = anyL ? ln.x : ln.y;
      continue;
    }
    bool found = false;
    while (sp > 0) {
      --sp;
      const bool want = stk_t[sp] <= h.t * kWiden;
      if (__any_sync(0xffffffffu, want)) { node = stk_node[sp]; found = true; break; }
    }
    if (!found) break;
  }
  if (!active) h.t = tfar;
  if (over_budget) {
    h.tri = -1;
    h.t = tfar;
    h.face = 0xffffffffu;
  }
}

template <int SS, int TB>
__device__ __forceinline__ void trace_ray(const DeviceMap& map, const V& o, const V& d, float tfar,
                                          unsigned budget, Hit& h, bool& over_budget) {
  if constexpr (TB == kWideTB) {
    trace_ray4(map, o, d, tfar, budget, h, over_budget);
  } else if constexpr (TB == kWide8TB) {
    trace_ray8(map, o, d, tfar, budget, h, over_budget);
  } else {
    RayTrav<SS, TB> r;
    ShortStack<SS> stack;
    if (r.init(map, o, d, tfar)) {
      while (!r.step(map, budget, stack)) {
      }
    }
    h = r.h;
    if (r.over) over_budget = true;
  }
}

struct TraceParams {
  DeviceMap map;
  SensorDev sen;
  Tf Tsb;
  const rmg_transform* Tbm;
  uint32_t n_poses;
  rmg_outputs out;
  uint32_t tile_w_log2;
  uint32_t tile_h;
  uint32_t tiles_x;
  uint32_t tiles_per_pose;
  uint64_t n_tiles;
  unsigned budget;
  int trail_bits;
  int full_stack;  // internal depth < kFullStack: the traversal may keep every pending child on a stack
  int wide;        // walk the 4-wide tree (map.nodes4)
  int wide8;       // walk the 8-wide quantized tree (map.nodes8; map.tris is then its triangle copy)
  int packet;      // warp-synchronous packet walk of the binary tree
};


// Hit point in the sensor frame: dir_s * t (+ orig_s for per-ray origins),
// SphereSimulatorEmbree.tcc:127-133 / O1DnSimulatorEmbree.tcc:132.
template <int OK>
__device__ __forceinline__ V hit_point(const V& dir_s, const V& orig_s, float t) {
  V p{mul(dir_s.x, t), mul(dir_s.y, t), mul(dir_s.z, t)};
  if (OK != ORIGIN_POSE) { p.x = add(p.x, orig_s.x); p.y = add(p.y, orig_s.y); p.z = add(p.z, orig_s.z); }
  return p;
}

// Unit geometric normal e1 x e2 of a packed triangle in its mesh frame
// (EmbreeMesh.cpp:275-295: Embree's Ng, normalised).
__device__ __forceinline__ V face_normal_unit(const Tri* tp) {
  const float4 p0 = __ldg(&tp->v0), p1 = __ldg(&tp->v1), p2 = __ldg(&tp->v2);
  const V e1{sub(p1.x, p0.x), sub(p1.y, p0.y), sub(p1.z, p0.z)};
  const V e2{sub(p2.x, p0.x), sub(p2.y, p0.y), sub(p2.z, p0.z)};
  const V n{sub(mul(e1.y, e2.z), mul(e1.z, e2.y)), sub(mul(e1.z, e2.x), mul(e1.x, e2.z)),
            sub(mul(e1.x, e2.y), mul(e1.y, e2.x))};
  const float len = __fsqrt_rn(add(add(mul(n.x, n.x), mul(n.y, n.y)), mul(n.z, n.z)));
  return V{__fdiv_rn(n.x, len), __fdiv_rn(n.y, len), __fdiv_rn(n.z, len)};
}

// Map-frame normal -> sensor frame, flipped to face the ray, normalised
// (SphereSimulatorEmbree.tcc:136-156).
__device__ __forceinline__ V normal_to_sensor(const V& n_map, const V& dir_s, const Tf& Tsm) {
  V n = qrot(qconj(Tsm.R), n_map);
  const float dp = add(add(mul(dir_s.x, n.x), mul(dir_s.y, n.y)), mul(dir_s.z, n.z));
  if (dp > 0.0f) n = V{-n.x, -n.y, -n.z};
  const float len = __fsqrt_rn(add(add(mul(n.x, n.x), mul(n.y, n.y)), mul(n.z, n.z)));
  return V{__fdiv_rn(n.x, len), __fdiv_rn(n.y, len), __fdiv_rn(n.z, len)};
}

// Unit face normal of the hit triangle in the sensor frame, flipped to face
// the ray (EmbreeMesh.cpp:275-295 + SphereSimulatorEmbree.tcc:136-156).
__device__ __forceinline__ V hit_normal(const DeviceMap& map, const Hit& h, const V& dir_s, const Tf& Tsm) {
  return normal_to_sensor(face_normal_unit(map.tris + h.tri), dir_s, Tsm);
}

// Writes all requested attributes of one ray (SphereSimulatorEmbree.tcc:104-249).
template <int OK>
__device__ __forceinline__ void write_attributes(const TraceParams& P, uint64_t gid, const Hit& h,
                                                 const V& dir_s, const V& orig_s, const Tf& Tsm) {
  const rmg_outputs& out = P.out;
  const float rmin = P.sen.range_min, rmax = P.sen.range_max;
  if (h.tri >= 0) {
    const float t = h.t;
    if (out.hits) out.hits[gid] = t >= rmin ? 1 : 0;
    if (out.ranges) out.ranges[gid] = t;
    if (out.points) {
      const V p = hit_point<OK>(dir_s, orig_s, t);
      float* po = reinterpret_cast<float*>(out.points) + 3 * gid;
      po[0] = p.x; po[1] = p.y; po[2] = p.z;
    }
    if (out.normals) {
      const V n = hit_normal(P.map, h, dir_s, Tsm);
      float* no = reinterpret_cast<float*>(out.normals) + 3 * gid;
      no[0] = n.x; no[1] = n.y; no[2] = n.z;
    }
    if (out.face_ids) out.face_ids[gid] = h.face;
    if (out.geom_ids) out.geom_ids[gid] = 0u;
    if (out.object_ids) out.object_ids[gid] = 0u;
  } else {
    const float nanf_ = __int_as_float(0x7fc00000);
    if (out.hits) out.hits[gid] = 0;
    if (out.ranges) out.ranges[gid] = add(rmax, 1.0f);
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

// Ray setup of one (pose, row, col): SphereSimulatorEmbree.tcc:69-99.
template <int OK>
__device__ __forceinline__ void setup_ray(const SensorDev& sen, const Tf& Tsm, uint32_t loc, V& dir_s,
                                          V& orig_s, V& o, V& d) {
  dir_s = V{__ldg(sen.dirs + 3 * loc), __ldg(sen.dirs + 3 * loc + 1), __ldg(sen.dirs + 3 * loc + 2)};
  d = qrot(Tsm.R, dir_s);
  if (OK == ORIGIN_POSE) {
    orig_s = V{0.0f, 0.0f, 0.0f};
    o = Tsm.t;
  } else {
    if (OK == ORIGIN_SINGLE) orig_s = V{sen.orig.x, sen.orig.y, sen.orig.z};
    else orig_s = V{__ldg(sen.origs + 3 * loc), __ldg(sen.origs + 3 * loc + 1), __ldg(sen.origs + 3 * loc + 2)};
    const V r = qrot(Tsm.R, orig_s);
    o = V{add(r.x, Tsm.t.x), add(r.y, Tsm.t.y), add(r.z, Tsm.t.z)};
  }
}

// One warp = one tile of tile_h x tile_w rays of one pose.
// Minimum resident CTAs per SM requested from the compiler for k_trace: 5
// CTAs of 256 threads cap the kernel at 48 registers (a few bytes of spills
// to L1-cached local memory) and lift occupancy from 50% to 62.5%; measured
// 9% faster than the unconstrained 62-register build on the 1M-triangle
// terrain (6,179 vs 5,661 Mrays/s), while 6 CTAs (40 registers) spill more
// and lose again.
#ifndef RMG_TRACE_MIN_BLOCKS
#define RMG_TRACE_MIN_BLOCKS 5
#endif

// The 8-wide walk holds a node's twenty words and three axes of plane
// addends at once: it gets 64 registers (4 CTAs of 256 threads per SM).
#ifndef RMG_TRACE8_MIN_BLOCKS
#define RMG_TRACE8_MIN_BLOCKS 4
#endif

template <int TB>
constexpr int trace_min_blocks() { return TB == kWide8TB ? RMG_TRACE8_MIN_BLOCKS : RMG_TRACE_MIN_BLOCKS; }

template <int OK, int SS, int TB>
__global__ void __launch_bounds__(256, trace_min_blocks<TB>()) k_trace(const TraceParams P) {
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
  const bool inside = vid < H && hid < W;
  if (TB != kPacketTB && !inside) return;  // the packet walk needs every lane
  const uint32_t loc = inside ? visit_loc(P.sen, vid * W + hid) : 0;
  const uint64_t gid = (uint64_t)pose * W * H + loc;

  const Tf Tsm = tmul(load_tf(P.Tbm[pose]), P.Tsb);
  V dir_s, orig_s, o, d;
  setup_ray<OK>(P.sen, Tsm, loc, dir_s, orig_s, o, d);
  Hit h;
  bool over = false;
  if constexpr (TB == kPacketTB) {
    trace_ray_packet(P.map, o, d, P.sen.range_max, inside, P.budget, h, over);
    if (!inside) return;
  } else {
    trace_ray<SS, TB>(P.map, o, d, P.sen.range_max, P.budget, h, over);
  }
  if (over) atomicExch(P.map.status, (unsigned)RMG_ERR_TRAVERSAL_BUDGET);
  write_attributes<OK>(P, gid, h, dir_s, orig_s, Tsm);
}

}  // namespace rmg

namespace rmg {

// Persistent variant with lane refill ("dynamic ray fetch").  Rays are numbered
// tile-major (ray = tile * 32 + slot, the slot inside the tile_h x tile_w tile),
// so consecutive numbers are neighbouring rays of one pose.  A warp takes
// `chunk` tiles at a time from a global counter; whenever fewer than `refill`
// of its lanes still hold an unfinished ray, the idle lanes take the next ray
// numbers, ranked with __ballot_sync / __popc so each gets a distinct one.
// Every lane then performs one traversal step.  A finished lane writes its
// outputs and becomes idle.  Per ray the work is exactly that of k_trace.
template <int OK>
__device__ __forceinline__ bool ray_coords(const TraceParams& P, uint64_t ray, uint32_t& pose, uint32_t& loc,
                                           uint64_t& gid) {
  const uint64_t tile = ray >> 5;
  const uint32_t slot = (uint32_t)(ray & 31u);
  pose = (uint32_t)(tile / P.tiles_per_pose);
  const uint32_t r = (uint32_t)(tile - (uint64_t)pose * P.tiles_per_pose);
  const uint32_t ty = r / P.tiles_x, tx = r - ty * P.tiles_x;
  const uint32_t tile_w = 1u << P.tile_w_log2;
  const uint32_t vid = ty * P.tile_h + (slot >> P.tile_w_log2);
  const uint32_t hid = tx * tile_w + (slot & (tile_w - 1));
  const uint32_t W = P.sen.width, H = P.sen.height;
  if (vid >= H || hid >= W) return false;
  loc = visit_loc(P.sen, vid * W + hid);
  gid = (uint64_t)pose * W * H + loc;
  return true;
}

template <int OK, int SS, int TB>
__global__ void __launch_bounds__(256) k_trace_refill(const TraceParams P, unsigned long long* counter,
                                                      uint32_t chunk, uint32_t refill) {
  const uint32_t lane = threadIdx.x & 31;
  const uint32_t lt = (1u << lane) - 1u;
  refill = refill ? refill : 1u;  // at least one idle lane triggers a fetch: the loop always progresses
  chunk = chunk ? chunk : 1u;
  uint64_t next = 0, end = 0;
  bool exhausted = false, active = false;
  uint64_t my_ray = 0;
  RayTrav<SS, TB> R;
  ShortStack<SS> stack;
  for (;;) {
    const unsigned act = __ballot_sync(0xffffffffu, active);
    if (!exhausted && (uint32_t)__popc(act) < refill) {
      unsigned idle = ~act;
      while (idle) {
        if (next >= end) {
          unsigned long long base = 0;
          if (lane == 0) base = atomicAdd(counter, (unsigned long long)chunk);
          base = __shfl_sync(0xffffffffu, base, 0);
          if (base >= P.n_tiles) { exhausted = true; break; }
          next = base * 32ull;
          end = min((uint64_t)base + chunk, P.n_tiles) * 32ull;
        }
        const uint32_t n_idle = (uint32_t)__popc(idle);
        const uint32_t take = (uint32_t)min((uint64_t)n_idle, end - next);
        const uint32_t rank = (uint32_t)__popc(idle & lt);
        const bool mine = ((idle >> lane) & 1u) && rank < take;
        if (mine) {
          my_ray = next + rank;
          uint32_t pose, loc;
          uint64_t gid;
          if (ray_coords<OK>(P, my_ray, pose, loc, gid)) {
            const Tf Tsm = tmul(load_tf(P.Tbm[pose]), P.Tsb);
            V dir_s, orig_s, o, d;
            setup_ray<OK>(P.sen, Tsm, loc, dir_s, orig_s, o, d);
            active = true;
            if (!R.init(P.map, o, d, P.sen.range_max)) {  // empty map: finished at once
              write_attributes<OK>(P, gid, R.h, dir_s, orig_s, Tsm);
              active = false;
            }
          }
        }
        idle &= ~__ballot_sync(0xffffffffu, mine);
        next += take;
      }
    }
    if (__ballot_sync(0xffffffffu, active) == 0) {
      if (exhausted) break;
      continue;
    }
    if (active && R.step(P.map, P.budget, stack)) {
      if (R.over) atomicExch(P.map.status, (unsigned)RMG_ERR_TRAVERSAL_BUDGET);
      uint32_t pose, loc;
      uint64_t gid;
      ray_coords<OK>(P, my_ray, pose, loc, gid);
      const Tf Tsm = tmul(load_tf(P.Tbm[pose]), P.Tsb);
      V dir_s, orig_s, o, d;
      setup_ray<OK>(P.sen, Tsm, loc, dir_s, orig_s, o, d);
      write_attributes<OK>(P, gid, R.h, dir_s, orig_s, Tsm);
      active = false;
    }
  }
}

}  // namespace rmg
