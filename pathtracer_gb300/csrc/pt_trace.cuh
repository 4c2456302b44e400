// pt_trace.cuh -- closest-hit and any-hit traversal of the BVH4.
//
// The BVH4 is collapsed from the reference's own binary trees (top level
// BVHNode, bvh.hpp:46-102; per mesh MeshBVHNode, meshBVH.cpp:6-55), so the
// leaves hold exactly the reference's leaf primitive sets.  Traversal is
// near-to-far with a per-thread stack in SHARED memory (column per thread,
// bank-conflict free).  Primitive tests restate the reference arithmetic
// with rounded, never-fused operations so that hit distances match the
// reference bit for bit:
//   triangle  MeshBVHNode::hitTriangle  meshBVH.cpp:85-143
//   rectangle AARectangle<axis>::intersect  primitive.cpp:31-122
//   sphere    Sphere::intersect  primitive.hpp:124-170
// Acceptance is inclusive (t == tmax accepted), so of two equal-t primitives
// the later one tested wins, as in the reference leaf loop.
#pragma once
#include "pt_scene.cuh"

namespace pt {


struct HitRec {
  float t;
  int32_t prim;
  float u, v;
};

// Moller-Trumbore exactly as hitTriangle orders it.
__device__ __forceinline__ bool hit_triangle(const Item &it, V3 o, V3 d, float tmin, float tmax,
                                             float &t_out, float &u_out, float &v_out) {
  V3 p0 = v3(it.a[0], it.a[1], it.a[2]);
  V3 e1 = v3(it.b[0], it.b[1], it.b[2]);
  V3 e2 = v3(it.c[0], it.c[1], it.c[2]);
  V3 P = xcross(d, e2);
  float det = xdot(e1, P);
  if (fabsf(det) < 1e-8f) return false;
  float inv = xdiv(1.0f, det);
  V3 T = xsubv(o, p0);
  float u = xmul(xdot(T, P), inv);
  if (u < 0.f || u > 1.f) return false;
  V3 Q = xcross(T, e1);
  float v = xmul(xdot(d, Q), inv);
  if (v < 0.f || xadd(u, v) > 1.f) return false;
  float t = xmul(xdot(e2, Q), inv);
  if (t < tmin || t > tmax) return false;
  t_out = t;
  u_out = u;
  v_out = v;
  return true;
}

// AARectangle<axis>::intersect with the normalised direction dn.
__device__ __forceinline__ bool hit_quad(const Item &it, V3 o, V3 dn, float tmin, float tmax,
                                         float &t_out) {
  const int axis = (int)it.b[2];
  const float k = it.a[0], d0min = it.a[1], d0max = it.a[2];
  const float d1min = it.b[0], d1max = it.b[1];
  float oa, da, o0, d0_, o1, d1_;
  if (axis == 0) {
    oa = o.x; da = dn.x; o0 = o.y; d0_ = dn.y; o1 = o.z; d1_ = dn.z;
  } else if (axis == 1) {
    oa = o.y; da = dn.y; o0 = o.x; d0_ = dn.x; o1 = o.z; d1_ = dn.z;
  } else {
    oa = o.z; da = dn.z; o0 = o.x; d0_ = dn.x; o1 = o.y; d1_ = dn.y;
  }
  float t = xdiv(xsub(k, oa), da);
  if (t < tmin || t > tmax) return false;
  float a0 = xadd(o0, xmul(t, d0_));
  float a1 = xadd(o1, xmul(t, d1_));
  if (a0 < d0min || a0 > d0max || a1 < d1min || a1 > d1max) return false;
  t_out = t;
  return true;
}

// Sphere::intersect with the normalised direction dn.
__device__ __forceinline__ bool hit_sphere(const Item &it, V3 o, V3 dn, float tmin, float tmax,
                                           float &t_out) {
  V3 c = v3(it.a[0], it.a[1], it.a[2]);
  const float r = it.b[0];
  V3 oc = xsubv(o, c);
  float a = xdot(dn, dn);
  float b = xmul(2.f, xdot(dn, oc));
  float cc = xsub(xdot(oc, oc), xmul(r, r));
  float disc = xsub(xmul(b, b), xmul(xmul(4.f, a), cc));
  if (disc < 0.f) return false;
  float delta = xsqrt(disc);
  float t = xdiv(xsub(-b, delta), xmul(2.f, a));
  if (t < tmin || t > tmax) {
    t = xdiv(xadd(-b, delta), xmul(2.f, a));
    if (t < tmin || t > tmax) return false;
  }
  t_out = t;
  return true;
}

// Cubic Bezier point and derivative (primitives/bezier.hpp:10-36).
// Bezier point with every operation separately rounded (never fused), in
// bezier.hpp:10-18's order, so that curve hits round like the reference's.
__device__ __forceinline__ V3 bezier_point(const float4 *cp, float u) {
  const float u1 = xsub(1.0f, u);
  const float b0 = xmul(xmul(u1, u1), u1), b1 = xmul(xmul(xmul(3.0f, u), u1), u1);
  const float b2 = xmul(xmul(xmul(3.0f, u), u), u1), b3 = xmul(xmul(u, u), u);
  const float4 c0 = __ldg(cp), c1 = __ldg(cp + 1), c2 = __ldg(cp + 2), c3 = __ldg(cp + 3);
  auto comb = [&](float a0, float a1, float a2, float a3) {
    return xadd(xadd(xadd(xmul(a0, b0), xmul(a1, b1)), xmul(a2, b2)), xmul(a3, b3));
  };
  return v3(comb(c0.x, c1.x, c2.x, c3.x), comb(c0.y, c1.y, c2.y, c3.y), comb(c0.z, c1.z, c2.z, c3.z));
}
__device__ __forceinline__ V3 bezier_tangent(const float4 *cp, float u) {
  const float4 c0 = __ldg(cp), c1 = __ldg(cp + 1), c2 = __ldg(cp + 2), c3 = __ldg(cp + 3);
  const V3 d0 = 3.0f * (v3(c1.x, c1.y, c1.z) - v3(c0.x, c0.y, c0.z));
  const V3 d1 = 3.0f * (v3(c2.x, c2.y, c2.z) - v3(c1.x, c1.y, c1.z));
  const V3 d2 = 3.0f * (v3(c3.x, c3.y, c3.z) - v3(c2.x, c2.y, c2.z));
  const float u1 = 1.0f - u;
  return d0 * (u1 * u1) + d1 * (2.0f * u * u1) + d2 * (u * u);
}

// Curve::intersect (primitives/curve.hpp:48-129): the Bezier split into 8
// segments, each an infinite cylinder of the segment's mean radius cut at its
// ends; roots from gl::solveQuadratic (utility.hpp:112-124).  Returns the
// segment in u and the position along it in v (fraction of its length).
__device__ __forceinline__ bool hit_curve(const float4 *cp, V3 o, V3 d, float tmin, float tmax, float &t_out,
                                          float &u_out, float &v_out) {
  const int N = 8;
  float best = tmax;
  bool found = false;
  // Exact (never fused) arithmetic throughout: the cylinder quadratic is
  // ill-conditioned for grazing rays (C is a difference of near-equal
  // squares), so contracted multiply-adds would move t by ~1e-5 relative.
  auto axpy = [](V3 a, float k, V3 b) {  // a - k b
    return v3(xsub(a.x, xmul(k, b.x)), xsub(a.y, xmul(k, b.y)), xsub(a.z, xmul(k, b.z)));
  };
  // the end points are recomputed per segment (as the reference does) and
  // the widths reloaded, which keeps fewer values live in the traversal loop
#pragma unroll 1
  for (int i = 0; i < N; ++i) {
    const float u0 = float(i) / N, u1 = float(i + 1) / N;
    const V3 pa = bezier_point(cp, u0), pb = bezier_point(cp, u1);
    const float w0 = __ldg(cp).w, w1 = __ldg(cp + 1).w;
    const float r0 = xadd(w0, xmul(xsub(w1, w0), u0)), r1 = xadd(w0, xmul(xsub(w1, w0), u1));
    const float radius = xmul(0.5f, xadd(r0, r1));
    const V3 ab = xsubv(pb, pa);
    const float seg_len = xsqrt(xdot(ab, ab));
    const V3 axis = v3(xdiv(ab.x, seg_len), xdiv(ab.y, seg_len), xdiv(ab.z, seg_len));
    const V3 d_perp = axpy(d, xdot(d, axis), axis);
    const V3 delta = xsubv(o, pa);
    const V3 o_perp = axpy(delta, xdot(delta, axis), axis);
    const float A = xdot(d_perp, d_perp), B = xmul(2.0f, xdot(d_perp, o_perp));
    const float C = xsub(xdot(o_perp, o_perp), xmul(radius, radius));
    const float disc = xsub(xmul(B, B), xmul(xmul(4.0f, A), C));
    if (disc >= 0.f) {
      const float sq = xsqrt(disc);
      const float q = B < 0 ? xmul(-0.5f, xsub(B, sq)) : xmul(-0.5f, xadd(B, sq));
      float ra = xdiv(q, A), rb = xdiv(C, q);
      if (ra > rb) {
        const float tt = ra;
        ra = rb;
        rb = tt;
      }
      const int nr = ra == rb ? 1 : 2;
      for (int r = 0; r < nr; ++r) {
        const float t = r == 0 ? ra : rb;
        if (t < tmin || t > best) continue;
        const V3 hp = v3(xadd(o.x, xmul(t, d.x)), xadd(o.y, xmul(t, d.y)), xadd(o.z, xmul(t, d.z)));
        const float proj = xdot(xsubv(hp, pa), axis);
        if (proj < 0.0f || proj > seg_len) continue;
        best = t;
        u_out = (float)i;
        v_out = xdiv(proj, seg_len);
        found = true;
      }
    }
  }
  if (found) t_out = best;
  return found;
}

__device__ __forceinline__ Item load_item(const Item *items, int i) {
  const float4 *p = reinterpret_cast<const float4 *>(items + i);
  float4 a = __ldg(p), b = __ldg(p + 1), c = __ldg(p + 2);
  Item it;
  it.a[0] = a.x; it.a[1] = a.y; it.a[2] = a.z; it.a[3] = a.w;
  it.b[0] = b.x; it.b[1] = b.y; it.b[2] = b.z; it.b[3] = b.w;
  it.c[0] = c.x; it.c[1] = c.y; it.c[2] = c.z; it.c[3] = c.w;
  return it;
}

// Tests one leaf; for ANY returns true on the first hit in [tmin, tmax].
// Origin of a ray of time `time` in the frame of a primitive moving with
// velocity v: o - v * time (rounded, never fused).
__device__ __forceinline__ V3 moved_origin(const SceneView &S, uint32_t motion, V3 o, float time) {
  const float4 v = __ldg(S.motion + (motion - 1u));
  return v3(xsub(o.x, xmul(v.x, time)), xsub(o.y, xmul(v.y, time)), xsub(o.z, xmul(v.z, time)));
}

// Tests leaf item `idx` (a whole leaf is its items in order); for ANY
// returns true on a hit in [tmin, tmax], for closest hit records the hit and
// shrinks tmax (acceptance is inclusive: of equal-t items the later wins).
// CURVES = false compiles the curve test out (curve items then never hit):
// the closest-hit kernel of a scene without curves keeps 8 fewer registers.
template <bool ANY, bool CURVES = true>
__device__ __forceinline__ bool test_item(const SceneView &S, int idx, V3 o_w, V3 d, V3 dn, float tmin,
                                          float &tmax, HitRec &hit, float time) {
  Item it = load_item(S.items, idx);
  const int type = (int)f2u(it.b[3]);
  const uint32_t motion = f2u(it.c[3]);
  const V3 o = motion ? moved_origin(S, motion, o_w, time) : o_w;
  float t, u = 0.f, v = 0.f;
  bool h;
  if (type == ITEM_TRI)
    h = hit_triangle(it, o, d, tmin, tmax, t, u, v);
  else if (type == ITEM_QUAD)
    h = hit_quad(it, o, dn, tmin, tmax, t);
  else if (type == ITEM_SPHERE)
    h = hit_sphere(it, o, dn, tmin, tmax, t);
  else if (CURVES)
    h = hit_curve(S.curves + 4 * (size_t)f2u(it.a[0]), o, d, tmin, tmax, t, u, v);
  else
    h = false;
  if (h && !ANY) {
    tmax = t;
    hit.t = t;
    hit.prim = (int32_t)f2u(it.a[3]);
    hit.u = u;
    hit.v = v;
  }
  return h;
}

// Traversal state of one ray.  The walk is a sequence of node visits and
// leaf tests (trav_step) so that a persistent warp can refill lanes whose
// rays have finished while the others continue.
struct TravRay {
  V3 o, d, dn, inv, oi;  // o, oi: the current frame (world, or a moving object's)
  V3 ow;                 // world origin
  float tmin, tmax;
  int32_t ref;   // next reference: node (>= 0, PT_INST_BIT: entering a moving
                 // object), leaf (< 0), PT_FRAME_END or PT_REF_EMPTY
  int sp;        // stack depth
  int iters;
  float time;    // motion blur: the ray's time
  bool found;
  HitRec hit;
};

__device__ __forceinline__ bool ref_is_node(int32_t r) { return r >= 0 || r == PT_FRAME_END; }
__device__ __forceinline__ bool ref_is_leaf(int32_t r) { return r < 0 && r != PT_FRAME_END && r != PT_REF_EMPTY; }

// 1/d of one axis for the slab test.  An axis the ray does not move along
// (d = +-0, or |d| so small that 1/d overflows) gets +-1e20 with d's sign in
// place of +-inf: the slab test computes fmaf(plane, inv, -o * inv), and with
// an infinite inv a ray inside the slab gives inf - inf = NaN, which the
// min / max then drop -- that slab is not tested at all, and an axis-aligned
// ray walks every box its other slabs cross (the whole tree, ~10^5 steps for
// one ray).  With a finite inv the slab gives (-huge, +huge) inside it and an
// entry beyond any tmax outside.
__device__ __forceinline__ float slab_inv(float d) { return fabsf(d) > 1e-20f ? 1.f / d : copysignf(1e20f, d); }

__device__ __forceinline__ void trav_init(TravRay &R, V3 o, V3 d, float tmin, float tmax, float time = 0.f) {
  R.time = time;
  R.o = o;
  R.ow = o;
  R.d = d;
  R.dn = xnormalize(d);
  R.inv = v3(slab_inv(d.x), slab_inv(d.y), slab_inv(d.z));
  R.oi = v3(-o.x * R.inv.x, -o.y * R.inv.y, -o.z * R.inv.z);
  R.tmin = tmin;
  R.tmax = tmax;
  R.ref = 0;  // node 0 is the root (the host always emits at least one node)
  R.sp = 0;
  R.iters = 0;
  R.found = false;
  R.hit.t = FLT_MAX;
  R.hit.prim = -1;
  R.hit.u = R.hit.v = 0.f;
}

__device__ __forceinline__ int32_t trav_pop(TravRay &R, const int32_t *stack, int stride) {
  return R.sp == 0 ? PT_REF_EMPTY : stack[(--R.sp) * stride];
}

// One node visit (or frame change).  R.ref must satisfy ref_is_node; after it
// R.ref is the next reference (the nearest hit child for closest hit, the
// first hit child in node order for any hit, else the top of the stack).
// `stack` points at this thread's column of a shared array laid out
// [PT_STACK][stride].  Returns false on a stack overflow (error flag set).
template <bool ANY>
__device__ __forceinline__ bool trav_node(const SceneView &S, TravRay &R, int32_t *stack, int stride, int *err) {
  if (R.ref == PT_FRAME_END) {
    // leaving a moving object's subtree: back to the world frame
    R.o = R.ow;
    R.oi = v3(-R.o.x * R.inv.x, -R.o.y * R.inv.y, -R.o.z * R.inv.z);
    R.ref = trav_pop(R, stack, stride);
    return true;
  }
  if (R.ref & PT_INST_BIT) {
    // entering a moving object's subtree: the ray in the object's frame at
    // its time, until PT_FRAME_END comes off the stack
    R.ref &= ~PT_INST_BIT;
    if (R.sp + 1 > S.stack_entries) {
      *err = 1;
      return false;
    }
    stack[(R.sp++) * stride] = PT_FRAME_END;
    R.o = moved_origin(S, (uint32_t)__ldg(S.node_motion + R.ref), R.ow, R.time);
    R.oi = v3(-R.o.x * R.inv.x, -R.o.y * R.inv.y, -R.o.z * R.inv.z);
  }
  const float4 *np = reinterpret_cast<const float4 *>(S.nodes + R.ref);
  // The slab each child's entry and exit come from is fixed by the ray's
  // octant: with 1/d >= 0 along an axis the low plane is the near one
  // (fma is monotonic, so fmaf(lo, inv, oi) <= fmaf(hi, inv, oi) and the
  // min / max the general slab test takes per child equal these picks), so
  // the near and far rows are loaded by the sign of 1/d and no per-child
  // min / max is spent choosing them (measured: traversal stage -5.5 %).
  const int sx = signbit(R.inv.x) ? 1 : 0, sy = signbit(R.inv.y) ? 1 : 0, sz = signbit(R.inv.z) ? 1 : 0;
  float4 nx = __ldg(np + sx), fx = __ldg(np + (sx ^ 1)), ny = __ldg(np + 2 + sy), fy = __ldg(np + 2 + (sy ^ 1));
  float4 nz = __ldg(np + 4 + sz), fz = __ldg(np + 4 + (sz ^ 1));
  // the children's traversal references, ready made by the upload (node
  // index, leaf reference, or PT_REF_EMPTY for an empty slot)
  const int4 rf = __ldg(reinterpret_cast<const int4 *>(np + 7));
  const float nxa[4] = {nx.x, nx.y, nx.z, nx.w}, fxa[4] = {fx.x, fx.y, fx.z, fx.w};
  const float nya[4] = {ny.x, ny.y, ny.z, ny.w}, fya[4] = {fy.x, fy.y, fy.z, fy.w};
  const float nza[4] = {nz.x, nz.y, nz.z, nz.w}, fza[4] = {fz.x, fz.y, fz.z, fz.w};
  const int rfa[4] = {rf.x, rf.y, rf.z, rf.w};
  const V3 inv = R.inv, oi = R.oi;
  const float tmin = R.tmin, tmax = R.tmax;
  // entry distance per child (+inf when missed or empty), kept in registers;
  // closest-hit visits near to far (sorting network), any-hit in node order.
  float d0, d1, d2, d3;
  int32_t r0, r1, r2, r3;
#define PT_CHILD(c, dd, rr)                                                                          \
  {                                                                                                  \
    float tn = fmaxf(fmaxf(fmaf(nxa[c], inv.x, oi.x), fmaf(nya[c], inv.y, oi.y)),                  \
                     fmaxf(fmaf(nza[c], inv.z, oi.z), tmin));                                        \
    float tf = fminf(fminf(fmaf(fxa[c], inv.x, oi.x), fmaf(fya[c], inv.y, oi.y)),                  \
                     fminf(fmaf(fza[c], inv.z, oi.z), tmax));                                        \
    dd = (rfa[c] != PT_REF_EMPTY && tn <= tf) ? tn : INFINITY;                                      \
    rr = rfa[c];                                                                                     \
  }
  PT_CHILD(0, d0, r0)
  PT_CHILD(1, d1, r1)
  PT_CHILD(2, d2, r2)
  PT_CHILD(3, d3, r3)
#undef PT_CHILD
  if (!ANY) {
#define PT_CSWAP(da, ra, db, rb)   \
  if (db < da) {                   \
    float tt = da;                 \
    da = db;                       \
    db = tt;                       \
    int32_t tr = ra;               \
    ra = rb;                       \
    rb = tr;                       \
  }
    PT_CSWAP(d0, r0, d1, r1)
    PT_CSWAP(d2, r2, d3, r3)
    PT_CSWAP(d0, r0, d2, r2)
    PT_CSWAP(d1, r1, d3, r3)
    PT_CSWAP(d1, r1, d2, r2)
#undef PT_CSWAP
  }
  const int nh = (d0 < INFINITY) + (d1 < INFINITY) + (d2 < INFINITY) + (d3 < INFINITY);
  if (nh == 0) {
    R.ref = trav_pop(R, stack, stride);
    return true;
  }
  if (R.sp + nh - 1 > S.stack_entries) {
    *err = 1;
    return false;
  }
  // push the farther hits (far first), descend into the nearest
  int32_t first = 0;
  int sp = R.sp;
  if (ANY) {
    // node order: descend into the first hit child, push the others
    bool have = false;
    if (d3 < INFINITY) { first = r3; have = true; }
    if (d2 < INFINITY) { if (have) stack[(sp++) * stride] = first; first = r2; have = true; }
    if (d1 < INFINITY) { if (have) stack[(sp++) * stride] = first; first = r1; have = true; }
    if (d0 < INFINITY) { if (have) stack[(sp++) * stride] = first; first = r0; have = true; }
  } else {
    if (d3 < INFINITY) stack[(sp++) * stride] = r3;
    if (d2 < INFINITY) stack[(sp++) * stride] = r2;
    if (d1 < INFINITY) stack[(sp++) * stride] = r1;
    first = r0;  // d0 is the smallest and finite (nh > 0)
  }
  R.sp = sp;
  R.ref = first;
  return true;
}

// One traversal step of one ray: a node visit or the test of ONE item of the
// current leaf (the leaf reference then advances to the leaf's next item, in
// item order, so hits and their order are those of a whole-leaf test).  The
// short step keeps a persistent warp's lanes close: a lane in a node and a
// lane in a 4-item leaf cost one node visit + one item test per turn, not a
// node visit + the leaf's whole loop.  Returns true
// when the ray is finished: closest -> R.found / R.hit hold the nearest hit;
// any -> R.found = occluded.  *err is set when the stack would overflow or
// the iteration cap is reached (never expected); the ray is then finished
// with what it has.
template <bool ANY, bool CURVES = true>
__device__ __forceinline__ bool trav_step(const SceneView &S, TravRay &R, int32_t *stack, int stride, int *err) {
  if (++R.iters > S.trav_cap) {
    *err = 2;
    return true;
  }
  if (R.ref == PT_REF_EMPTY) return true;
  if (ref_is_node(R.ref)) return !trav_node<ANY>(S, R, stack, stride, err);
  // one leaf item per step, the leaf's items in order
  const int32_t code = ~R.ref;  // first_item << 3 | count - 1
  if (test_item<ANY, CURVES>(S, code >> 3, R.o, R.d, R.dn, R.tmin, R.tmax, R.hit, R.time)) {
    R.found = true;
    if (ANY) return true;
  }
  // the rest of the leaf, (first + 1, count - 1), is ~(code + 7) = ref - 7
  R.ref = (code & 7) ? R.ref - 7 : trav_pop(R, stack, stride);
  return false;
}

// The kind of step a warp's lanes take this turn: leaf-item tests when at
// least half of the active lanes stand at a leaf, else node visits (lanes
// whose traversal has ended take theirs in node turns).  Every lane steps in
// one code path per turn instead of the warp issuing both paths each turn for
// its mix of lanes; lanes of the other kind wait a turn.  Each ray takes the
// same steps in the same order either way, so hits are unchanged.  Called by
// every lane of the warp.
__device__ __forceinline__ bool warp_leaf_turn(bool active, int32_t ref) {
  const unsigned am = __ballot_sync(0xffffffffu, active);
  const unsigned lm = __ballot_sync(0xffffffffu, active && ref_is_leaf(ref));
  return 2 * __popc(lm) >= __popc(am);
}
__device__ __forceinline__ bool lane_turn(bool active, int32_t ref, bool leaf_turn) {
  return active && ref_is_leaf(ref) == leaf_turn;
}

// Whole traversal of one ray by one thread (batch test kernels).
template <bool ANY>
__device__ bool traverse(const SceneView &S, V3 o, V3 d, float tmin, float tmax, HitRec &hit,
                         int32_t *stack, int stride, int *err, float time = 0.f) {
  TravRay R;
  trav_init(R, o, d, tmin, tmax, time);
  while (!trav_step<ANY>(S, R, stack, stride, err)) {
  }
  hit = R.hit;
  return R.found;
}

}  // namespace pt
