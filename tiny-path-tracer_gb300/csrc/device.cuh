// device.cuh - sm_103a device code of the hot path: Philox RNG, exact
// closest-hit traversal (slab test, sphere/rect/box/instance/medium), hit
// finalisation, textures, materials, mixture-pdf light sampling and the
// per-vertex shading step shared by the wavefront and persistent engines.
//
// Exactness: every operation of the hit path is an explicit round-to-nearest
// intrinsic (x* helpers below), which the compiler never contracts into an
// FMA, in the reference's float operation order; the sphere root - which the
// reference evaluates in double (sphere.cc:23,32: unqualified sqrt on float
// promotes) - is reproduced with a float-float evaluation instead of slow
// FP64.  Shading, which is compared statistically, uses ordinary (fusable)
// arithmetic and fast intrinsics.
#ifndef TPT_DEVICE_CUH
#define TPT_DEVICE_CUH

#include <cuda_runtime.h>
#include <math_constants.h>
#include <stdint.h>

#include "../../include/tpt.h"
#include "arena.h"

namespace tpt {

// ---------------------------------------------------------- float3 math --
__device__ __forceinline__ float3 v3(float a, float b, float c) { return make_float3(a, b, c); }
__device__ __forceinline__ float3 operator+(float3 a, float3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ float3 operator-(float3 a, float3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ float3 operator-(float3 a) { return v3(-a.x, -a.y, -a.z); }
__device__ __forceinline__ float3 operator*(float3 a, float3 b) { return v3(a.x * b.x, a.y * b.y, a.z * b.z); }
__device__ __forceinline__ float3 operator*(float3 a, float t) { return v3(a.x * t, a.y * t, a.z * t); }
__device__ __forceinline__ float3 operator*(float t, float3 a) { return v3(a.x * t, a.y * t, a.z * t); }
__device__ __forceinline__ float3 operator/(float3 a, float t) { return v3(a.x / t, a.y / t, a.z / t); }
__device__ __forceinline__ float dot3(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ float3 cross3(float3 a, float3 b) {
  return v3(a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y);
}
__device__ __forceinline__ float length3(float3 a) { return sqrtf(dot3(a, a)); }
__device__ __forceinline__ float3 unit3(float3 a) { return a * rsqrtf(dot3(a, a)); }  // shading only
__device__ __forceinline__ float comp(float3 v, int i) { return i == 0 ? v.x : (i == 1 ? v.y : v.z); }
__device__ __forceinline__ float3 f3(const f4 &a) { return v3(a.x, a.y, a.z); }
__device__ __forceinline__ f4 ldg4(const f4 *p) {
  float4 q = __ldg(reinterpret_cast<const float4 *>(p));
  return f4{q.x, q.y, q.z, q.w};
}
__device__ __forceinline__ i4 ldg4(const i4 *p) {
  int4 q = __ldg(reinterpret_cast<const int4 *>(p));
  return i4{q.x, q.y, q.z, q.w};
}

// Unfused IEEE round-to-nearest operations for the hit path.
__device__ __forceinline__ float xm(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float xa(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float xs(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float xd(float a, float b) { return __fdiv_rn(a, b); }
__device__ __forceinline__ float3 xadd3(float3 a, float3 b) { return v3(xa(a.x, b.x), xa(a.y, b.y), xa(a.z, b.z)); }
__device__ __forceinline__ float3 xsub3(float3 a, float3 b) { return v3(xs(a.x, b.x), xs(a.y, b.y), xs(a.z, b.z)); }
__device__ __forceinline__ float3 xscl3(float3 a, float t) { return v3(xm(a.x, t), xm(a.y, t), xm(a.z, t)); }
__device__ __forceinline__ float3 xdiv3(float3 a, float t) { return v3(xd(a.x, t), xd(a.y, t), xd(a.z, t)); }
__device__ __forceinline__ float xdot3(float3 a, float3 b) {  // vec3.h:77-79 order
  return xa(xa(xm(a.x, b.x), xm(a.y, b.y)), xm(a.z, b.z));
}
// n / d correctly rounded, given y = RN(1/d): q = RN(n*y) is within an ulp
// and the FMA remainder step of Markstein (IBM J. R&D 34(1), 1990) rounds
// it correctly.  Outside that theorem's range (d = 0 or tiny, overflow,
// subnormal or zero quotients) the IEEE division is used.
__device__ __forceinline__ float xdiv_rcp(float n, float d, float y) {
  const float q = xm(n, y);
  const float r = __fmaf_rn(-q, d, n);
  const float q2 = __fmaf_rn(r, y, q);
  const float a = fabsf(q2);
  if (!(a <= 1.0e37f) || a < 1.0e-36f || !(fabsf(y) <= 1.0e36f)) return xd(n, d);
  return q2;
}

struct Ray {
  float3 o, d;
  float time;
};
__device__ __forceinline__ float3 at(const Ray &r, float t) { return xadd3(r.o, xscl3(r.d, t)); }  // ray.h:13

// -------------------------------------------------------------- Philox ---
// Philox-4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11): counter-based, so every
// (pixel, sample, bounce, purpose) tuple owns an independent stream.
__device__ __forceinline__ uint4 philox(uint4 c, uint2 k) {
#pragma unroll
  for (int i = 0; i < 10; i++) {
    uint32_t lo0 = 0xD2511F53u * c.x, hi0 = __umulhi(0xD2511F53u, c.x);
    uint32_t lo1 = 0xCD9E8D57u * c.z, hi1 = __umulhi(0xCD9E8D57u, c.z);
    c = make_uint4(hi1 ^ c.y ^ k.x, lo1, hi0 ^ c.w ^ k.y, lo0);
    k.x += 0x9E3779B9u;
    k.y += 0xBB67AE85u;
  }
  return c;
}
__device__ __forceinline__ float u01(uint32_t x) { return (float)(x >> 8) * (1.0f / 16777216.0f); }
__device__ __forceinline__ float4 uniforms(uint4 c, uint2 k) {
  uint4 r = philox(c, k);
  return make_float4(u01(r.x), u01(r.y), u01(r.z), u01(r.w));
}

// Stream purposes (counter word w).
enum { RNG_CAMERA_A = 0, RNG_CAMERA_B = 1, RNG_SCATTER = 2, RNG_MEDIUM = 3, RNG_GUIDE = 4 };

// Medium free-flight uniforms: a trace query keys them by (ray index,
// medium id); a render path by (pixel, sample, bounce, medium id).
struct MediumRng {
  uint4 ctr;   // .z or .w receives the medium id (see medium_u)
  uint2 key;
  int mode;    // 0: trace query, 1: render
};
__device__ __forceinline__ float medium_u(const MediumRng &m, int medium_user) {
  uint4 c = m.ctr;
  if (m.mode == 0)
    c.z = (uint32_t)medium_user;
  else
    c.w = RNG_MEDIUM + 16u * (uint32_t)medium_user;
  return u01(philox(c, m.key).x);
}

// ---------------------------------------------------------- slab test ----
// Precomputed per ray: 1.0f/d (aabb.cc:5, IEEE division) and whether each
// reciprocal is negative (the swap of aabb.cc:8-10).
struct RayPre {
  float3 o, inv;
  bool nx, ny, nz;
  float inv_len;  // 1/|d|, for the prune margin
  float slack;    // origin-magnitude term of the prune margin
};
__device__ __forceinline__ RayPre precompute(const Ray &r) {
  RayPre p;
  p.o = r.o;
  p.inv = v3(__frcp_rn(r.d.x), __frcp_rn(r.d.y), __frcp_rn(r.d.z));  // == 1.0f / d, IEEE
  p.nx = p.inv.x < 0.0f;
  p.ny = p.inv.y < 0.0f;
  p.nz = p.inv.z < 0.0f;
  p.inv_len = rsqrtf(dot3(r.d, r.d));
  p.slack = 3.814697265625e-06f * (fabsf(r.o.x) + fabsf(r.o.y) + fabsf(r.o.z)) * p.inv_len;  // 2^-18
  return p;
}

// Lower bound on the t a primitive inside box (lo, hi) can report, given the
// box entry.  The reference's float arithmetic does not place a hit exactly
// on the geometry: its sphere quadratic loses up to ~2^-10 |o-c|/|d| in t
// (disc = b*b - 4ac cancels near tangency), so a hit can lie outside the
// primitive's box.  The bound subtracts 2^-8 (entry + box diagonal / |d|),
// four times that error, plus a term for rounding of a transformed origin.
__device__ __forceinline__ float prune_key_ext(const RayPre &r, float ext, float entry) {
  return entry * 0.99609375f - ext * 0.00390625f * r.inv_len - r.slack;
}
__device__ __forceinline__ float prune_key(const RayPre &r, const f4 &lo, const f4 &hi, float entry) {
  const float ext = (hi.x - lo.x) + (hi.y - lo.y) + (hi.z - lo.z);  // >= box diagonal
  return prune_key_ext(r, ext, entry);
}

// AABB::hit (aabb.cc:3-19) evaluated without the early exit: the interval
// bounds are monotone and never become NaN (a NaN slab value fails the
// comparison and leaves the bound unchanged, which fmaxf/fminf reproduce),
// so the final emptiness test equals the reference's early-exit result.
__device__ __forceinline__ bool slab(const RayPre &r, const f4 &lo, const f4 &hi, float tmin, float tmax,
                                     float &entry) {
  float n0 = xm(xs(r.nx ? hi.x : lo.x, r.o.x), r.inv.x);
  float f0 = xm(xs(r.nx ? lo.x : hi.x, r.o.x), r.inv.x);
  float n1 = xm(xs(r.ny ? hi.y : lo.y, r.o.y), r.inv.y);
  float f1 = xm(xs(r.ny ? lo.y : hi.y, r.o.y), r.inv.y);
  float n2 = xm(xs(r.nz ? hi.z : lo.z, r.o.z), r.inv.z);
  float f2 = xm(xs(r.nz ? lo.z : hi.z, r.o.z), r.inv.z);
  tmin = fmaxf(fmaxf(fmaxf(n0, tmin), n1), n2);
  tmax = fminf(fminf(fminf(f0, tmax), f1), f2);
  entry = tmin;
  return !(tmin > tmax);
}

// -------------------------------------------------------- primitives -----
// The reference's (float)(((double)(-b) -/+ sqrt((double)disc)) / (2a))
// (sphere.cc:23,32), in float-float arithmetic: sqrt to ~2^-47 via the
// exact FMA residual, the numerator as an unevaluated sum, the quotient with
// an exact remainder, and one final rounding.  Agrees with the double
// evaluation except when the root lies within ~2^-44 relative of a float
// rounding boundary.
__device__ __forceinline__ float ref_root(float b, float disc, float a2, bool far_root) {
  float sh = __fsqrt_rn(disc);
  float e = __fmaf_rn(-sh, sh, disc);
  float sl = __fdividef(e, xm(2.0f, sh));
  float x = -b;
  float y = far_root ? sh : -sh;
  float yl = far_root ? sl : -sl;
  float s = __fadd_rn(x, y);
  float bb = __fsub_rn(s, x);
  float err = __fadd_rn(__fsub_rn(x, __fsub_rn(s, bb)), __fsub_rn(y, bb));
  float nl = __fadd_rn(err, yl);
  float nh = __fadd_rn(s, nl);
  nl = __fsub_rn(nl, __fsub_rn(nh, s));
  float qh = __fdiv_rn(nh, a2);
  float r = __fmaf_rn(-qh, a2, nh);
  float ql = __fdividef(__fadd_rn(r, nl), a2);
  return __fadd_rn(qh, ql);
}

// sphere::hit candidate (sphere.cc:13-43): near root if it lies in
// (tmin, tmax), else the far root.
__device__ __forceinline__ bool sphere_t(float3 c, float radius, const Ray &r, float tmin, float tmax, float &t) {
  float3 oc = xsub3(r.o, c);
  float a = xdot3(r.d, r.d);
  float b = xm(2.0f, xdot3(r.d, oc));
  float cc = xs(xdot3(oc, oc), xm(radius, radius));
  float disc = xs(xm(b, b), xm(xm(4.0f, a), cc));
  if (!(disc > 0.0f)) return false;
  float a2 = xm(2.0f, a);
  float tn = ref_root(b, disc, a2, false);
  if (tn < tmax && tn > tmin) {
    t = tn;
    return true;
  }
  float tf = ref_root(b, disc, a2, true);
  if (tf < tmax && tf > tmin) {
    t = tf;
    return true;
  }
  return false;
}

__device__ __forceinline__ float3 msphere_center(const f4 &d0, const f4 &d1, const f4 &d2, float time) {
  // sphere.h:29-32
  return xadd3(f3(d0), xscl3(xsub3(f3(d1), f3(d0)), xd(xs(time, d1.w), xs(d2.x, d1.w))));
}

// Axis-aligned rectangle (rect_box.cc:8-24,51-68,75-91): plane axis ax,
// in-plane axes (ia, ib); closed interval [tmin, tmax].
template <int AX>
__device__ __forceinline__ bool rect_t(float a0, float a1, float b0, float b1, float k, const Ray &r, float y,
                                       float tmin, float tmax, float &t) {
  constexpr int IA = AX == 0 ? 1 : 0;
  constexpr int IB = AX == 2 ? 1 : 2;
  float tt = xdiv_rcp(xs(k, comp(r.o, AX)), comp(r.d, AX), y);
  if (tt > tmax || tt < tmin) return false;
  float a = xa(comp(r.o, IA), xm(tt, comp(r.d, IA)));
  float b = xa(comp(r.o, IB), xm(tt, comp(r.d, IB)));
  if (a < a0 || a > a1 || b < b0 || b > b1) return false;
  t = tt;
  return true;
}
__device__ __forceinline__ bool rect_any(int ax, float4 ab, float k, const Ray &r, float3 inv, float tmin, float tmax,
                                         float &t) {
  if (ax == 0) return rect_t<0>(ab.x, ab.y, ab.z, ab.w, k, r, inv.x, tmin, tmax, t);
  if (ax == 1) return rect_t<1>(ab.x, ab.y, ab.z, ab.w, k, r, inv.y, tmin, tmax, t);
  return rect_t<2>(ab.x, ab.y, ab.z, ab.w, k, r, inv.z, tmin, tmax, t);
}

// box (rect_box.cc:93-119): a hitable_list of six faces, sequential with the
// shrinking closest_so_far; a face is accepted when t <= closest, so a tie
// goes to the later face.
__device__ __forceinline__ bool box_t(float3 p0, float3 p1, const Ray &r, float3 inv, float tmin, float tmax,
                                      float &t, int &face) {
  bool any = false;
  float closest = tmax, tt;
  if (rect_t<2>(p0.x, p1.x, p0.y, p1.y, p1.z, r, inv.z, tmin, closest, tt)) { closest = tt; face = 0; any = true; }
  if (rect_t<2>(p0.x, p1.x, p0.y, p1.y, p0.z, r, inv.z, tmin, closest, tt)) { closest = tt; face = 1; any = true; }
  if (rect_t<1>(p0.x, p1.x, p0.z, p1.z, p1.y, r, inv.y, tmin, closest, tt)) { closest = tt; face = 2; any = true; }
  if (rect_t<1>(p0.x, p1.x, p0.z, p1.z, p0.y, r, inv.y, tmin, closest, tt)) { closest = tt; face = 3; any = true; }
  if (rect_t<0>(p0.y, p1.y, p0.z, p1.z, p1.x, r, inv.x, tmin, closest, tt)) { closest = tt; face = 4; any = true; }
  if (rect_t<0>(p0.y, p1.y, p0.z, p1.z, p0.x, r, inv.x, tmin, closest, tt)) { closest = tt; face = 5; any = true; }
  t = closest;
  return any;
}

// translate / rotate_y applied to a ray, world to object (rect_box.h:87-95,
// rect_box.cc:171-182).
__device__ __forceinline__ Ray to_object(const f4 *data, int nops, Ray r) {
  for (int i = 0; i < nops; i++) {
    f4 op = ldg4(data + 1 + i);
    if (op.x == (float)OP_TRANSLATE) {
      r.o = xsub3(r.o, v3(op.y, op.z, op.w));
    } else {
      float sn = op.y, cs = op.z;
      float3 o = r.o, d = r.d;
      r.o = v3(xs(xm(cs, o.x), xm(sn, o.z)), o.y, xa(xm(sn, o.x), xm(cs, o.z)));
      r.d = v3(xs(xm(cs, d.x), xm(sn, d.z)), d.y, xa(xm(sn, d.x), xm(cs, d.z)));
    }
  }
  return r;
}
// hit point and normal back to world (rect_box.cc:183-190, rect_box.h:92)
__device__ __forceinline__ void to_world(const f4 *data, int nops, float3 &p, float3 &n) {
  for (int i = nops - 1; i >= 0; i--) {
    f4 op = ldg4(data + 1 + i);
    if (op.x == (float)OP_TRANSLATE) {
      p = xadd3(p, v3(op.y, op.z, op.w));
    } else {
      float sn = op.y, cs = op.z;
      p = v3(xa(xm(cs, p.x), xm(sn, p.z)), p.y, xa(xm(-sn, p.x), xm(cs, p.z)));
      n = v3(xa(xm(cs, n.x), xm(sn, n.z)), n.y, xa(xm(-sn, n.x), xm(cs, n.z)));
    }
  }
}

// Candidate of a geometric primitive leaf (sphere, moving sphere, rect,
// box).  face: box face or -1.
// Scene feature sets the traversal can be specialised for: every leaf kind
// (the general case), spheres only (no rects, boxes, moving spheres,
// instances or media), or no media and no moving spheres; their kernels
// carry none of the code of the kinds they exclude.
enum { FEAT_ALL = 0, FEAT_SPHERES = 1, FEAT_NO_MEDIA = 2 };  // NO_MEDIA: no media, no moving spheres

template <int FEAT = FEAT_ALL>
__device__ __forceinline__ bool prim_t(const DevScene &S, const i4 &h, const Ray &r, float3 inv, float tmin,
                                       float tmax, float &t, int &face) {
  const f4 *d = S.leaf_data + h.y;
  int type = h.x & LEAF_TYPE_MASK;
  face = -1;
  if (FEAT == FEAT_SPHERES || type == LT_SPHERE) {
    f4 s = ldg4(d);
    return sphere_t(f3(s), s.w, r, tmin, tmax, t);
  }
  if (type == LT_RECT) {
    f4 ab = ldg4(d), k = ldg4(d + 1);
    return rect_any((h.x >> LEAF_AXIS_SHIFT) & 3, make_float4(ab.x, ab.y, ab.z, ab.w), k.x, r, inv, tmin, tmax, t);
  }
  if (type == LT_BOX) {
    f4 p0 = ldg4(d), p1 = ldg4(d + 1);
    return box_t(f3(p0), f3(p1), r, inv, tmin, tmax, t, face);
  }
  if (FEAT != FEAT_NO_MEDIA && type == LT_MSPHERE) {
    f4 d0 = ldg4(d), d1 = ldg4(d + 1), d2 = ldg4(d + 2);
    return sphere_t(msphere_center(d0, d1, d2, r.time), d0.w, r, tmin, tmax, t);
  }
  return false;
}

// A primitive or a transformed primitive (medium boundaries).
__device__ __forceinline__ float3 recip3(float3 d) { return v3(__frcp_rn(d.x), __frcp_rn(d.y), __frcp_rn(d.z)); }

__device__ __noinline__ bool simple_t(const DevScene &S, int leaf, const Ray &r, float tmin, float tmax, float &t) {
  i4 h = ldg4(S.leaf_hdr + leaf);
  int face;
  if ((h.x & LEAF_TYPE_MASK) == LT_INSTANCE) {
    const f4 *d = S.leaf_data + h.y;
    Ray o = to_object(d, (int)ldg4(d).x, r);
    i4 ch = ldg4(S.leaf_hdr + ~h.w);
    return prim_t(S, ch, o, recip3(o.d), tmin, tmax, t, face);
  }
  return prim_t(S, h, r, recip3(r.d), tmin, tmax, t, face);
}

// constant_medium::hit (hitable.cc:98-128) with the free-flight uniform u.
__device__ __forceinline__ bool medium_t(const DevScene &S, const i4 &h, const Ray &r, float tmin, float tmax, float u,
                                         float &t) {
  float t1, t2;
  if (!simple_t(S, h.w, r, -3.402823466e38f, 3.402823466e38f, t1)) return false;
  if (!simple_t(S, h.w, r, (float)((double)t1 + 0.0001), 3.402823466e38f, t2)) return false;
  if (t1 < tmin) t1 = tmin;
  if (t2 > tmax) t2 = tmax;
  if (t1 >= t2) return false;
  float dl = __fsqrt_rn(xdot3(r.d, r.d));
  float inside = xm(xs(t2, t1), dl);
  float density = ldg4(S.leaf_data + h.y).x;
  float dist = xm(xd(-1.0f, density), logf(u));
  if (dist < inside) {
    t = xa(t1, xd(dist, dl));
    return true;
  }
  return false;
}

// -------------------------------------------------------------- traversal -
struct HitRef {
  float t;
  int leaf;  // primitive / medium leaf
  int inst;  // instance leaf, or -1
  int face;  // box face, or -1
};

// Tie order inside one item: larger (outer, inner) wins - the reference's
// bvh_node keeps the right child on equal t (hitable.cc:71).
__device__ __forceinline__ bool beats(float t, int outer, int inner, float bt, int bouter, int binner) {
  return t < bt || (t == bt && (outer > bouter || (outer == bouter && inner > binner)));
}

// Stack entries {what, prune key}: what >= 0 an internal node whose box
// passed; STK_RESTORE leave object space; what <= -2 the leaf -2-what (an
// instanced BVH is entered when its leaf is popped).  Leaves go through the
// stack too, so the primitive tests have a single call site.
enum { STK_RESTORE = -1 };
// Stackless walks over at most this many nodes skip the pruning test.
enum { FLAT_PRUNE_MIN = 32 };

// Closest hit of the world for ray wr over [tmin, FLT_MAX] with the exact
// semantics of hitable_list::hit across the top-level items (sequential,
// shrinking t_max) and bvh_node::hit within an item (every child tested with
// the same interval, ties to the right).  The candidate set is the
// reference's: a leaf is tested iff every ancestor box passes.  BVHs of at
// most flat_max nodes are walked stacklessly in pre-order (a box miss jumps
// to the node's skip index), which keeps a warp's lanes on the same node
// sequence; larger ones near-first with a shared-memory stack.  Both prune,
// which cannot change the result: the winner is the minimum of
// (t, -leaf order), and a subtree is skipped only when the lower bound
// prune_key() on any t its primitives can report exceeds the best t.  stk: this thread's stack slots, `stride`
// entries apart.  err receives TPT_ERR_STACK_OVERFLOW on overflow.
template <int FEAT = FEAT_ALL, bool INL = true>
__device__ bool trace_closest(const DevScene &S, const Ray &wr, float tmin, int2 *stk, int stride,
                              const MediumRng &mrng, HitRef &res, int &err) {
  const RayPre W = precompute(wr);
  float closest = 3.402823466e38f;  // std::numeric_limits<float>::max()
  bool found = false;
  const int never_pruned = __float_as_int(-CUDART_INF_F);
  for (int it = 0; it < S.n_items; it++) {
    const int2 item = *reinterpret_cast<const int2 *>(S.items + it);
    const float tmax = closest;
    float bt = CUDART_INF_F;
    int bl = -1, bi = -1, bf = -1, bo = -1, bn = -1;
    int sp = 0;
    bool overflow = false;
    Ray cur = wr;
    RayPre curp = W;
    int cur_inst = -1;

    auto push = [&](int what, int key) {
      if (sp >= TRAVERSAL_STACK) {
        overflow = true;
      } else {
        stk[sp * stride] = make_int2(what, key);
        sp++;
      }
    };

    auto run_stack = [&]() {
      while (sp > 0 && !overflow) {
        --sp;
        const int2 e = stk[sp * stride];
        if (FEAT != FEAT_SPHERES && e.x == STK_RESTORE) {
          cur = wr;
          curp = W;
          cur_inst = -1;
          continue;
        }
        if (__int_as_float(e.y) > bt) continue;
        if (e.x <= -2) {  // a leaf
          const int leaf = -2 - e.x;
          const i4 h = ldg4(S.leaf_hdr + leaf);
          const int type = h.x & LEAF_TYPE_MASK;
          float t;
          int face = -1;
          if (FEAT != FEAT_SPHERES && type == LT_INSTANCE) {
            const f4 *d = S.leaf_data + h.y;
            const Ray o = to_object(d, (int)ldg4(d).x, wr);
            const RayPre op = precompute(o);
            if (h.w < 0) {  // one transformed primitive
              const int cl = ~h.w;
              if (prim_t(S, ldg4(S.leaf_hdr + cl), o, op.inv, tmin, tmax, t, face) && beats(t, leaf, cl, bt, bo, bn)) {
                bt = t; bl = cl; bi = leaf; bf = face; bo = leaf; bn = cl;
              }
            } else {  // instanced BVH: enter object space if its root box passes
              float en;
              const f4 rlo = ldg4(S.node_lo + h.w), rhi = ldg4(S.node_hi + h.w);
              if (slab(op, rlo, rhi, tmin, tmax, en)) {
                push(STK_RESTORE, 0);
                push(h.w, __float_as_int(prune_key(op, rlo, rhi, en)));
                cur = o;
                curp = op;
                cur_inst = leaf;
              }
            }
            continue;
          }
          const int outer = cur_inst >= 0 ? cur_inst : leaf;
          const int inner = cur_inst >= 0 ? leaf : -1;
          bool ok;
          if (FEAT == FEAT_ALL && type == LT_MEDIUM)
            ok = medium_t(S, h, cur, tmin, tmax, medium_u(mrng, S.leaf_user[leaf]), t);
          else
            ok = prim_t<FEAT>(S, h, cur, curp.inv, tmin, tmax, t, face);
          if (ok && beats(t, outer, inner, bt, bo, bn)) {
            bt = t; bl = leaf; bi = cur_inst; bf = face; bo = outer; bn = inner;
          }
          continue;
        }
        // internal node: test the child boxes (stored with the node, one
        // 64-byte record), push near child last
        const f4 *kid = S.node_kids + 4 * (size_t)e.x;
        const f4 k0 = ldg4(kid), k1 = ldg4(kid + 1), k2 = ldg4(kid + 2), k3 = ldg4(kid + 3);
        const int left = __float_as_int(k0.w), right = __float_as_int(k2.w);
        int2 q[2];
        float ent[2];
        int nq = 0;
        for (int c = 0; c < 2; c++) {
          const int ref = c == 0 ? left : right;
          if (c == 1 && right == left) break;  // n == 1 node: left_ == right_
          if (ref >= 0) {
            float en;
            const f4 clo = c == 0 ? k0 : k2, chi = c == 0 ? k1 : k3;
            if (slab(curp, clo, chi, tmin, tmax, en)) {
              const float key = prune_key_ext(curp, chi.w, en);  // chi.w: box size term
              // the general persistent kernel (!INL) also prunes here rather
              // than when the entry is popped (bt only falls, so the result
              // is the same): measured faster there, slower in the others
              if (INL || !(key > bt)) {
                ent[nq] = en;
                q[nq++] = make_int2(ref, __float_as_int(key));
              }
            }
          } else if (INL && (FEAT == FEAT_SPHERES || (c == 0 ? k1 : k3).y != 0.f)) {
            // a sphere leaf: its center and radius ride in the child's box
            // slot, so it is tested here, with no stack entry and no header
            // or data load (INL: compiled in; the general persistent kernel
            // leaves it out, which keeps tiny mixed scenes' code smaller)
            const f4 sc = c == 0 ? k0 : k2;
            const int leaf = ~ref;
            const int outer = cur_inst >= 0 ? cur_inst : leaf, inner = cur_inst >= 0 ? leaf : -1;
            float t;
            if (sphere_t(v3(sc.x, sc.y, sc.z), (c == 0 ? k1 : k3).x, cur, tmin, tmax, t) &&
                beats(t, outer, inner, bt, bo, bn)) {
              bt = t; bl = leaf; bi = cur_inst; bf = -1; bo = outer; bn = inner;
            }
          } else {
            push(-2 - ~ref, never_pruned);
          }
        }
        if (nq == 2 && ent[1] > ent[0]) {
          const int2 tq = q[0];
          q[0] = q[1];
          q[1] = tq;
        }
        for (int k = 0; k < nq; k++) push(q[k].x, q[k].y);
        // leaves pushed above go after the near child; order does not matter
      }
    };

    if (item.x == ITEM_BVH) {
      const int root = item.y;
      const int end = __ldg(S.node_skip + root);
      if (end - root <= S.flat_max) {
        // pruning pays only on trees with more than a few boxes per path
        const bool prune = end - root > FLAT_PRUNE_MIN;
        for (int i = root; i < end && !overflow;) {
          const f4 lo = ldg4(S.node_lo + i), hi = ldg4(S.node_hi + i);
          float en;
          if (slab(W, lo, hi, tmin, tmax, en) && !(prune && prune_key(W, lo, hi, en) > bt)) {
            const int left = __float_as_int(lo.w), right = __float_as_int(hi.w);
            if (right < 0) push(-2 - ~right, never_pruned);
            if (left < 0 && left != right) push(-2 - ~left, never_pruned);
            if (sp > 0) run_stack();
            i++;
          } else {
            i = __ldg(S.node_skip + i);
          }
        }
      } else {
        float en;
        const f4 lo = ldg4(S.node_lo + root), hi = ldg4(S.node_hi + root);
        if (slab(W, lo, hi, tmin, tmax, en)) {
          push(root, never_pruned);
          run_stack();
        }
      }
    } else {
      push(-2 - item.y, never_pruned);
      run_stack();
    }
    if (overflow) err = TPT_ERR_STACK_OVERFLOW;
    if (bl >= 0) {
      closest = bt;
      res = HitRef{bt, bl, bi, bf};
      found = true;
    }
  }
  return found;
}

// ------------------------------------------------------ hit finalisation --
struct Surface {
  float3 p, n;
  float u, v;
  int mat;
};

// get_uv_map (utils.h:38-43)
__device__ __forceinline__ void uv_map(float3 q, float &u, float &v) {
  u = atan2f(q.z, q.x) / 6.28318530717958647692f + 0.5f;
  v = asinf(q.y) / 3.14159265358979323846f + 0.5f;
}

// Rebuilds the hit record (point, normal, uv, material) the reference's hit
// functions fill in, from the traversal result: the instance's object-space
// ray is recomputed with the same operations, the primitive's record is
// formed in object space and carried back to world (rect_box.cc:183-190).
// all_uv: compute (u, v) for every hit (the closest-hit API reports them);
// otherwise only where the material's texture reads them (image textures),
// which spares renders the sphere's atan2/asin and the rect's two divisions.
__device__ void finalize(const DevScene &S, const Ray &wr, const HitRef &h, Surface &s, bool all_uv = true) {
  Ray r = wr;
  const f4 *idata = nullptr;
  int nops = 0;
  bool iflip = false;
  if (h.inst >= 0) {
    const i4 ih = ldg4(S.leaf_hdr + h.inst);
    idata = S.leaf_data + ih.y;
    nops = (int)ldg4(idata).x;
    r = to_object(idata, nops, wr);
    iflip = (ih.x & LEAF_FLIP) != 0;
  }
  const i4 lh = ldg4(S.leaf_hdr + h.leaf);
  const f4 *d = S.leaf_data + lh.y;
  const float t = h.t;
  const int type = lh.x & LEAF_TYPE_MASK;
  s.mat = lh.z;
  const bool uv = all_uv || ldg4(S.mat_i + lh.z).w != 0;
  s.u = 0.f;
  s.v = 0.f;
  if (type == LT_SPHERE || type == LT_MSPHERE) {  // sphere.cc:24-28,56-60
    const f4 d0 = ldg4(d);
    float3 c0 = f3(d0), c = c0;
    if (type == LT_MSPHERE) c = msphere_center(d0, ldg4(d + 1), ldg4(d + 2), r.time);
    s.p = at(r, t);
    if (uv) uv_map(xdiv3(xsub3(s.p, c0), d0.w), s.u, s.v);
    s.n = xdiv3(xsub3(s.p, c), d0.w);
  } else if (type == LT_RECT || type == LT_BOX) {
    int ax;
    float a0, a1, b0, b1;
    bool fflip = false;
    if (type == LT_RECT) {
      const f4 ab = ldg4(d);
      ax = (lh.x >> LEAF_AXIS_SHIFT) & 3;
      a0 = ab.x; a1 = ab.y; b0 = ab.z; b1 = ab.w;
    } else {  // box faces in the order of rect_box.cc:101-113
      const float3 p0 = f3(ldg4(d)), p1 = f3(ldg4(d + 1));
      const int f = h.face;
      ax = f < 2 ? 2 : (f < 4 ? 1 : 0);
      fflip = (f & 1) != 0;
      a0 = ax == 0 ? p0.y : p0.x;
      a1 = ax == 0 ? p1.y : p1.x;
      b0 = ax == 2 ? p0.y : p0.z;
      b1 = ax == 2 ? p1.y : p1.z;
    }
    if (uv) {
      const int ia = ax == 0 ? 1 : 0, ib = ax == 2 ? 1 : 2;
      const float a = xa(comp(r.o, ia), xm(t, comp(r.d, ia)));
      const float b = xa(comp(r.o, ib), xm(t, comp(r.d, ib)));
      s.u = xd(xs(a, a0), xs(a1, a0));
      s.v = xd(xs(b, b0), xs(b1, b0));
    }
    s.p = at(r, t);
    s.n = v3(ax == 0 ? 1.f : 0.f, ax == 1 ? 1.f : 0.f, ax == 2 ? 1.f : 0.f);
    if (fflip) s.n = -s.n;
  } else {  // medium: hitable.cc:118-123 (random normal; uv left untouched)
    s.p = at(r, t);
    s.n = v3(1.f, 0.f, 0.f);
  }
  if (lh.x & LEAF_FLIP) s.n = -s.n;
  if (h.inst >= 0) {
    to_world(idata, nops, s.p, s.n);
    if (iflip) s.n = -s.n;
  }
}

// ---------------------------------------------------------------- textures -
// perlin noise (utils.cc:160-225): quintic fade, gradient trilinear, |.|
__device__ float perlin_noise(const DevScene &S, float3 p) {
  const float fx = floorf(p.x), fy = floorf(p.y), fz = floorf(p.z);
  float u = p.x - fx, v = p.y - fy, w = p.z - fz;
  const int i = (int)fx & 255, j = (int)fy & 255, k = (int)fz & 255;
  auto fade = [](float x) { return x * x * x * (x * (x * 6.f - 15.f) + 10.f); };
  u = fade(u); v = fade(v); w = fade(w);
  float acc = 0.f;
#pragma unroll
  for (int di = 0; di < 2; di++)
#pragma unroll
    for (int dj = 0; dj < 2; dj++)
#pragma unroll
      for (int dk = 0; dk < 2; dk++) {
        const int idx = __ldg(S.perlin_perm + ((i + di) & 255)) ^ __ldg(S.perlin_perm + 256 + ((j + dj) & 255)) ^
                        __ldg(S.perlin_perm + 512 + ((k + dk) & 255));
        const float3 g = f3(ldg4(S.perlin_grad + idx));
        const float3 wv = v3(u - di, v - dj, w - dk);
        acc += (di ? u : 1.f - u) * (dj ? v : 1.f - v) * (dk ? w : 1.f - w) * dot3(g, wv);
      }
  return fabsf(acc);
}
// Out of line: one copy shared by every texture lookup site keeps the fused
// render loops smaller (instruction-cache pressure), and perlin textures are rare.
__device__ __noinline__ float perlin_turb(const DevScene &S, float3 p) {  // utils.cc:193-203
  float acc = 0.f, weight = 1.f;
  for (int i = 0; i < 5; i++) {
    acc += weight * perlin_noise(S, p);
    weight *= 0.5f;
    p = p * 2.f;
  }
  return fabsf(acc);
}

// texture::value (texture.h:15-51, texture.cc:4-42)
__device__ __noinline__ float3 tex_value_any(const DevScene &S, int t, float u, float v, float3 p);

// Constant textures inline (the common case); the others in one out-of-line
// copy shared by every call site.
__device__ __forceinline__ float3 tex_value(const DevScene &S, int t, float u, float v, float3 p) {
  const i4 ti = ldg4(S.tex_i + t);
  if (ti.x == TT_CONST) return f3(ldg4(S.tex_f + t));
  return tex_value_any(S, t, u, v, p);
}

__device__ __noinline__ float3 tex_value_any(const DevScene &S, int t, float u, float v, float3 p) {
  for (int guard = 0; guard < 16; guard++) {
    const i4 ti = ldg4(S.tex_i + t);
    if (ti.x == TT_CONST) return f3(ldg4(S.tex_f + t));
    if (ti.x == TT_CHECKER) {
      const float sgn = sinf(10.f * p.x) * sinf(10.f * p.y) * sinf(10.f * p.z);
      t = sgn < 0.f ? ti.y : ti.z;
      continue;
    }
    if (ti.x == TT_PERLIN) {
      const float scale = ldg4(S.tex_f + t).x;
      const float g = 0.5f * (1.f + sinf(scale * p.z + 10.f * perlin_turb(S, p)));
      return v3(g, g, g);
    }
    if (ti.x == TT_IMAGE) {
      const int w = ti.y, hh = ti.z;
      int i = (int)(u * w), j = (int)((1.f - v) * hh);
      i = i < 0 ? 0 : (i > w - 1 ? w - 1 : i);
      j = j < 0 ? 0 : (j > hh - 1 ? hh - 1 : j);
      const uint8_t *q = S.images + ti.w + 3 * (size_t)i + 3 * (size_t)w * j;
      return v3(__ldg(q) / 255.f, __ldg(q + 1) / 255.f, __ldg(q + 2) / 255.f);
    }
    break;
  }
  return v3(0.f, 0.f, 0.f);
}

// -------------------------------------------------------------- samplers ---
// Same distributions as the reference's samplers, drawn by inversion from
// counter-based uniforms instead of rejection loops.
__device__ __forceinline__ float3 in_unit_sphere(float a, float b, float c) {  // utils.cc:21-27
  const float r = cbrtf(a);
  const float z = 1.f - 2.f * b;
  const float s = sqrtf(fmaxf(0.f, 1.f - z * z));
  float sn, cs;
  sincospif(2.f * c, &sn, &cs);
  return v3(r * s * cs, r * s * sn, r * z);
}
__device__ __forceinline__ float3 cos_hemisphere(float r1, float r2) {  // utils.cc:427-435
  float sn, cs;
  sincospif(2.f * r1, &sn, &cs);
  const float sr = sqrtf(r2);
  return v3(cs * sr, sn * sr, sqrtf(1.f - r2));
}
__device__ __forceinline__ float3 reflect3(float3 v, float3 n) { return v - 2.f * dot3(v, n) * n; }  // utils.cc:53-56

struct Onb {  // utils.cc:437-450
  float3 u, v, w;
  __device__ explicit Onb(float3 n) {
    w = n;
    const float3 a = fabsf(n.x) > 0.9f ? v3(0.f, 1.f, 0.f) : v3(1.f, 0.f, 0.f);
    v = unit3(cross3(n, a));
    u = cross3(v, w);
  }
  __device__ float3 local(float3 a) const { return a.x * u + a.y * v + a.z * w; }
};

// -------------------------------------------------------- light shapes -----
// pdf_value of the light_shape (hitable_list.cc:24-31, rect_box.cc:26-37,
// sphere.cc:93-106; other hitables: 0, hitable.h:35-37).
__device__ float light_item_pdf(const DevScene &S, int i, float3 o, float3 d) {
  const i4 li = ldg4(S.light_i + i);
  const f4 a = ldg4(S.light_f + 2 * i);
  const Ray r{o, d, 0.f};
  float t;
  if (li.x == LS_XZ_RECT) {
    const float k = ldg4(S.light_f + 2 * i + 1).x;
    if (!rect_t<1>(a.x, a.y, a.z, a.w, k, r, __frcp_rn(d.y), 0.0001f, 3.402823466e38f, t)) return 0.f;
    const float area = fabsf((a.y - a.x) * (a.w - a.z));
    const float3 td = t * d;
    const float d2 = dot3(td, td);
    const float cosine = fabsf(d.y / length3(d));
    return d2 / (cosine * area);
  }
  if (li.x == LS_SPHERE) {
    // sphere::pdf_value (sphere.cc:93-106) only asks whether the ray hits the
    // sphere in (0.001, FLT_MAX); a float test (not the double-root
    // reproduction of the closest-hit path) differs only on grazing rays,
    // a set of measure zero for the estimate
    {
      const float3 oc = o - f3(a);
      const float qa = dot3(d, d), qb = dot3(oc, d), qc = dot3(oc, oc) - a.w * a.w;
      const float disc = qb * qb - qa * qc;
      if (!(disc > 0.f)) return 0.f;
      const float sq = sqrtf(disc);
      // a root t = (-qb -/+ sq) / qa lies beyond 0.001 (qa > 0)
      if (!(-qb + sq > 0.001f * qa)) return 0.f;
    }
    const float3 oc = f3(a) - o;
    const float tmp = (a.w * a.w) / dot3(oc, oc);
    const float cmax = sqrtf(1.f - tmp);
    const float solid = 6.28318530717958647692f * (1.f - cmax);
    if (isnan(solid)) return 0.f;
    return 1.f / solid;
  }
  return 0.f;
}
__device__ float light_pdf(const DevScene &S, float3 o, float3 d) {
  if (!S.light_is_list) return light_item_pdf(S, 0, o, d);
  float sum = 0.f;
  for (int i = 0; i < S.n_lights; i++) sum += ldg4(S.light_f + 2 * i + 1).y * light_item_pdf(S, i, o, d);
  return sum;
}
// random() of the light_shape (hitable_list.cc:33-36, rect_box.cc:39-43,
// sphere.cc:108-120; other hitables: (1,0,0), hitable.h:38).
__device__ float3 light_random(const DevScene &S, float3 o, float pick, float r1, float r2) {
  int i = 0;
  if (S.light_is_list) {
    while (i < S.n_lights - 1 && pick >= ldg4(S.light_f + 2 * i + 1).z) i++;
  }
  const i4 li = ldg4(S.light_i + i);
  const f4 a = ldg4(S.light_f + 2 * i);
  if (li.x == LS_XZ_RECT) {
    const float k = ldg4(S.light_f + 2 * i + 1).x;
    return v3(a.x + r1 * (a.y - a.x), k, a.z + r2 * (a.w - a.z)) - o;
  }
  if (li.x == LS_SPHERE) {
    const float3 dir = f3(a) - o;
    const Onb uvw(unit3(dir));
    const float tmp = (a.w * a.w) / dot3(dir, dir);
    const float cmax = sqrtf(1.f - tmp);
    const float z = 1.f + r2 * (cmax - 1.f);
    float sn, cs;
    sincospif(2.f * r1, &sn, &cs);
    const float sz = sqrtf(1.f - z * z);
    return uvw.local(v3(cs * sz, sn * sz, z));
  }
  return v3(1.f, 0.f, 0.f);
}

__device__ float3 guide_sample(const float4 *lob, float u_lobe, float u1, float u2) {
  const float4 c0 = __ldg(lob + 8), c1 = __ldg(lob + 9);
  const int pick = (u_lobe >= c0.x) + (u_lobe >= c0.y) + (u_lobe >= c0.z) + (u_lobe >= c0.w) + (u_lobe >= c1.x) +
                   (u_lobe >= c1.y) + (u_lobe >= c1.z);
  const float4 a = __ldg(lob + pick);
  const float k = sqrtf(a.x * a.x + a.y * a.y + a.z * a.z);
  const float ik = 1.f / k;
  const float e2 = __expf(-2.f * k);
  float w = 1.f + __logf(u1 + (1.f - u1) * e2) * ik;
  w = fminf(fmaxf(w, -1.f), 1.f);
  const float sw = sqrtf(fmaxf(0.f, 1.f - w * w));
  float sn, cs;
  sincospif(2.f * u2, &sn, &cs);
  const Onb f(v3(a.x * ik, a.y * ik, a.z * ik));
  return f.local(v3(cs * sw, sn * sw, w));
}

// ----------------------------------------------------------------- camera -
// camera::get_ray (camera.cc:23-31) at the pixel-jittered (s, t) of
// main.cpp:121-124.  Row j counts from the bottom of the image.
__device__ __forceinline__ Ray camera_ray(const Camera &c, int i, int j, int nx, int ny, uint32_t pixel,
                                          uint32_t sample, uint2 key) {
  const float4 a = uniforms(make_uint4(pixel, sample, 0u, RNG_CAMERA_A), key);
  const float s = ((float)i + a.x) / (float)nx;
  const float t = ((float)j + a.y) / (float)ny;
  const float3 cu = v3(c.u[0], c.u[1], c.u[2]), cv = v3(c.v[0], c.v[1], c.v[2]);
  const float3 org = v3(c.origin[0], c.origin[1], c.origin[2]);
  float3 off = v3(0.f, 0.f, 0.f);
  if (c.lens_radius != 0.f) {
    float sn, cs;
    sincospif(2.f * a.w, &sn, &cs);
    const float rr = c.lens_radius * sqrtf(a.z);
    off = cu * (rr * cs) + cv * (rr * sn);
  }
  float time = c.t0;
  if (c.t1 != c.t0) time = c.t0 + uniforms(make_uint4(pixel, sample, 0u, RNG_CAMERA_B), key).x * (c.t1 - c.t0);
  const float3 ll = v3(c.lower_left[0], c.lower_left[1], c.lower_left[2]);
  const float3 hz = v3(c.horizontal[0], c.horizontal[1], c.horizontal[2]);
  const float3 vt = v3(c.vertical[0], c.vertical[1], c.vertical[2]);
  return Ray{org + off, ll + s * hz + t * vt - org - off, time};
}

// ---------------------------------------------------------- path guiding --
// The guiding network, evaluated on a res^3 grid of the scene box x 6 normal
// bins after each training round, as a table of GUIDE_ENTRY float4 per
// entry: 8 lobes {kappa mu.xyz, log(pi kappa / (2 pi (1 - exp(-2 kappa)))) - kappa}
// (so a lobe's density at w is exp(dot(kappa mu, w) + .w)), then the lobe
// weights' running sums {c0, c1, c2, c3}, {c4, c5, c6, c7} (GUIDE_ENTRY, arena.h).
struct GuideView {
  const float4 *lobes;  // nullptr: not guided
  float3 lo, inv_ext;
  int res;
  float alpha;        // probability of sampling the guide at a diffuse vertex
  float light_share;  // light sampling's share of the other techniques (0.5: the plain mixture)
};
// The first diffuse vertex of a path, kept to form a training record.
struct GuideRec {
  float3 x, n, d, T, L;
  bool valid;
};

__device__ __forceinline__ const float4 *guide_entry(const GuideView &g, float3 p, float3 n) {
  const int r = g.res;
  const int cx = min(max((int)((p.x - g.lo.x) * g.inv_ext.x * r), 0), r - 1);
  const int cy = min(max((int)((p.y - g.lo.y) * g.inv_ext.y * r), 0), r - 1);
  const int cz = min(max((int)((p.z - g.lo.z) * g.inv_ext.z * r), 0), r - 1);
  const float ax = fabsf(n.x), ay = fabsf(n.y), az = fabsf(n.z);
  const int bin = (ax >= ay && ax >= az) ? (n.x >= 0.f ? 0 : 1) : (ay >= az ? (n.y >= 0.f ? 2 : 3) : (n.z >= 0.f ? 4 : 5));
  return g.lobes + ((size_t)((cz * r + cy) * r + cx) * 6 + bin) * GUIDE_ENTRY;
}

// Mixture density of unit direction w (solid-angle measure).
__device__ __forceinline__ float guide_pdf(const float4 *lob, float3 w) {
  float p = 0.f;
#pragma unroll
  for (int i = 0; i < 8; i++) {
    const float4 a = __ldg(lob + i);
    p += __expf(a.x * w.x + a.y * w.y + a.z * w.z + a.w);
  }
  return p;
}

// Picks a lobe by its weight, then samples the von Mises-Fisher lobe by
// inverting its cosine distribution: cos = 1 + log(u + (1-u) e^{-2k}) / k.
__device__ float3 guide_sample(const float4 *lob, float u_lobe, float u1, float u2);

// ------------------------------------------------------------- shading ----
struct RenderCfg {
  int max_depth;
  int semantics;   // 0 reference, 1 physical
  int background;  // 0 black, 1 sky
  float sky_scale;
  uint2 key;
  int refill;      // persistent engines: idle lanes per warp that trigger new camera samples
};

__device__ __forceinline__ float3 background(const RenderCfg &cfg, const Ray &r) {  // utils.cc:85-90
  if (cfg.background == 0) return v3(0.f, 0.f, 0.f);
  const float3 ud = unit3(r.d);
  const float t = (ud.y + 1.0f) * 0.5f;
  return cfg.sky_scale * ((1.f - t) * v3(1.f, 1.f, 1.f) + t * v3(0.5f, 0.7f, 1.0f));
}

__device__ __forceinline__ bool finite3(float3 v) { return isfinite(v.x) && isfinite(v.y) && isfinite(v.z); }

__device__ __forceinline__ bool nonzero(float3 e) { return e.x != 0.f || e.y != 0.f || e.z != 0.f; }

// One vertex of color() (utils.cc:58-94), iterated: the radiance estimate
// L accumulates T * emitted, T the product of the bounce weights.  On the
// terminal vertex T * emitted is always added, so a NaN weight anywhere on
// the path makes the sample NaN as the recursive form does (de_nan then
// zeroes it).  Returns true with `ray` replaced when the path continues.
// Radiance-cache features of a hit vertex: position, outgoing direction,
// normal, albedo, roughness (lambertian/isotropic 1, metal fuzz, dielectric 0).
struct VertexInfo {
  float3 p, wo, n, albedo;
  float rough;
  int kind;  // material type (MatType)
};

__device__ __forceinline__ void vertex_info(const DevScene &S, const Ray &ray, const Surface &sf, const i4 &mi,
                                            VertexInfo &vi) {
  vi.p = sf.p;
  vi.wo = -unit3(ray.d);
  vi.n = sf.n;
  vi.kind = mi.x;
  vi.rough = 1.f;
  vi.albedo = v3(0.f, 0.f, 0.f);
  if (mi.x == MT_LAMBERTIAN || mi.x == MT_ISOTROPIC) {
    vi.albedo = tex_value(S, mi.y, sf.u, sf.v, sf.p);
  } else if (mi.x == MT_METAL) {
    const f4 mf = ldg4(S.mat_f + sf.mat);
    vi.albedo = f3(mf);
    vi.rough = mf.w;
  } else if (mi.x == MT_DIELECTRIC) {
    vi.albedo = v3(1.f, 1.f, 1.f);
    vi.rough = 0.f;
  }
}

// Path spread (Mueller et al. 2021, "Real-time Neural Radiance Caching for
// Path Tracing", section 5): the footprint a(x_1..x_n) = (sum over i >= 2 of
// sqrt(|x_{i-1} - x_i|^2 / (p(w_i) |cos theta_i|)))^2 of a path grows with
// its bounces; the path may end into the radiance cache once a exceeds
// c a_0, where a_0 = |x_0 - x_1|^2 / (4 pi cos theta_1) is the camera
// vertex's footprint.  Kept as square roots: thr = sqrt(c a_0), sum =
// sqrt(a).  Specular bounces (metal, dielectric) leave the spread as it is;
// a medium vertex has no normal (|cos| = 1) and samples 1 / (4 pi).
struct Spread {
  float thr;  // sqrt(c) until the camera hit, sqrt(c a_0) after it
  float sum;  // sqrt(a) of the vertices so far
  float pdf;  // solid-angle density the last direction was sampled with (0: specular)
};

__device__ __forceinline__ bool spread_step(Spread &sp, const Ray &ray, const HitRef &h, const Surface &sf,
                                            bool medium, int depth) {
  const float dl = length3(ray.d);
  const float dist = h.t * dl;
  const float cs = medium ? 1.f : fmaxf(fabsf(dot3(sf.n, ray.d)) / dl, 1e-4f);
  if (depth == 0) {
    sp.thr *= dist * rsqrtf(12.566370614359172954f * cs);
    sp.sum = 0.f;
    return false;
  }
  if (sp.pdf > 0.f) sp.sum += dist * rsqrtf(sp.pdf * cs);
  return sp.sum > sp.thr;
}

template <bool GUIDED>
__device__ bool shade_vertex_t(const DevScene &S, const RenderCfg &cfg, Ray &ray, bool hit, const HitRef &h,
                               float3 &T, float3 &L, int depth, uint32_t pixel, uint32_t sample, const GuideView &gv,
                               GuideRec &rec, VertexInfo *vi = nullptr, int query_depth = 1 << 30,
                               bool *queried = nullptr, Spread *sp = nullptr) {
  if (!hit) {
    L = L + T * background(cfg, ray);
    return false;
  }
  Surface sf;
  finalize(S, ray, h, sf, false);
  const i4 mi = ldg4(S.mat_i + sf.mat);
  if (vi) vertex_info(S, ray, sf, mi, *vi);
  float3 E = v3(0.f, 0.f, 0.f);
  if (mi.x == MT_LIGHT && dot3(sf.n, ray.d) < 0.f) E = tex_value(S, mi.y, sf.u, sf.v, sf.p);  // material.cc:79-86
  if (depth >= cfg.max_depth) {
    L = L + T * E;
    return false;
  }
  // radiance-cache query: the path ends here at a diffuse vertex (no
  // emission there) and the cache supplies its outgoing radiance; past
  // query_depth, or earlier once the path's spread is wide enough
  const bool spread_end = sp && spread_step(*sp, ray, h, sf, mi.x == MT_ISOTROPIC, depth);
  if (queried && (depth >= query_depth || spread_end) &&
      (mi.x == MT_LAMBERTIAN || (mi.x == MT_ISOTROPIC && cfg.semantics == 1))) {
    *queried = true;
    return false;
  }
  if (sp) sp->pdf = 0.f;  // specular unless a diffuse lobe below samples
  const float4 r = uniforms(make_uint4(pixel, sample, (uint32_t)depth, RNG_SCATTER), cfg.key);
  float3 dir, wgt;
  float time = ray.time;
  switch (mi.x) {
    case MT_METAL: {  // material.cc:88-98
      const f4 mf = ldg4(S.mat_f + sf.mat);
      dir = reflect3(unit3(ray.d), sf.n) + mf.w * in_unit_sphere(r.x, r.y, r.z);
      if (!(dot3(dir, sf.n) > 0.f)) {
        L = L + T * E;
        return false;
      }
      wgt = f3(mf);
      break;
    }
    case MT_DIELECTRIC: {  // material.cc:19-70 + refract/schlick (utils.cc:34-51)
      const float ior = ldg4(S.mat_f + sf.mat).x;
      const float3 refl = reflect3(ray.d, sf.n);
      float3 outward, refr = v3(0.f, 0.f, 0.f);
      float ni, cosine;
      const float dn = dot3(ray.d, sf.n);
      const float dl = length3(ray.d);
      if (dn > 0.f) {
        outward = -sf.n;
        ni = ior;
        cosine = dn / dl;
        cosine = sqrtf(1.f - ior * ior * (1.f - cosine * cosine));
      } else {
        outward = sf.n;
        ni = 1.0f / ior;
        cosine = -dn / dl;
      }
      const float3 uv = unit3(ray.d);
      const float dt = dot3(uv, outward);
      const float disc = 1.0f - ni * ni * (1.f - dt * dt);
      float prob = 1.0f;
      if (disc > 0.f) {
        refr = ni * (uv - outward * dt) - outward * sqrtf(disc);
        float r0 = (1.f - ior) / (1.f + ior);
        r0 = r0 * r0;
        const float m = 1.f - cosine;
        prob = r0 + (1.f - r0) * (m * m * m * m * m);
      }
      dir = r.x < prob ? refl : refr;
      wgt = v3(1.f, 1.f, 1.f);
      break;
    }
    case MT_ISOTROPIC: {  // material.cc:72-77: never reached by the reference (hidden overload)
      if (cfg.semantics == 0) {
        L = L + T * E;
        return false;
      }
      dir = in_unit_sphere(r.x, r.y, r.z);
      wgt = tex_value(S, mi.y, sf.u, sf.v, sf.p);
      time = 0.f;  // ray(rec.point, random_in_unit_sphere()) keeps the default time
      if (sp) sp->pdf = 0.0795774715459476679f;  // a point in the unit ball: uniform direction
      break;
    }
    case MT_LAMBERTIAN: {  // material.cc:3-17 + mixture_pdf (rect_box.h:118-131)
      const float3 atten = tex_value(S, mi.y, sf.u, sf.v, sf.p);
      const Onb uvw(sf.n);
      const float cos_scale = cfg.semantics == 0 ? 1.f : 0.318309886183790671538f;
      float pdf;
      const float4 *lob = nullptr;
      float u = r.x;  // technique choice; rescaled to [0,1) for the technique chosen
      if (GUIDED && gv.lobes) lob = guide_entry(gv, sf.p, sf.n);
      // light sampling's share of the non-guide techniques: the plain
      // mixture's 0.5, or the guided render's light_share
      const float ls = !S.has_lights ? 0.f : (GUIDED && lob) ? gv.light_share : 0.5f;
      if (GUIDED && lob && u < gv.alpha) {
        dir = guide_sample(lob, u / gv.alpha, r.z, r.w);
      } else {
        if (GUIDED && lob) u = (u - gv.alpha) / (1.f - gv.alpha);
        dir = u < ls ? light_random(S, sf.p, r.y, r.z, r.w) : uvw.local(cos_hemisphere(r.z, r.w));
      }
      {
        const float c = dot3(unit3(dir), uvw.w);
        const float pc = c > 0.f ? c * cos_scale : 0.f;
        pdf = ls > 0.f ? ls * light_pdf(S, sf.p, dir) + (1.f - ls) * pc : pc;
        if (GUIDED && lob) pdf = gv.alpha * guide_pdf(lob, unit3(dir)) + (1.f - gv.alpha) * pdf;
      }
      if (GUIDED && !rec.valid) rec = GuideRec{sf.p, sf.n, unit3(dir), T, L, true};
      if (sp) sp->pdf = pdf;
      const float cs = dot3(sf.n, unit3(dir));
      const float spdf = cs < 0.f ? 0.f : cs * 0.318309886183790671538f;
      wgt = atten * __fdividef(spdf, pdf);
      break;
    }
    default:  // diffuse_light and the base material: no scatter
      L = L + T * E;
      return false;
  }
  if (nonzero(E)) L = L + T * E;
  T = T * wgt;
  ray = Ray{sf.p, dir, time};
  return true;
}

__device__ __forceinline__ bool shade_vertex(const DevScene &S, const RenderCfg &cfg, Ray &ray, bool hit,
                                             const HitRef &h, float3 &T, float3 &L, int depth, uint32_t pixel,
                                             uint32_t sample) {
  GuideView gv{};
  GuideRec rec{};
  return shade_vertex_t<false>(S, cfg, ray, hit, h, T, L, depth, pixel, sample, gv, rec);
}

// utils.h:100-109
__device__ __forceinline__ float3 de_nan(float3 v) {
  return v3(isnan(v.x) ? 0.f : v.x, isnan(v.y) ? 0.f : v.y, isnan(v.z) ? 0.f : v.z);
}

}  // namespace tpt
#endif
