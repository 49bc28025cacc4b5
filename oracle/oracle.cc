// oracle.cc - CPU restatement of the tiny-path-tracer hot path.
//
// TEST INFRASTRUCTURE ONLY (see oracle.h).  Written from the reference's
// behaviour, organised as flat structs with switch dispatch instead of the
// reference's virtual class tree.  Arithmetic keeps the reference's types
// (float vectors, and double wherever the reference's expressions promote to
// double) so that closest-hit queries reproduce the reference bit for bit.
// Build with -ffp-contract=off: contraction into FMA would change bits.
//
// Reference files cited as path:line within BlurryLight/tiny-path-tracer.
#include "oracle.h"

#include <algorithm>
#include <atomic>
#include <cfloat>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <limits>
#include <random>
#include <sstream>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

namespace {

// ---------------------------------------------------------------- vec3 ----
// headers/vec3.h:6-157: three floats, component-wise float arithmetic.
struct V {
  float e[3];
  V() : e{0.f, 0.f, 0.f} {}
  V(float a, float b, float c) : e{a, b, c} {}
  float x() const { return e[0]; }
  float y() const { return e[1]; }
  float z() const { return e[2]; }
  float operator[](int i) const { return e[i]; }
  float &operator[](int i) { return e[i]; }
  float length() const { return std::sqrt(e[0] * e[0] + e[1] * e[1] + e[2] * e[2]); }
  float squared_length() const { return e[0] * e[0] + e[1] * e[1] + e[2] * e[2]; }
};
inline V operator+(const V &a, const V &b) { return V(a.e[0] + b.e[0], a.e[1] + b.e[1], a.e[2] + b.e[2]); }
inline V operator-(const V &a, const V &b) { return V(a.e[0] - b.e[0], a.e[1] - b.e[1], a.e[2] - b.e[2]); }
inline V operator-(const V &a) { return V(-a.e[0], -a.e[1], -a.e[2]); }
inline V operator*(const V &a, const V &b) { return V(a.e[0] * b.e[0], a.e[1] * b.e[1], a.e[2] * b.e[2]); }
inline V operator*(const V &a, float t) { return V(a.e[0] * t, a.e[1] * t, a.e[2] * t); }
inline V operator*(float t, const V &a) { return V(a.e[0] * t, a.e[1] * t, a.e[2] * t); }
inline V operator/(const V &a, float t) { return V(a.e[0] / t, a.e[1] / t, a.e[2] / t); }
inline float dot(const V &a, const V &b) { return a.e[0] * b.e[0] + a.e[1] * b.e[1] + a.e[2] * b.e[2]; }
inline V cross(const V &a, const V &b) {
  return V(a.e[1] * b.e[2] - b.e[1] * a.e[2], a.e[2] * b.e[0] - b.e[2] * a.e[0],
           a.e[0] * b.e[1] - b.e[0] * a.e[1]);
}
inline V unit(const V &v) { return v / v.length(); }  // vec3.h:143-144
inline V vmin(const V &a, const V &b) {
  return V(std::min(a.e[0], b.e[0]), std::min(a.e[1], b.e[1]), std::min(a.e[2], b.e[2]));
}
inline V vmax(const V &a, const V &b) {
  return V(std::max(a.e[0], b.e[0]), std::max(a.e[1], b.e[1]), std::max(a.e[2], b.e[2]));
}

struct Ray {
  V o, d;
  float time = 0.f;
  V at(float t) const { return o + t * d; }  // ray.h:13
};

struct Box {
  V mn, mx;
};

// aabb.cc:3-19 - slab test with the reciprocal, swap on a negative
// reciprocal, early exit when the interval empties.
inline bool box_hit(const Box &b, const Ray &r, float tmin, float tmax) {
  for (int i = 0; i < 3; i++) {
    float inv = 1.0f / r.d[i];
    float t0 = (b.mn[i] - r.o[i]) * inv;
    float t1 = (b.mx[i] - r.o[i]) * inv;
    if (inv < 0.0f) std::swap(t0, t1);
    tmin = t0 > tmin ? t0 : tmin;
    tmax = t1 < tmax ? t1 : tmax;
    if (tmin > tmax) return false;
  }
  return true;
}

// aabb.cc:21-30 (float_min / float_max of utils.h:23-24)
inline Box surround(const Box &a, const Box &b) {
  auto fmn = [](float p, float q) { return p < q ? p : q; };
  auto fmx = [](float p, float q) { return p > q ? p : q; };
  return Box{V(fmn(a.mn.x(), b.mn.x()), fmn(a.mn.y(), b.mn.y()), fmn(a.mn.z(), b.mn.z())),
             V(fmx(a.mx.x(), b.mx.x()), fmx(a.mx.y(), b.mx.y()), fmx(a.mx.z(), b.mx.z()))};
}

// ---------------------------------------------------------------- RNG -----
// utils.cc:28-32: drand_r = uniform_real_distribution<double>(min,max) over a
// std::mt19937.  The oracle owns the engine explicitly.
struct Rng {
  std::mt19937 gen;
  double operator()(double a = 0.0, double b = 1.0) {
    std::uniform_real_distribution<double> dis(a, b);
    return dis(gen);
  }
};

// Philox-4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as
// easy as 1, 2, 3", SC'11): ten rounds of the 4x32 multiply-xor bijection,
// with the Weyl key schedule between rounds.
void philox10(const uint32_t c_in[4], const uint32_t k_in[2], uint32_t out[4]) {
  uint32_t c[4] = {c_in[0], c_in[1], c_in[2], c_in[3]};
  uint32_t k0 = k_in[0], k1 = k_in[1];
  for (int round = 0; round < 10; round++) {
    uint64_t p0 = (uint64_t)0xD2511F53u * c[0];
    uint64_t p1 = (uint64_t)0xCD9E8D57u * c[2];
    uint32_t n0 = (uint32_t)(p1 >> 32) ^ c[1] ^ k0;
    uint32_t n1 = (uint32_t)p1;
    uint32_t n2 = (uint32_t)(p0 >> 32) ^ c[3] ^ k1;
    uint32_t n3 = (uint32_t)p0;
    c[0] = n0; c[1] = n1; c[2] = n2; c[3] = n3;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  out[0] = c[0]; out[1] = c[1]; out[2] = c[2]; out[3] = c[3];
}
inline float u01(uint32_t x) { return (float)(x >> 8) * (1.0f / 16777216.0f); }

// Free-flight uniform of a constant_medium in trace queries (media_mode 0);
// the product computes the same value on the GPU.
float medium_uniform(uint64_t seed, uint64_t ray_index, int32_t medium_id) {
  uint32_t ctr[4] = {(uint32_t)ray_index, (uint32_t)(ray_index >> 32), (uint32_t)medium_id, 0x4d454449u};
  uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
  uint32_t o[4];
  philox10(ctr, key, o);
  return u01(o[0]);
}

// ------------------------------------------------------------ scene -------
enum Kind {
  K_SPHERE = 1, K_MSPHERE, K_XY, K_XZ, K_YZ, K_FLIP, K_BOX, K_TRANSLATE,
  K_ROTY, K_MEDIUM, K_LIST, K_BVH
};
enum TexKind { T_CONST = 1, T_CHECKER, T_PERLIN, T_IMAGE };
enum MatKind { M_LAMB = 1, M_METAL, M_DIEL, M_LIGHT, M_ISO };

struct Tex {
  int kind = 0;
  V c;
  int odd = -1, even = -1;
  float scale = 1.f;
  int w = 0, h = 0;
  std::vector<uint8_t> px;
};
struct Mat {
  int kind = 0;
  int tex = -1;
  V albedo;
  float fuzz = 0.f, ior = 1.f;
};
struct Node {
  int kind = 0;
  int sd = -1;             // SD id of the statement (-1 for internal nodes)
  int mat = -1;
  V c0, c1;                // sphere centre / moving-sphere centres
  float r = 0.f, t0 = 0.f, t1 = 0.f;
  float a0 = 0, a1 = 0, b0 = 0, b1 = 0, k = 0;  // rect bounds and plane
  V pmin, pmax;            // box
  int child = -1;          // flip / translate / rotate / medium boundary
  V off;                   // translate
  float sn = 0.f, cs = 1.f;  // rotate_y
  bool has_box = false;
  Box rbox;
  float density = 0.f;     // medium
  int phase = -1;          // medium phase material (isotropic)
  std::vector<int> items;  // list items / box faces
  int left = -1, right = -1;
  Box bbox;                // bvh node box
};

struct Scene {
  std::vector<Tex> texs;
  std::vector<Mat> mats;
  std::vector<Node> nodes;
  std::unordered_map<int, int> node_of_sd, tex_of_sd, mat_of_sd;
  int world = -1, lights = -1;
  bool has_cam = false;
  // camera (camera.cc:2-21)
  V cam_o, cam_ll, cam_h, cam_v, cam_u, cam_vv, cam_w;
  float lens_r = 0.f, ct0 = 0.f, ct1 = 0.f;
  // perlin tables (perlin_noise.h:13-16; shared by all perlin textures)
  V pgrad[256];
  int pperm[3][256];
  bool has_perlin = false;
  int n_internal = 0;
};

// ------------------------------------------------------- bounding boxes ---
bool bounding_box(const Scene &S, int n, float t0, float t1, Box &out);

inline V msphere_center(const Node &nd, float time) {  // sphere.h:29-32
  return nd.c0 + (time - nd.t0) / (nd.t1 - nd.t0) * (nd.c1 - nd.c0);
}

bool bounding_box(const Scene &S, int n, float t0, float t1, Box &out) {
  const Node &nd = S.nodes[n];
  switch (nd.kind) {
    case K_SPHERE:  // sphere.cc:87-91
      out = Box{nd.c0 - V(nd.r, nd.r, nd.r), nd.c0 + V(nd.r, nd.r, nd.r)};
      return true;
    case K_MSPHERE: {  // sphere.cc:77-85
      V ca = msphere_center(nd, t0), cb = msphere_center(nd, t1);
      Box a{ca - V(nd.r, nd.r, nd.r), ca + V(nd.r, nd.r, nd.r)};
      Box b{cb - V(nd.r, nd.r, nd.r), cb + V(nd.r, nd.r, nd.r)};
      out = surround(a, b);
      return true;
    }
    case K_XY:  // rect_box.cc:3-6 (padding 0.0001 evaluated in double)
      out = Box{V(nd.a0, nd.b0, (float)(nd.k - 0.0001)), V(nd.a1, nd.b1, (float)(nd.k + 0.0001))};
      return true;
    case K_XZ:  // rect_box.cc:45-49
      out = Box{V(nd.a0, (float)(nd.k - 0.0001), nd.b0), V(nd.a1, (float)(nd.k + 0.0001), nd.b1)};
      return true;
    case K_YZ:  // rect_box.cc:70-73
      out = Box{V((float)(nd.k - 0.0001), nd.a0, nd.b0), V((float)(nd.k + 0.0001), nd.a1, nd.b1)};
      return true;
    case K_FLIP:  // rect_box.h:47-49
    case K_MEDIUM:  // hitable.h:64-66
      return bounding_box(S, nd.child, t0, t1, out);
    case K_BOX:  // rect_box.h:66-69
      out = Box{nd.pmin, nd.pmax};
      return true;
    case K_TRANSLATE: {  // rect_box.h:80-86
      if (!bounding_box(S, nd.child, t0, t1, out)) return false;
      out = Box{out.mn + nd.off, out.mx + nd.off};
      return true;
    }
    case K_ROTY:  // rect_box.h:104-107
      out = nd.rbox;
      return nd.has_box;
    case K_LIST: {  // hitable_list.cc:3-22
      if (nd.items.empty()) return false;
      Box tmp;
      if (!bounding_box(S, nd.items[0], t0, t1, tmp)) return false;
      out = tmp;
      for (size_t i = 1; i < nd.items.size(); i++) {
        if (!bounding_box(S, nd.items[i], t0, t1, tmp)) return false;
        out = surround(out, tmp);
      }
      return true;
    }
    case K_BVH:  // hitable.cc:58-61
      out = nd.bbox;
      return true;
  }
  return false;
}

// ------------------------------------------------------ BVH build ---------
// hitable.cc:32-56: random axis from drand_r(0,3), std::sort of the slice by
// box.min[axis] (box taken at times 0,0, comparator hitable.cc:10-30), median
// split n/2; n==1 duplicates the item, n==2 keeps the pair.
int build_bvh(Scene &S, Rng &rng, int *l, int n, float t0, float t1, std::string &err) {
  int axis = int(rng(0, 3.0));
  auto cmp = [&S, &err, axis](int a, int b) {
    Box ba, bb;
    bool ha = bounding_box(S, a, 0, 0, ba), hb = bounding_box(S, b, 0, 0, bb);
    if (!ha || !hb) {
      err = "No bounding box in BVH node constructor";
      return false;
    }
    return !std::isgreaterequal(ba.mn[axis], bb.mn[axis]);
  };
  if (axis < 0 || axis > 2) axis = 2;
  std::sort(l, l + n, cmp);
  Node nd;
  nd.kind = K_BVH;
  if (n == 1) {
    nd.left = nd.right = l[0];
  } else if (n == 2) {
    nd.left = l[0];
    nd.right = l[1];
  } else {
    nd.left = build_bvh(S, rng, l, n / 2, t0, t1, err);
    nd.right = build_bvh(S, rng, l + n / 2, n - n / 2, t0, t1, err);
  }
  Box bl, br;
  if (!bounding_box(S, nd.left, t0, t1, bl) || !bounding_box(S, nd.right, t0, t1, br))
    err = "no bounding box in bvh constructor";
  nd.bbox = surround(bl, br);
  S.nodes.push_back(nd);
  S.n_internal++;
  return (int)S.nodes.size() - 1;
}

// rect_box.cc:142-190: rotate_y constructor - angle to radians through double,
// float sin/cos, and the column-wise min/max box transform.
void init_rotate(Scene &S, Node &nd, float angle) {
  float radians = angle / 180.0f * M_PI;
  nd.sn = std::sin(radians);
  nd.cs = std::cos(radians);
  Box b;
  nd.has_box = bounding_box(S, nd.child, 0, 0, b);
  V c1(nd.cs, 0, -nd.sn), c2(0, 1, 0), c3(nd.sn, 0, nd.cs);
  V xa = c1 * b.mx.x(), xb = c1 * b.mn.x();
  V ya = c2 * b.mx.y(), yb = c2 * b.mn.y();
  V za = c3 * b.mx.z(), zb = c3 * b.mn.z();
  nd.rbox = Box{vmin(xa, xb) + vmin(ya, yb) + vmin(za, zb), vmax(xa, xb) + vmax(ya, yb) + vmax(za, zb)};
}

// -------------------------------------------------------- hit record ------
struct Hit {
  float t = 0.f, u = 0.f, v = 0.f;
  V p, n;
  int mat = -1;   // material index
  int prim = -1;  // SD id of the leaf primitive
};

struct Ctx {
  const Scene *S;
  Rng *rng = nullptr;          // media_mode 1 / rendering
  bool philox_media = false;   // media_mode 0
  uint64_t seed = 0, ray_index = 0;
  oracle_counters *cnt = nullptr;
  double draw() { return (*rng)(); }
};

// utils.h:38-43
inline void uv_map(const V &p, float &u, float &v) {
  u = std::atan2(p.z(), p.x()) / (2 * M_PI);
  v = std::asin(p.y()) / M_PI;
  u += 0.5f;
  v += 0.5f;
}

bool hit(Ctx &C, int n, const Ray &r, float tmin, float tmax, Hit &rec);

// sphere.cc:13-43 (and 45-75 for the moving sphere).  The root is evaluated
// in double: unqualified sqrt on a float resolves to ::sqrt(double).
inline bool sphere_hit(const V &center, float radius, const V &uv_center, int mat, int prim,
                       const Ray &r, float tmin, float tmax, Hit &rec) {
  V oc = r.o - center;
  float a = dot(r.d, r.d);
  float b = 2.0 * dot(r.d, oc);
  float c = dot(oc, oc) - radius * radius;
  float disc = b * b - 4 * a * c;
  if (disc > 0) {
    float temp = (-b - ::sqrt(b * b - 4 * a * c)) / (2 * a);
    if (temp < tmax && temp > tmin) {
      rec.t = temp;
      rec.p = r.at(temp);
      uv_map((rec.p - uv_center) / radius, rec.u, rec.v);
      rec.n = (rec.p - center) / radius;
      rec.mat = mat;
      rec.prim = prim;
      return true;
    }
    temp = (-b + ::sqrt(b * b - 4 * a * c)) / (2 * a);
    if (temp < tmax && temp > tmin) {
      rec.t = temp;
      rec.p = r.at(temp);
      uv_map((rec.p - uv_center) / radius, rec.u, rec.v);
      rec.n = (rec.p - center) / radius;
      rec.mat = mat;
      rec.prim = prim;
      return true;
    }
  }
  return false;
}

// rect_box.cc:8-24, 51-68, 75-91: plane axis `ax`, in-plane axes (ia, ib).
inline bool rect_hit(const Node &nd, int ax, int ia, int ib, const Ray &r, float tmin,
                     float tmax, Hit &rec) {
  float t = (nd.k - r.o[ax]) / r.d[ax];
  if (t > tmax || t < tmin) return false;
  float a = r.o[ia] + t * r.d[ia];
  float b = r.o[ib] + t * r.d[ib];
  if (a < nd.a0 || a > nd.a1 || b < nd.b0 || b > nd.b1) return false;
  rec.u = (a - nd.a0) / (nd.a1 - nd.a0);
  rec.v = (b - nd.b0) / (nd.b1 - nd.b0);
  rec.t = t;
  rec.mat = nd.mat;
  rec.p = r.at(t);
  V nn(0, 0, 0);
  nn[ax] = 1;
  rec.n = nn;
  rec.prim = nd.sd;
  return true;
}

// hitable_list.cc:38-51: sequential, shrinking closest_so_far (a double).
bool list_hit(Ctx &C, const std::vector<int> &items, const Ray &r, float tmin, float tmax,
              Hit &rec) {
  Hit tmp;
  bool any = false;
  double closest = tmax;
  for (int it : items) {
    if (hit(C, it, r, tmin, closest, tmp)) {
      any = true;
      closest = tmp.t;
      rec = tmp;
    }
  }
  return any;
}

bool hit(Ctx &C, int n, const Ray &r, float tmin, float tmax, Hit &rec) {
  const Scene &S = *C.S;
  const Node &nd = S.nodes[n];
  switch (nd.kind) {
    case K_SPHERE:
      if (C.cnt) C.cnt->sphere_tests++;
      return sphere_hit(nd.c0, nd.r, nd.c0, nd.mat, nd.sd, r, tmin, tmax, rec);
    case K_MSPHERE: {
      if (C.cnt) C.cnt->sphere_tests++;
      V c = msphere_center(nd, r.time);
      return sphere_hit(c, nd.r, nd.c0, nd.mat, nd.sd, r, tmin, tmax, rec);
    }
    case K_XY:
      if (C.cnt) C.cnt->rect_tests++;
      return rect_hit(nd, 2, 0, 1, r, tmin, tmax, rec);
    case K_XZ:
      if (C.cnt) C.cnt->rect_tests++;
      return rect_hit(nd, 1, 0, 2, r, tmin, tmax, rec);
    case K_YZ:
      if (C.cnt) C.cnt->rect_tests++;
      return rect_hit(nd, 0, 1, 2, r, tmin, tmax, rec);
    case K_FLIP:  // rect_box.h:50-57
      if (hit(C, nd.child, r, tmin, tmax, rec)) {
        rec.n = -rec.n;
        return true;
      }
      return false;
    case K_BOX: {  // rect_box.cc:117-119 -> list of six faces
      bool h = list_hit(C, nd.items, r, tmin, tmax, rec);
      if (h) rec.prim = nd.sd;
      return h;
    }
    case K_LIST:
      return list_hit(C, nd.items, r, tmin, tmax, rec);
    case K_TRANSLATE: {  // rect_box.h:87-95
      if (C.cnt) C.cnt->instance_xforms++;
      Ray moved{r.o - nd.off, r.d, r.time};
      if (hit(C, nd.child, moved, tmin, tmax, rec)) {
        rec.p = rec.p + nd.off;
        return true;
      }
      return false;
    }
    case K_ROTY: {  // rect_box.cc:171-195
      if (C.cnt) C.cnt->instance_xforms++;
      V o = r.o, d = r.d;
      o[0] = nd.cs * r.o[0] - nd.sn * r.o[2];
      o[2] = nd.sn * r.o[0] + nd.cs * r.o[2];
      d[0] = nd.cs * r.d[0] - nd.sn * r.d[2];
      d[2] = nd.sn * r.d[0] + nd.cs * r.d[2];
      Ray rr{o, d, r.time};
      if (hit(C, nd.child, rr, tmin, tmax, rec)) {
        V p = rec.p, nn = rec.n;
        p[0] = nd.cs * rec.p[0] + nd.sn * rec.p[2];
        p[2] = -nd.sn * rec.p[0] + nd.cs * rec.p[2];
        nn[0] = nd.cs * rec.n[0] + nd.sn * rec.n[2];
        nn[2] = -nd.sn * rec.n[0] + nd.cs * rec.n[2];
        rec.p = p;
        rec.n = nn;
        return true;
      }
      return false;
    }
    case K_MEDIUM: {  // hitable.cc:98-128
      if (C.cnt) C.cnt->medium_tests++;
      Hit r1, r2;
      if (hit(C, nd.child, r, std::numeric_limits<float>::lowest(),
              std::numeric_limits<float>::max(), r1)) {
        if (hit(C, nd.child, r, r1.t + 0.0001, std::numeric_limits<float>::max(), r2)) {
          if (r1.t < tmin) r1.t = tmin;
          if (r2.t > tmax) r2.t = tmax;
          if (r1.t >= r2.t) return false;
          float inside = (r2.t - r1.t) * r.d.length();
          double u = C.philox_media ? (double)medium_uniform(C.seed, C.ray_index, nd.sd) : C.draw();
          float dist = (-1 / nd.density) * std::log(u);
          if (dist < inside) {
            rec.t = r1.t + dist / r.d.length();
            rec.p = r.at(rec.t);
            if (C.philox_media) {
              rec.n = V(1, 0, 0);
            } else {
              // vec3(drand_r(), drand_r(), drand_r()): g++ evaluates the
              // arguments last to first; make_unit_vector scales by 1.0/len.
              double z = C.draw(), y = C.draw(), x = C.draw();
              V nn((float)x, (float)y, (float)z);
              float k = 1.0 / nn.length();
              rec.n = V(nn.e[0] * k, nn.e[1] * k, nn.e[2] * k);
            }
            // rec.u / rec.v are left as the caller's record held them.
            rec.mat = nd.phase;
            rec.prim = nd.sd;
            return true;
          }
        }
      }
      return false;
    }
    case K_BVH: {  // hitable.cc:63-90: both children, same interval, ties -> right
      if (C.cnt) C.cnt->aabb_tests++;
      if (box_hit(nd.bbox, r, tmin, tmax)) {
        Hit lr, rr;
        bool hl = hit(C, nd.left, r, tmin, tmax, lr);
        bool hr = hit(C, nd.right, r, tmin, tmax, rr);
        if (hl && hr) {
          rec = (lr.t < rr.t) ? lr : rr;
          return true;
        } else if (hl) {
          rec = lr;
          return true;
        } else if (hr) {
          rec = rr;
          return true;
        }
        return false;
      }
      return false;
    }
  }
  return false;
}


// ------------------------------------------------------------ textures ----
// utils.cc:160-225 (noise, turb, quintic-fade gradient interpolation).
float perlin_noise(const Scene &S, const V &p) {
  float u = p.x() - std::floor(p.x());
  float v = p.y() - std::floor(p.y());
  float w = p.z() - std::floor(p.z());
  int i = int(std::floor(p.x())) & 255;
  int j = int(std::floor(p.y())) & 255;
  int k = int(std::floor(p.z())) & 255;
  V c[2][2][2];
  for (int di = 0; di < 2; di++)
    for (int dj = 0; dj < 2; dj++)
      for (int dk = 0; dk < 2; dk++)
        c[di][dj][dk] = S.pgrad[S.pperm[0][(i + di) & 255] ^ S.pperm[1][(j + dj) & 255] ^
                                S.pperm[2][(k + dk) & 255]];
  auto fade = [](float x) {
    return (float)(6 * std::pow(x, 5) - 15 * std::pow(x, 4) + 10 * std::pow(x, 3));
  };
  u = fade(u);
  v = fade(v);
  w = fade(w);
  float acc = 0.0f;
  for (int di = 0; di < 2; di++)
    for (int dj = 0; dj < 2; dj++)
      for (int dk = 0; dk < 2; dk++) {
        V wv(u - di, v - dj, w - dk);
        acc += (di * u + (1 - di) * (1 - u)) * (dj * v + (1 - dj) * (1 - v)) *
               (dk * w + (1 - dk) * (1 - w)) * dot(c[di][dj][dk], wv);
      }
  return std::abs(acc);
}
float perlin_turb(const Scene &S, const V &p) {  // utils.cc:193-203
  float acc = 0;
  V tmp = p;
  float weight = 1.0;
  for (int i = 0; i < 5; i++) {
    acc += weight * perlin_noise(S, tmp);
    weight *= 0.5;
    tmp = tmp * 2.0f;
  }
  return std::abs(acc);
}

V tex_value(const Scene &S, int t, float u, float v, const V &p) {
  for (int guard = 0; guard < 64; guard++) {
    const Tex &tx = S.texs[t];
    switch (tx.kind) {
      case T_CONST:  // texture.h:15-24
        return tx.c;
      case T_CHECKER: {  // texture.cc:4-16
        float s = std::sin(10 * p.x()) * std::sin(10 * p.y()) * std::sin(10 * p.z());
        t = std::isless(s, 0.0f) ? tx.odd : tx.even;
        continue;
      }
      case T_PERLIN:  // texture.cc:18-25 (turb ignores scale)
        return V(1, 1, 1) * 0.5f * (1 + std::sin(tx.scale * p.z() + 10 * perlin_turb(S, p)));
      case T_IMAGE: {  // texture.cc:27-42
        int i = u * tx.w;
        int j = (1 - v) * tx.h;
        if (i < 0) i = 0;
        if (i > tx.w - 1) i = tx.w - 1;
        if (j > tx.h - 1) j = tx.h - 1;
        if (j < 0) j = 0;
        const uint8_t *q = &tx.px[3 * (size_t)i + 3 * (size_t)tx.w * j];
        return V(int(q[0]) / 255.0f, int(q[1]) / 255.0f, int(q[2]) / 255.0f);
      }
    }
    break;
  }
  return V(0, 0, 0);
}

// ----------------------------------------------------------- samplers -----
struct Sampler {  // per-thread drand_r stream
  Rng rng;
  double operator()() { return rng(); }
};

V random_in_unit_disk(Sampler &R) {  // utils.cc:13-19
  V p;
  do {
    double a = R(), b = R();
    p = 2.0f * V((float)a, (float)b, 0) - V(1, 1, 0);
  } while (dot(p, p) >= 1.0);
  return p;
}
V random_in_unit_sphere(Sampler &R) {  // utils.cc:21-27
  V p;
  do {
    double a = R(), b = R(), c = R();
    p = 2.0f * V((float)a, (float)b, (float)c) - V(1, 1, 1);
  } while (p.length() >= 1.0);
  return p;
}
V random_on_hemisphere(Sampler &R) {  // utils.cc:427-435 (cosine-weighted)
  float r1 = R();
  float r2 = R();
  float phi = 2 * M_PI * r1;
  return V(std::cos(phi) * std::sqrt(r2), std::sin(phi) * std::sqrt(r2), std::sqrt(1 - r2));
}
V reflect(const V &v, const V &n) { return v - 2 * dot(v, n) * n; }  // utils.cc:53-56
bool refract(const V &v, const V &n, float ni_nt, V &out) {  // utils.cc:34-44
  V uv = unit(v);
  float dt = dot(uv, n);
  float disc = 1.0 - ni_nt * ni_nt * (1 - dt * dt);
  if (disc > 0) {
    out = ni_nt * (uv - n * dt) - n * (float)::sqrt(disc);
    return true;
  }
  return false;
}
float schlick(float c, float ri) {  // utils.cc:46-51
  float r0 = (1 - ri) / (1 + ri);
  r0 = r0 * r0;
  return r0 + (1 - r0) * ::pow((1 - c), 5);
}

struct Onb {  // utils.h:47-63, utils.cc:437-450
  V a[3];
  explicit Onb(const V &n) {
    a[2] = n;
    V tmp = std::abs(n.x()) > 0.9 ? V(0, 1, 0) : V(1, 0, 0);
    a[1] = unit(cross(n, tmp));
    a[0] = cross(a[1], a[2]);
  }
  V local(float x, float y, float z) const { return x * a[0] + y * a[1] + z * a[2]; }
  V local(const V &v) const { return v.x() * a[0] + v.y() * a[1] + v.z() * a[2]; }
};

// ------------------------------------------------------ light shapes ------
// hitable::pdf_value / random defaults (hitable.h:35-38), xz_rect
// (rect_box.cc:26-43), sphere (sphere.cc:93-120), hitable_list
// (hitable_list.cc:24-36).
float light_pdf(Ctx &C, int n, const V &o, const V &d) {
  const Node &nd = C.S->nodes[n];
  if (C.cnt) C.cnt->light_pdf_evals++;
  switch (nd.kind) {
    case K_XZ: {
      Hit rec;
      if (rect_hit(nd, 1, 0, 2, Ray{o, d, 0.f}, 0.0001, std::numeric_limits<float>::max(), rec)) {
        float area = std::abs((nd.a1 - nd.a0) * (nd.b1 - nd.b0));
        float d2 = (rec.t * d).squared_length();
        float cosine = std::abs(dot(d, rec.n) / d.length());
        return d2 / (cosine * area);
      }
      return 0.0f;
    }
    case K_SPHERE: {
      Hit rec;
      if (sphere_hit(nd.c0, nd.r, nd.c0, nd.mat, nd.sd, Ray{o, d, 0.f}, 0.001,
                     std::numeric_limits<float>::max(), rec)) {
        float tmp = (nd.r * nd.r) / (nd.c0 - o).squared_length();
        float cmax = ::sqrt(1 - tmp);
        float solid = 2 * M_PI * (1 - cmax);
        if (std::isnan(solid)) return 0;
        return 1 / solid;
      }
      return 0;
    }
    case K_LIST: {
      float w = 1.0 / nd.items.size();
      float sum = 0;
      for (int it : nd.items) sum += w * light_pdf(C, it, o, d);
      return sum;
    }
    default:
      return 0.0;
  }
}
V light_random(Ctx &C, Sampler &R, int n, const V &o) {
  const Node &nd = C.S->nodes[n];
  switch (nd.kind) {
    case K_XZ: {
      float x = nd.a0 + R() * (nd.a1 - nd.a0);
      float z = nd.b0 + R() * (nd.b1 - nd.b0);
      return V(x, nd.k, z) - o;
    }
    case K_SPHERE: {
      V dir = nd.c0 - o;
      Onb uvw(unit(dir));
      float tmp = (nd.r * nd.r) / (nd.c0 - o).squared_length();
      float cmax = ::sqrt(1 - tmp);
      float r1 = R();
      float r2 = R();
      float z = 1 + r2 * (cmax - 1);
      float x = std::cos(2 * M_PI * r1) * std::sqrt(1 - z * z);
      float y = std::sin(2 * M_PI * r1) * std::sqrt(1 - z * z);
      return uvw.local(x, y, z);
    }
    case K_LIST: {
      int idx = int(R() * nd.items.size());
      if (idx >= (int)nd.items.size()) idx = (int)nd.items.size() - 1;
      return light_random(C, R, nd.items[idx], o);
    }
    default:
      return V(1, 0, 0);
  }
}

// ------------------------------------------------------------ color() -----
struct RenderCfg {
  int max_depth = 50;
  int semantics = 0;
  int background = 0;
  float sky_scale = 1.f;
};

V background(const RenderCfg &cfg, const Ray &r) {  // utils.cc:85-90
  if (cfg.background == 0) return V(0, 0, 0);
  V ud = unit(r.d);
  float t = (ud.y() + 1.0f) * 0.5f;
  return cfg.sky_scale * ((1 - t) * V(1.0f, 1.0f, 1.0f) + t * V(0.5f, 0.7f, 1.0f));
}

// utils.cc:58-94.  Recursive estimator; materials material.cc:3-98.
V color(Ctx &C, Sampler &R, const RenderCfg &cfg, const Ray &r, int depth) {
  const Scene &S = *C.S;
  Hit rec;
  if (C.cnt) C.cnt->segments++;
  if (!hit(C, S.world, r, 0.001, std::numeric_limits<float>::max(), rec)) return background(cfg, r);
  const Mat &m = S.mats[rec.mat];
  V emitted(0, 0, 0);
  if (m.kind == M_LIGHT && dot(rec.n, r.d) < 0) emitted = tex_value(S, m.tex, rec.u, rec.v, rec.p);
  if (depth >= cfg.max_depth) return emitted;
  switch (m.kind) {
    case M_METAL: {  // material.cc:88-98
      if (C.cnt) C.cnt->metal++;
      V refl = reflect(unit(r.d), rec.n);
      Ray sr{rec.p, refl + m.fuzz * random_in_unit_sphere(R), r.time};
      if (!(dot(sr.d, rec.n) > 0)) return emitted;
      return m.albedo * color(C, R, cfg, sr, depth + 1);
    }
    case M_DIEL: {  // material.cc:19-70
      if (C.cnt) C.cnt->dielectric++;
      V outward, refr;
      V refl = reflect(r.d, rec.n);
      float ni_nt, cosine, prob;
      if (dot(r.d, rec.n) > 0) {
        outward = -rec.n;
        ni_nt = m.ior;
        cosine = dot(r.d, rec.n) / r.d.length();
        cosine = std::sqrt(1 - m.ior * m.ior * (1 - cosine * cosine));
      } else {
        outward = rec.n;
        ni_nt = 1.0 / m.ior;
        cosine = -dot(r.d, rec.n) / r.d.length();
      }
      if (refract(r.d, outward, ni_nt, refr))
        prob = schlick(cosine, m.ior);
      else
        prob = 1.0;
      Ray sr{rec.p, (R() < prob) ? refl : refr, r.time};
      return V(1.0f, 1.0f, 1.0f) * color(C, R, cfg, sr, depth + 1);
    }
    case M_ISO: {  // material.cc:72-77; hidden in reference semantics
      if (cfg.semantics == 0) return emitted;
      Ray sr{rec.p, random_in_unit_sphere(R), 0.0f};
      return tex_value(S, m.tex, rec.u, rec.v, rec.p) * color(C, R, cfg, sr, depth + 1);
    }
    case M_LAMB: {  // material.cc:3-17 + utils.cc:73-81
      if (C.cnt) C.cnt->lambertian++;
      V atten = tex_value(S, m.tex, rec.u, rec.v, rec.p);
      Onb uvw(rec.n);
      V dir;
      float pdf;
      const float inv_pi = cfg.semantics == 0 ? 1.0f : (float)(1.0 / M_PI);
      auto cos_value = [&](const V &d) {
        float c = dot(unit(d), uvw.a[2]);
        return c > 0 ? c * (cfg.semantics == 0 ? 1.0f : inv_pi) : 0.0f;
      };
      if (S.lights >= 0) {  // mixture_pdf (rect_box.h:118-131)
        if (R() < 0.5)
          dir = light_random(C, R, S.lights, rec.p);
        else
          dir = uvw.local(random_on_hemisphere(R));
        pdf = 0.5 * light_pdf(C, S.lights, rec.p, dir) + 0.5 * cos_value(dir);
      } else {
        dir = uvw.local(random_on_hemisphere(R));
        pdf = cos_value(dir);
      }
      Ray sr{rec.p, dir, r.time};
      float c = dot(rec.n, unit(sr.d));
      float spdf = c < 0 ? 0.0f : (float)(c / M_PI);
      return emitted + atten * spdf * color(C, R, cfg, sr, depth + 1) / pdf;
    }
    default:
      return emitted;
  }
}

// camera.cc:23-31
Ray camera_ray(const Scene &S, Sampler &R, float s, float t) {
  V rd = S.lens_r * random_in_unit_disk(R);
  V off = S.cam_u * rd.x() + S.cam_vv * rd.y();
  float time = S.ct0 + R() * (S.ct1 - S.ct0);
  return Ray{S.cam_o + off, S.cam_ll + s * S.cam_h + t * S.cam_v - S.cam_o - off, time};
}

inline V de_nan(V v) {  // utils.h:100-109
  for (int i = 0; i < 3; i++)
    if (std::isnan(v[i])) v[i] = 0;
  return v;
}

// ------------------------------------------------------------ SD parser ---
struct Parser {
  Scene &S;
  Rng build_rng;  // drand_r stream for BVH construction: fresh default seed
  std::string err;
  explicit Parser(Scene &s) : S(s) {}

  int node_ref(int sd) {
    auto it = S.node_of_sd.find(sd);
    if (it == S.node_of_sd.end()) {
      err = "undefined node " + std::to_string(sd);
      return -1;
    }
    return it->second;
  }
  int mat_ref(int sd) {
    auto it = S.mat_of_sd.find(sd);
    if (it == S.mat_of_sd.end()) {
      err = "undefined material " + std::to_string(sd);
      return -1;
    }
    return it->second;
  }
  int tex_ref(int sd) {
    auto it = S.tex_of_sd.find(sd);
    if (it == S.tex_of_sd.end()) {
      err = "undefined texture " + std::to_string(sd);
      return -1;
    }
    return it->second;
  }
  int add(Node nd, int sd) {
    nd.sd = sd;
    S.nodes.push_back(nd);
    int idx = (int)S.nodes.size() - 1;
    S.node_of_sd[sd] = idx;
    return idx;
  }
  int add_internal(Node nd) {
    S.nodes.push_back(nd);
    return (int)S.nodes.size() - 1;
  }

  bool line(const std::string &ln) {
    std::istringstream is(ln);
    std::string kw;
    if (!(is >> kw) || kw[0] == '#') return true;
    auto F = [&is, this]() -> float {
      std::string s;
      if (!(is >> s)) { err = "missing number"; return 0.f; }
      return std::strtof(s.c_str(), nullptr);
    };
    auto I = [&is, this]() -> int {
      long v;
      if (!(is >> v)) { err = "missing integer"; return -1; }
      return (int)v;
    };
    if (kw == "tex") {
      int id = I();
      std::string ty;
      is >> ty;
      Tex t;
      if (ty == "const") { t.kind = T_CONST; float r = F(), g = F(), b = F(); t.c = V(r, g, b); }
      else if (ty == "checker") { t.kind = T_CHECKER; t.odd = tex_ref(I()); t.even = tex_ref(I()); }
      else if (ty == "perlin") { t.kind = T_PERLIN; t.scale = F(); }
      else if (ty == "image") {
        t.kind = T_IMAGE; t.w = I(); t.h = I();
        uint32_t seed = (uint32_t)I();
        if (t.w <= 0 || t.h <= 0) { err = "bad image size"; return false; }
        t.px.resize((size_t)t.w * t.h * 3);
        oracle_procedural_image(t.w, t.h, seed, t.px.data());
      } else { err = "unknown texture " + ty; return false; }
      S.texs.push_back(t);
      S.tex_of_sd[id] = (int)S.texs.size() - 1;
    } else if (kw == "perlin_tables") {
      for (int i = 0; i < 256; i++) { float x = F(), y = F(), z = F(); S.pgrad[i] = V(x, y, z); }
      for (int a = 0; a < 3; a++)
        for (int i = 0; i < 256; i++) S.pperm[a][i] = I() & 255;
      S.has_perlin = true;
    } else if (kw == "mat") {
      int id = I();
      std::string ty;
      is >> ty;
      Mat m;
      if (ty == "lambertian") { m.kind = M_LAMB; m.tex = tex_ref(I()); }
      else if (ty == "metal") {  // material.h:41-46 fuzz clamp
        m.kind = M_METAL; float r = F(), g = F(), b = F(); m.albedo = V(r, g, b);
        float fz = F();
        m.fuzz = (fz < 1 && fz >= 0) ? fz : 1;
      } else if (ty == "dielectric") { m.kind = M_DIEL; m.ior = F(); }
      else if (ty == "diffuse_light") { m.kind = M_LIGHT; m.tex = tex_ref(I()); }
      else if (ty == "isotropic") { m.kind = M_ISO; m.tex = tex_ref(I()); }
      else { err = "unknown material " + ty; return false; }
      S.mats.push_back(m);
      S.mat_of_sd[id] = (int)S.mats.size() - 1;
    } else if (kw == "node") {
      int id = I();
      std::string ty;
      is >> ty;
      Node nd;
      if (ty == "sphere") {
        nd.kind = K_SPHERE; float x = F(), y = F(), z = F(); nd.c0 = V(x, y, z); nd.r = F(); nd.mat = mat_ref(I());
      } else if (ty == "moving_sphere") {
        nd.kind = K_MSPHERE;
        float x = F(), y = F(), z = F(); nd.c0 = V(x, y, z);
        x = F(); y = F(); z = F(); nd.c1 = V(x, y, z);
        nd.t0 = F(); nd.t1 = F(); nd.r = F(); nd.mat = mat_ref(I());
      } else if (ty == "xy_rect" || ty == "xz_rect" || ty == "yz_rect") {
        nd.kind = ty == "xy_rect" ? K_XY : ty == "xz_rect" ? K_XZ : K_YZ;
        nd.a0 = F(); nd.a1 = F(); nd.b0 = F(); nd.b1 = F(); nd.k = F(); nd.mat = mat_ref(I());
      } else if (ty == "flip_normal") {
        nd.kind = K_FLIP; nd.child = node_ref(I());
      } else if (ty == "box") {  // rect_box.cc:93-115
        nd.kind = K_BOX;
        float x0 = F(), y0 = F(), z0 = F(), x1 = F(), y1 = F(), z1 = F();
        nd.pmin = V(x0, y0, z0); nd.pmax = V(x1, y1, z1); nd.mat = mat_ref(I());
        auto face = [&](int kind, float a0, float a1, float b0, float b1, float k, bool flip) {
          Node f; f.kind = kind; f.a0 = a0; f.a1 = a1; f.b0 = b0; f.b1 = b1; f.k = k; f.mat = nd.mat; f.sd = id;
          int fi = add_internal(f);
          if (!flip) return fi;
          Node fl; fl.kind = K_FLIP; fl.child = fi; fl.sd = id;
          return add_internal(fl);
        };
        V a = nd.pmin, b = nd.pmax;
        nd.items.push_back(face(K_XY, a.x(), b.x(), a.y(), b.y(), b.z(), false));
        nd.items.push_back(face(K_XY, a.x(), b.x(), a.y(), b.y(), a.z(), true));
        nd.items.push_back(face(K_XZ, a.x(), b.x(), a.z(), b.z(), b.y(), false));
        nd.items.push_back(face(K_XZ, a.x(), b.x(), a.z(), b.z(), a.y(), true));
        nd.items.push_back(face(K_YZ, a.y(), b.y(), a.z(), b.z(), b.x(), false));
        nd.items.push_back(face(K_YZ, a.y(), b.y(), a.z(), b.z(), a.x(), true));
      } else if (ty == "translate") {
        nd.kind = K_TRANSLATE; nd.child = node_ref(I()); float x = F(), y = F(), z = F(); nd.off = V(x, y, z);
      } else if (ty == "rotate_y") {
        nd.kind = K_ROTY; nd.child = node_ref(I());
        if (nd.child < 0) return false;
        init_rotate(S, nd, F());
      } else if (ty == "constant_medium") {  // hitable.cc:92-96
        nd.kind = K_MEDIUM; nd.child = node_ref(I()); nd.density = F();
        Mat iso; iso.kind = M_ISO; iso.tex = tex_ref(I());
        S.mats.push_back(iso);
        nd.phase = (int)S.mats.size() - 1;
        nd.mat = nd.phase;
      } else if (ty == "hitable_list") {
        nd.kind = K_LIST; int n = I();
        for (int i = 0; i < n; i++) nd.items.push_back(node_ref(I()));
      } else if (ty == "bvh_node") {
        float t0 = F(), t1 = F();
        int n = I();
        if (n < 1) { err = "empty bvh_node"; return false; }
        std::vector<int> l;
        for (int i = 0; i < n; i++) l.push_back(node_ref(I()));
        if (!err.empty()) return false;
        int root = build_bvh(S, build_rng, l.data(), n, t0, t1, err);
        if (!err.empty()) return false;
        S.nodes[root].sd = id;
        S.node_of_sd[id] = root;
        return true;
      } else { err = "unknown node " + ty; return false; }
      if (!err.empty()) return false;
      add(nd, id);
    } else if (kw == "world") {
      S.world = node_ref(I());
    } else if (kw == "lights") {
      S.lights = node_ref(I());
    } else if (kw == "camera") {  // camera.cc:2-21
      float fx = F(), fy = F(), fz = F(), ax = F(), ay = F(), az = F(), ux = F(), uy = F(), uz = F();
      float vfov = F(), aspect = F(), aperture = F(), focus = F(), t0 = F(), t1 = F();
      V from(fx, fy, fz), at(ax, ay, az), vup(ux, uy, uz);
      S.ct0 = t0; S.ct1 = t1;
      S.lens_r = aperture / 2;
      float theta = vfov * M_PI / 180;
      float hh = ::tan(theta / 2);
      float hw = aspect * hh;
      S.cam_o = from;
      S.cam_w = unit(from - at);
      S.cam_u = unit(cross(vup, S.cam_w));
      S.cam_vv = unit(cross(S.cam_w, S.cam_u));
      S.cam_ll = S.cam_o - hw * focus * S.cam_u - hh * focus * S.cam_vv - S.cam_w * focus;
      S.cam_h = 2 * hw * S.cam_u * focus;
      S.cam_v = 2 * hh * S.cam_vv * focus;
      S.has_cam = true;
    } else {
      err = "unknown statement " + kw;
      return false;
    }
    return err.empty();
  }
};

// Pre-order flattening of a built BVH, used by oracle_bvh_dump.
void dump_bvh(const Scene &S, int n, std::vector<float> &boxes, std::vector<int> &kids) {
  const Node &nd = S.nodes[n];
  int me = (int)kids.size() / 2;
  kids.push_back(0);
  kids.push_back(0);
  for (int i = 0; i < 3; i++) boxes.push_back(nd.bbox.mn[i]);
  for (int i = 0; i < 3; i++) boxes.push_back(nd.bbox.mx[i]);
  int ch[2] = {nd.left, nd.right};
  for (int c = 0; c < 2; c++) {
    const Node &cn = S.nodes[ch[c]];
    int ref;
    if (cn.kind == K_BVH && cn.sd < 0) {  // internal (not another SD bvh_node)
      ref = (int)kids.size() / 2;
      dump_bvh(S, ch[c], boxes, kids);
    } else {
      ref = -(1 + cn.sd);
    }
    kids[2 * me + c] = ref;
  }
}

}  // namespace

// ================================================================ C API ===
struct oracle_scene {
  Scene S;
};

extern "C" {

void oracle_philox(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
  philox10(ctr, key, out);
}

// lowbias32 integer hash (Chris Wellons, "Prospecting for Hash Functions").
static uint32_t hash32(uint32_t x) {
  x ^= x >> 16;
  x *= 0x7feb352du;
  x ^= x >> 15;
  x *= 0x846ca68bu;
  x ^= x >> 16;
  return x;
}

void oracle_procedural_image(int32_t w, int32_t h, uint32_t seed, uint8_t *rgb) {
  for (int32_t y = 0; y < h; y++)
    for (int32_t x = 0; x < w; x++) {
      uint32_t cell = hash32(seed ^ hash32((uint32_t)(x >> 5) + 65536u * (uint32_t)(y >> 5)));
      uint32_t fine = hash32(seed + (uint32_t)x * 2654435761u + (uint32_t)y * 40503u);
      uint8_t *p = rgb + 3 * ((size_t)y * w + x);
      p[0] = (uint8_t)((cell & 0xffu) / 2 + ((uint32_t)x * 127u) / (uint32_t)w);
      p[1] = (uint8_t)(((cell >> 8) & 0xffu) / 2 + ((uint32_t)y * 127u) / (uint32_t)h);
      p[2] = (uint8_t)(((cell >> 16) & 0xffu) / 2 + (fine & 127u));
    }
}

oracle_scene *oracle_scene_load(const char *sd_text, char *err, int errlen) {
  auto *os = new oracle_scene();
  Parser P(os->S);
  std::istringstream in(sd_text ? sd_text : "");
  std::string ln;
  int lineno = 0;
  while (std::getline(in, ln)) {
    lineno++;
    if (!P.line(ln)) {
      if (err && errlen > 0)
        std::snprintf(err, errlen, "line %d: %s", lineno, P.err.empty() ? "parse error" : P.err.c_str());
      delete os;
      return nullptr;
    }
  }
  if (os->S.world < 0) {
    if (err && errlen > 0) std::snprintf(err, errlen, "no world statement");
    delete os;
    return nullptr;
  }
  return os;
}

void oracle_scene_free(oracle_scene *s) { delete s; }

void oracle_scene_info(const oracle_scene *s, int32_t *out) {
  const Scene &S = s->S;
  int leaves = 0;
  for (auto &n : S.nodes)
    if (n.kind != K_BVH && n.kind != K_LIST && n.kind != K_FLIP && n.kind != K_TRANSLATE && n.kind != K_ROTY)
      leaves++;
  out[0] = (int32_t)S.nodes.size();
  out[1] = leaves;
  out[2] = S.n_internal;
  out[3] = (int32_t)S.mats.size();
  out[4] = (int32_t)S.texs.size();
  out[5] = S.world;
  out[6] = S.lights;
  out[7] = S.has_cam ? 1 : 0;
}

int32_t oracle_bvh_dump(const oracle_scene *s, int32_t sd_id, float *boxes, int32_t *kids, int32_t cap) {
  const Scene &S = s->S;
  auto it = S.node_of_sd.find(sd_id);
  if (it == S.node_of_sd.end() || S.nodes[it->second].kind != K_BVH) return -1;
  std::vector<float> b;
  std::vector<int> k;
  // the root is dumped even though it carries an SD id
  const Node &root = S.nodes[it->second];
  k.push_back(0);
  k.push_back(0);
  for (int i = 0; i < 3; i++) b.push_back(root.bbox.mn[i]);
  for (int i = 0; i < 3; i++) b.push_back(root.bbox.mx[i]);
  int ch[2] = {root.left, root.right};
  for (int c = 0; c < 2; c++) {
    const Node &cn = S.nodes[ch[c]];
    int ref;
    if (cn.kind == K_BVH && cn.sd < 0) {
      ref = (int)k.size() / 2;
      dump_bvh(S, ch[c], b, k);
    } else {
      ref = -(1 + cn.sd);
    }
    k[c] = ref;
  }
  int n = (int)k.size() / 2;
  if (n > cap) return n;
  std::memcpy(boxes, b.data(), b.size() * sizeof(float));
  std::memcpy(kids, k.data(), k.size() * sizeof(int));
  return n;
}

int32_t oracle_world_box(const oracle_scene *s, float *box6) {
  Box b;
  if (!bounding_box(s->S, s->S.world, 0, 0, b)) return 0;
  for (int i = 0; i < 3; i++) box6[i] = b.mn[i];
  for (int i = 0; i < 3; i++) box6[3 + i] = b.mx[i];
  return 1;
}

static void add_counters(oracle_counters *dst, const oracle_counters &src) {
  if (!dst) return;
  dst->segments += src.segments;
  dst->aabb_tests += src.aabb_tests;
  dst->sphere_tests += src.sphere_tests;
  dst->rect_tests += src.rect_tests;
  dst->instance_xforms += src.instance_xforms;
  dst->medium_tests += src.medium_tests;
  dst->lambertian += src.lambertian;
  dst->metal += src.metal;
  dst->dielectric += src.dielectric;
  dst->light_pdf_evals += src.light_pdf_evals;
}

int32_t oracle_trace(const oracle_scene *s, const float *rays, int64_t n, uint64_t seed, int32_t media_mode,
                     float *out_f, int32_t *out_i, int32_t nthreads, oracle_counters *cnt) {
  if (!s || n < 0) return 1;
  if (media_mode == 1) nthreads = 1;  // one drand_r stream, reference order
  if (nthreads < 1) nthreads = 1;
  std::vector<oracle_counters> part(nthreads);
  std::memset(part.data(), 0, sizeof(oracle_counters) * part.size());
  auto work = [&](int tid) {
    Rng rng;
    Ctx C;
    C.S = &s->S;
    C.rng = &rng;
    C.philox_media = media_mode == 0;
    C.seed = seed;
    C.cnt = cnt ? &part[tid] : nullptr;
    for (int64_t i = tid; i < n; i += nthreads) {
      const float *q = rays + 7 * i;
      Ray r{V(q[0], q[1], q[2]), V(q[3], q[4], q[5]), q[6]};
      C.ray_index = (uint64_t)i;
      Hit rec;
      bool h = hit(C, s->S.world, r, 0.001, std::numeric_limits<float>::max(), rec);
      float *o = out_f + 9 * i;
      if (h) {
        o[0] = rec.t; o[1] = rec.u; o[2] = rec.v;
        o[3] = rec.p[0]; o[4] = rec.p[1]; o[5] = rec.p[2];
        o[6] = rec.n[0]; o[7] = rec.n[1]; o[8] = rec.n[2];
        out_i[2 * i] = 1;
        out_i[2 * i + 1] = rec.prim;
      } else {
        for (int k = 0; k < 9; k++) o[k] = 0.f;
        out_i[2 * i] = 0;
        out_i[2 * i + 1] = -1;
      }
    }
  };
  std::vector<std::thread> th;
  for (int t = 1; t < nthreads; t++) th.emplace_back(work, t);
  work(0);
  for (auto &t : th) t.join();
  for (auto &p : part) add_counters(cnt, p);
  return 0;
}

void oracle_make_rays(const oracle_scene *s, int64_t n, uint64_t seed, float frac_camera, float frac_axis,
                      float *rays) {
  const Scene &S = s->S;
  Box wb;
  bool has = bounding_box(S, S.world, 0, 0, wb);
  if (!has) wb = Box{V(-1, -1, -1), V(1, 1, 1)};
  // keep huge enclosing primitives (ground spheres) from dominating
  for (int i = 0; i < 3; i++) {
    if (wb.mn[i] < -2000.f) wb.mn[i] = -2000.f;
    if (wb.mx[i] > 2000.f) wb.mx[i] = 2000.f;
  }
  uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
  int64_t ncam = S.has_cam ? (int64_t)(frac_camera * (float)n) : 0;
  for (int64_t i = 0; i < n; i++) {
    uint32_t ctr[4] = {(uint32_t)i, (uint32_t)(i >> 32), 0u, 0x52415953u};
    uint32_t a[4], b[4];
    philox10(ctr, key, a);
    ctr[2] = 1u;
    philox10(ctr, key, b);
    float *q = rays + 7 * i;
    if (i < ncam) {
      // camera ray (camera.cc:23-31) with uniforms from Philox; the lens
      // point is drawn by rejection on the uniforms of successive blocks.
      float s = u01(a[0]), t = u01(a[1]);
      V rd;
      uint32_t blk = 2;
      for (;;) {
        float x = 2.0f * u01(b[0]) - 1.0f, y = 2.0f * u01(b[1]) - 1.0f;
        if (x * x + y * y < 1.0f) { rd = V(x, y, 0); break; }
        ctr[2] = blk++;
        philox10(ctr, key, b);
      }
      rd = S.lens_r * rd;
      V off = S.cam_u * rd.x() + S.cam_vv * rd.y();
      float time = S.ct0 + u01(a[2]) * (S.ct1 - S.ct0);
      V o = S.cam_o + off;
      V d = S.cam_ll + s * S.cam_h + t * S.cam_v - S.cam_o - off;
      q[0] = o[0]; q[1] = o[1]; q[2] = o[2]; q[3] = d[0]; q[4] = d[1]; q[5] = d[2]; q[6] = time;
    } else {
      V o(wb.mn.x() + u01(a[0]) * (wb.mx.x() - wb.mn.x()), wb.mn.y() + u01(a[1]) * (wb.mx.y() - wb.mn.y()),
          wb.mn.z() + u01(a[2]) * (wb.mx.z() - wb.mn.z()));
      V d;
      uint32_t blk = 2;
      for (;;) {
        float x = 2.0f * u01(b[0]) - 1.0f, y = 2.0f * u01(b[1]) - 1.0f, z = 2.0f * u01(b[2]) - 1.0f;
        float l2 = x * x + y * y + z * z;
        if (l2 < 1.0f && l2 > 1e-4f) {
          float len = std::sqrt(l2);
          float scale = (0.5f + 1.5f * u01(b[3])) / len;
          d = V(x * scale, y * scale, z * scale);
          break;
        }
        ctr[2] = blk++;
        philox10(ctr, key, b);
      }
      float axis_pick = u01(a[3]);
      if (axis_pick < frac_axis) {
        int zero = (int)(u01(b[3]) * 3.0f) % 3;
        d[zero] = 0.0f;
        if (axis_pick < 0.3f * frac_axis) d[(zero + 1) % 3] = 0.0f;
      }
      q[0] = o[0]; q[1] = o[1]; q[2] = o[2]; q[3] = d[0]; q[4] = d[1]; q[5] = d[2];
      q[6] = S.ct0 + u01(a[3]) * (S.ct1 - S.ct0);
    }
  }
}

int32_t oracle_render(const oracle_scene *s, const oracle_render_params *p, float *mean_rgb,
                      oracle_counters *cnt) {
  if (!s || !p || p->width <= 0 || p->height <= 0 || p->spp <= 0 || !s->S.has_cam) return 1;
  const Scene &S = s->S;
  RenderCfg cfg;
  cfg.max_depth = p->max_depth;
  cfg.semantics = p->semantics;
  cfg.background = p->background;
  cfg.sky_scale = p->sky_scale;
  int nx = p->width, ny = p->height, ns = p->spp;
  int rb = p->row_begin < 0 ? 0 : p->row_begin;
  int re = p->row_end <= 0 || p->row_end > ny ? ny : p->row_end;
  int nthreads = p->nthreads < 1 ? 1 : p->nthreads;
  std::vector<oracle_counters> part(nthreads);
  std::memset(part.data(), 0, sizeof(oracle_counters) * part.size());
  std::atomic<int> next_row(rb);
  auto work = [&](int tid) {
    Ctx C;
    C.S = &S;
    C.cnt = cnt ? &part[tid] : nullptr;
    Sampler R;
    C.rng = &R.rng;
    for (;;) {
      int row = next_row.fetch_add(1);
      if (row >= re) break;
      int j = ny - 1 - row;  // reference rows run bottom-up (main.cpp:157)
      std::seed_seq sq{(uint32_t)p->seed, (uint32_t)(p->seed >> 32), (uint32_t)j, 0x5eedu};
      R.rng.gen.seed(sq);
      for (int i = 0; i < nx; i++) {  // main.cpp:115-135
        V col(0, 0, 0);
        for (int k = 0; k < ns; k++) {
          float u = ((float)i + R()) / (float)nx;
          float v = ((float)j + R()) / (float)ny;
          Ray r = camera_ray(S, R, u, v);
          col = col + de_nan(color(C, R, cfg, r, 0));
        }
        col = col / float(ns);
        float *o = mean_rgb + 3 * ((size_t)row * nx + i);
        o[0] = col[0]; o[1] = col[1]; o[2] = col[2];
      }
    }
  };
  std::vector<std::thread> th;
  for (int t = 1; t < nthreads; t++) th.emplace_back(work, t);
  work(0);
  for (auto &t : th) t.join();
  for (auto &q : part) add_counters(cnt, q);
  return 0;
}

void oracle_quantize(const float *mean_rgb, int64_t n_pixels, uint8_t *rgb8) {
  for (int64_t i = 0; i < 3 * n_pixels; i++) {
    float c = std::sqrt(mean_rgb[i]);
    int q = int(255.99f * c);
    if (q < 0) q = 0;
    if (q > 255) q = 255;
    rgb8[i] = (uint8_t)q;
  }
}

}  // extern "C"
