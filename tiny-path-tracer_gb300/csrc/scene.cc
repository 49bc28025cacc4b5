// scene.cc - host front end: the reference's scene classes as builder
// records, the bvh_node construction rule, and the compiler that flattens a
// scene graph into the device arena of arena.h.  Also the scene-description
// text loader and the host output helpers of tpt.h.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <limits>
#include <memory>
#include <random>
#include <sstream>
#include <string>
#include <unordered_map>
#include <vector>

#include "../../include/tpt.h"
#include "arena.h"
#include "scene_internal.h"

namespace tpt {

// ------------------------------------------------------------- vectors ----
// Float component arithmetic with the reference's operation order
// (headers/vec3.h); the build uses -ffp-contract=off.
struct v3 {
  float e[3];
};
static inline v3 mk(float a, float b, float c) { return v3{{a, b, c}}; }
static inline v3 add(v3 a, v3 b) { return mk(a.e[0] + b.e[0], a.e[1] + b.e[1], a.e[2] + b.e[2]); }
static inline v3 sub(v3 a, v3 b) { return mk(a.e[0] - b.e[0], a.e[1] - b.e[1], a.e[2] - b.e[2]); }
static inline v3 scl(v3 a, float t) { return mk(a.e[0] * t, a.e[1] * t, a.e[2] * t); }
static inline v3 dvs(v3 a, float t) { return mk(a.e[0] / t, a.e[1] / t, a.e[2] / t); }
static inline float len(v3 a) { return std::sqrt(a.e[0] * a.e[0] + a.e[1] * a.e[1] + a.e[2] * a.e[2]); }
static inline v3 unit(v3 a) { return dvs(a, len(a)); }
static inline v3 crs(v3 a, v3 b) {
  return mk(a.e[1] * b.e[2] - b.e[1] * a.e[2], a.e[2] * b.e[0] - b.e[2] * a.e[0], a.e[0] * b.e[1] - b.e[0] * a.e[1]);
}

struct box3 {
  v3 mn, mx;
};
// surrounding_box (aabb.cc:21-30)
static box3 surround(const box3 &a, const box3 &b) {
  auto lo = [](float p, float q) { return p < q ? p : q; };
  auto hi = [](float p, float q) { return p > q ? p : q; };
  return box3{mk(lo(a.mn.e[0], b.mn.e[0]), lo(a.mn.e[1], b.mn.e[1]), lo(a.mn.e[2], b.mn.e[2])),
              mk(hi(a.mx.e[0], b.mx.e[0]), hi(a.mx.e[1], b.mx.e[1]), hi(a.mx.e[2], b.mx.e[2]))};
}

}  // namespace tpt

using namespace tpt;

// ------------------------------------------------------------ builder -----
enum HKind {
  H_SPHERE = 1, H_MSPHERE, H_XY, H_XZ, H_YZ, H_FLIP, H_BOX, H_TRANSLATE, H_ROTY, H_MEDIUM, H_LIST, H_BVH
};

struct HTex {
  int kind = 0;
  float c[3] = {0, 0, 0};
  int odd = -1, even = -1;
  float scale = 1.f;
  int w = 0, h = 0;
  std::vector<uint8_t> px;
};
struct HMat {
  int kind = 0;
  int tex = -1;
  float albedo[3] = {0, 0, 0};
  float fuzz = 0.f, ior = 1.f;
};
struct HNode {
  int kind = 0;
  int user = -1;        // user id reported for hits / dumps
  bool internal = false;  // BVH node created by a bvh_node build
  int mat = -1;
  v3 c0{}, c1{};
  float r = 0, t0 = 0, t1 = 0;
  float a0 = 0, a1 = 0, b0 = 0, b1 = 0, k = 0;
  v3 pmin{}, pmax{};
  int child = -1;
  v3 off{};
  float sn = 0, cs = 1;
  bool has_box = false;
  box3 rbox{};
  float density = 0;
  int phase_tex = -1;
  std::vector<int> items;
  int left = -1, right = -1;
  box3 bbox{};
};

struct tpt_builder {
  std::vector<HTex> texs;
  std::vector<HMat> mats;
  std::vector<HNode> nodes;
  std::unordered_map<int, int> handle_of_user;
  std::mt19937 drand_gen;  // drand_r stream of bvh_node (utils.cc:28-32)
  bool has_perlin = false;
  bool perlin_draws = true;  // perlin textures consume drand_r like the reference
  float pgrad[768] = {};
  int32_t pperm[768] = {};
  int world = -1, lights = -1;
  bool has_cam = false;
  Camera cam{};
  float cam_in[15] = {};  // tpt_builder_set_camera's arguments
  int bvh_build = TPT_BVH_REFERENCE;  // topology the compiler flattens
  std::string err;

  double drand(double a = 0.0, double b = 1.0) {
    std::uniform_real_distribution<double> dis(a, b);
    return dis(drand_gen);
  }
  bool valid_node(int h) const { return h >= 0 && h < (int)nodes.size(); }
  bool valid_mat(int h) const { return h >= 0 && h < (int)mats.size(); }
  bool valid_tex(int h) const { return h >= 0 && h < (int)texs.size(); }
  bool auto_user = true;  // user id = handle (API builds); SD loads set SD ids
  int add_node(HNode n) {
    nodes.push_back(std::move(n));
    int h = (int)nodes.size() - 1;
    if (!nodes[h].internal && auto_user) set_user(h, h);
    return h;
  }
  void set_user(int h, int user) {
    nodes[h].user = user;
    handle_of_user[user] = h;
  }
};

static v3 msphere_center(const HNode &n, float time) {  // sphere.h:29-32
  return add(n.c0, scl(sub(n.c1, n.c0), (time - n.t0) / (n.t1 - n.t0)));
}

// bounding_box of every hitable kind (sphere.cc:77-91, rect_box.cc:3-6,45-49,
// 70-73, rect_box.h:47-49,66-69,80-86,104-107, hitable.h:64-66,
// hitable_list.cc:3-22, hitable.cc:58-61).
static bool hbox(const tpt_builder &B, int h, float t0, float t1, box3 &out) {
  const HNode &n = B.nodes[h];
  switch (n.kind) {
    case H_SPHERE: {
      v3 r = mk(n.r, n.r, n.r);
      out = box3{sub(n.c0, r), add(n.c0, r)};
      return true;
    }
    case H_MSPHERE: {
      v3 r = mk(n.r, n.r, n.r);
      v3 ca = msphere_center(n, t0), cb = msphere_center(n, t1);
      out = surround(box3{sub(ca, r), add(ca, r)}, box3{sub(cb, r), add(cb, r)});
      return true;
    }
    case H_XY:
      out = box3{mk(n.a0, n.b0, (float)(n.k - 0.0001)), mk(n.a1, n.b1, (float)(n.k + 0.0001))};
      return true;
    case H_XZ:
      out = box3{mk(n.a0, (float)(n.k - 0.0001), n.b0), mk(n.a1, (float)(n.k + 0.0001), n.b1)};
      return true;
    case H_YZ:
      out = box3{mk((float)(n.k - 0.0001), n.a0, n.b0), mk((float)(n.k + 0.0001), n.a1, n.b1)};
      return true;
    case H_FLIP:
    case H_MEDIUM:
      return hbox(B, n.child, t0, t1, out);
    case H_BOX:
      out = box3{n.pmin, n.pmax};
      return true;
    case H_TRANSLATE:
      if (!hbox(B, n.child, t0, t1, out)) return false;
      out = box3{add(out.mn, n.off), add(out.mx, n.off)};
      return true;
    case H_ROTY:
      out = n.rbox;
      return n.has_box;
    case H_LIST: {
      if (n.items.empty()) return false;
      box3 tmp;
      if (!hbox(B, n.items[0], t0, t1, tmp)) return false;
      out = tmp;
      for (size_t i = 1; i < n.items.size(); i++) {
        if (!hbox(B, n.items[i], t0, t1, tmp)) return false;
        out = surround(out, tmp);
      }
      return true;
    }
    case H_BVH:
      out = n.bbox;
      return true;
  }
  return false;
}

// bvh_node construction rule (hitable.cc:32-56): one drand_r(0,3) draw picks
// the axis, the slice is std::sort-ed by box.min[axis] of bounding_box(0,0)
// (comparator of hitable.cc:10-30), then split at n/2.  std::sort is the same
// libstdc++ introsort the reference uses, so equal inputs give equal trees.
static int build_bvh(tpt_builder &B, int *l, int n, float t0, float t1) {
  int axis = int(B.drand(0, 3.0));
  if (axis > 2) axis = 2;
  bool missing = false;
  auto cmp = [&B, axis, &missing](int a, int b) {
    box3 ba, bb;
    if (!hbox(B, a, 0, 0, ba) || !hbox(B, b, 0, 0, bb)) {
      missing = true;
      return false;
    }
    return !std::isgreaterequal(ba.mn.e[axis], bb.mn.e[axis]);
  };
  std::sort(l, l + n, cmp);
  if (missing) return -TPT_ERR_NO_BOUNDING_BOX;
  HNode nd;
  nd.kind = H_BVH;
  nd.internal = true;
  if (n == 1) {
    nd.left = nd.right = l[0];
  } else if (n == 2) {
    nd.left = l[0];
    nd.right = l[1];
  } else {
    nd.left = build_bvh(B, l, n / 2, t0, t1);
    if (nd.left < 0) return nd.left;
    nd.right = build_bvh(B, l + n / 2, n - n / 2, t0, t1);
    if (nd.right < 0) return nd.right;
  }
  box3 bl, br;
  if (!hbox(B, nd.left, t0, t1, bl) || !hbox(B, nd.right, t0, t1, br)) return -TPT_ERR_NO_BOUNDING_BOX;
  nd.bbox = surround(bl, br);
  return B.add_node(std::move(nd));
}

// rotate_y constructor (rect_box.cc:142-190).
static void init_rotate(tpt_builder &B, HNode &n, float angle) {
  float radians = angle / 180.0f * M_PI;
  n.sn = std::sin(radians);
  n.cs = std::cos(radians);
  box3 b{};
  n.has_box = hbox(B, n.child, 0, 0, b);
  auto cmin = [](v3 p, v3 q) {
    return mk(std::min(p.e[0], q.e[0]), std::min(p.e[1], q.e[1]), std::min(p.e[2], q.e[2]));
  };
  auto cmax = [](v3 p, v3 q) {
    return mk(std::max(p.e[0], q.e[0]), std::max(p.e[1], q.e[1]), std::max(p.e[2], q.e[2]));
  };
  v3 col1 = mk(n.cs, 0, -n.sn), col2 = mk(0, 1, 0), col3 = mk(n.sn, 0, n.cs);
  v3 xa = scl(col1, b.mx.e[0]), xb = scl(col1, b.mn.e[0]);
  v3 ya = scl(col2, b.mx.e[1]), yb = scl(col2, b.mn.e[1]);
  v3 za = scl(col3, b.mx.e[2]), zb = scl(col3, b.mn.e[2]);
  n.rbox = box3{add(add(cmin(xa, xb), cmin(ya, yb)), cmin(za, zb)), add(add(cmax(xa, xb), cmax(ya, yb)), cmax(za, zb))};
}

// perlin tables from the drand_r stream (perlin_noise.cc:4-9) and a
// fixed-seed shuffle (the reference seeds it from the clock).
static void default_perlin(tpt_builder &B) {
  for (int i = 0; i < 256; i++) {
    float f1 = (float)(2 * B.drand() - 1), f2 = (float)(2 * B.drand() - 1), f3 = (float)(2 * B.drand() - 1);
    v3 u = unit(mk(f1, f2, f3));
    B.pgrad[3 * i] = u.e[0];
    B.pgrad[3 * i + 1] = u.e[1];
    B.pgrad[3 * i + 2] = u.e[2];
  }
  std::default_random_engine eng(5489u);
  for (int a = 0; a < 3; a++) {
    int32_t *p = B.pperm + 256 * a;
    for (int i = 0; i < 256; i++) p[i] = i;
    std::shuffle(p, p + 256, eng);
  }
  B.has_perlin = true;
}

// lowbias32 integer hash (Chris Wellons, "Prospecting for Hash Functions").
static uint32_t lowbias32(uint32_t x) {
  x ^= x >> 16;
  x *= 0x7feb352du;
  x ^= x >> 15;
  x *= 0x846ca68bu;
  x ^= x >> 16;
  return x;
}

// Procedural RGB8 image of the scene-description 'image' texture: a hashed
// 32x32-texel cell colour plus horizontal/vertical ramps and per-texel noise.
static void procedural_image(int w, int h, uint32_t seed, uint8_t *rgb) {
  for (int y = 0; y < h; y++)
    for (int x = 0; x < w; x++) {
      uint32_t cell = lowbias32(seed ^ lowbias32((uint32_t)(x >> 5) + 65536u * (uint32_t)(y >> 5)));
      uint32_t fine = lowbias32(seed + (uint32_t)x * 2654435761u + (uint32_t)y * 40503u);
      uint8_t *p = rgb + 3 * ((size_t)y * w + x);
      p[0] = (uint8_t)((cell & 0xffu) / 2 + ((uint32_t)x * 127u) / (uint32_t)w);
      p[1] = (uint8_t)(((cell >> 8) & 0xffu) / 2 + ((uint32_t)y * 127u) / (uint32_t)h);
      p[2] = (uint8_t)(((cell >> 16) & 0xffu) / 2 + (fine & 127u));
    }
}

// =========================================================== C API: build ==
extern "C" {

const char *tpt_status_string(tpt_status s) {
  switch (s) {
    case TPT_OK: return "ok";
    case TPT_ERR_INVALID_ARGUMENT: return "invalid argument";
    case TPT_ERR_PARSE: return "scene text parse error";
    case TPT_ERR_UNSUPPORTED: return "scene shape not supported by the device layout";
    case TPT_ERR_NO_BOUNDING_BOX: return "No bounding box in BVH node constructor";
    case TPT_ERR_CUDA: return "CUDA error";
    case TPT_ERR_OUT_OF_MEMORY: return "out of device memory";
    case TPT_ERR_DEVICE_TIMEOUT: return "device loop reached its iteration limit";
    case TPT_ERR_STACK_OVERFLOW: return "traversal stack overflow";
    case TPT_ERR_NO_DEVICE: return "no CUDA device";
    case TPT_ERR_BAD_HANDLE: return "bad handle";
  }
  return "unknown status";
}

const char *tpt_version(void) { return "tpt-gb300 0.1"; }

tpt_status tpt_builder_create(tpt_builder **out) {
  if (!out) return TPT_ERR_INVALID_ARGUMENT;
  *out = new tpt_builder();
  return TPT_OK;
}
void tpt_builder_destroy(tpt_builder *b) { delete b; }

#define TPT_BAD(b) if (!(b)) return -TPT_ERR_INVALID_ARGUMENT

int32_t tpt_constant_texture(tpt_builder *b, float r, float g, float bl) {
  TPT_BAD(b);
  HTex t;
  t.kind = TT_CONST;
  t.c[0] = r; t.c[1] = g; t.c[2] = bl;
  b->texs.push_back(t);
  return (int32_t)b->texs.size() - 1;
}
int32_t tpt_checker_texture(tpt_builder *b, int32_t odd, int32_t even) {
  TPT_BAD(b);
  if (!b->valid_tex(odd) || !b->valid_tex(even)) return -TPT_ERR_BAD_HANDLE;
  HTex t;
  t.kind = TT_CHECKER;
  t.odd = odd;
  t.even = even;
  b->texs.push_back(t);
  return (int32_t)b->texs.size() - 1;
}
int32_t tpt_perlin_noise_texture(tpt_builder *b, float scale) {
  TPT_BAD(b);
  // perlin_noise's constructor refills the shared tables from drand_r
  // (perlin_noise.cc:3-21), which advances the stream later bvh_node
  // constructions draw from; the builder does the same.
  if (b->perlin_draws) default_perlin(*b);
  HTex t;
  t.kind = TT_PERLIN;
  t.scale = scale;
  b->texs.push_back(t);
  return (int32_t)b->texs.size() - 1;
}
tpt_status tpt_perlin_tables(tpt_builder *b, const float *g, const int32_t *perm) {
  if (!b || !g || !perm) return TPT_ERR_INVALID_ARGUMENT;
  std::memcpy(b->pgrad, g, sizeof(b->pgrad));
  for (int i = 0; i < 768; i++) b->pperm[i] = perm[i] & 255;
  b->has_perlin = true;
  return TPT_OK;
}
int32_t tpt_image_texture(tpt_builder *b, const uint8_t *rgb, int32_t w, int32_t h) {
  TPT_BAD(b);
  if (!rgb || w <= 0 || h <= 0) return -TPT_ERR_INVALID_ARGUMENT;
  HTex t;
  t.kind = TT_IMAGE;
  t.w = w;
  t.h = h;
  t.px.assign(rgb, rgb + (size_t)w * h * 3);
  b->texs.push_back(std::move(t));
  return (int32_t)b->texs.size() - 1;
}

static int32_t add_mat(tpt_builder *b, HMat m) {
  b->mats.push_back(m);
  return (int32_t)b->mats.size() - 1;
}
int32_t tpt_lambertian(tpt_builder *b, int32_t tex) {
  TPT_BAD(b);
  if (!b->valid_tex(tex)) return -TPT_ERR_BAD_HANDLE;
  HMat m;
  m.kind = MT_LAMBERTIAN;
  m.tex = tex;
  return add_mat(b, m);
}
int32_t tpt_metal(tpt_builder *b, float r, float g, float bl, float fuzz) {
  TPT_BAD(b);
  HMat m;
  m.kind = MT_METAL;
  m.albedo[0] = r; m.albedo[1] = g; m.albedo[2] = bl;
  m.fuzz = (fuzz < 1 && fuzz >= 0) ? fuzz : 1;  // material.h:41-46
  return add_mat(b, m);
}
int32_t tpt_dielectric(tpt_builder *b, float ri) {
  TPT_BAD(b);
  HMat m;
  m.kind = MT_DIELECTRIC;
  m.ior = ri;
  return add_mat(b, m);
}
int32_t tpt_diffuse_light(tpt_builder *b, int32_t tex) {
  TPT_BAD(b);
  if (!b->valid_tex(tex)) return -TPT_ERR_BAD_HANDLE;
  HMat m;
  m.kind = MT_LIGHT;
  m.tex = tex;
  return add_mat(b, m);
}
int32_t tpt_isotropic(tpt_builder *b, int32_t tex) {
  TPT_BAD(b);
  if (!b->valid_tex(tex)) return -TPT_ERR_BAD_HANDLE;
  HMat m;
  m.kind = MT_ISOTROPIC;
  m.tex = tex;
  return add_mat(b, m);
}

int32_t tpt_sphere(tpt_builder *b, float cx, float cy, float cz, float r, int32_t mat) {
  TPT_BAD(b);
  if (!b->valid_mat(mat)) return -TPT_ERR_BAD_HANDLE;
  HNode n;
  n.kind = H_SPHERE;
  n.c0 = mk(cx, cy, cz);
  n.r = r;
  n.mat = mat;
  return b->add_node(n);
}
int32_t tpt_moving_sphere(tpt_builder *b, float c0x, float c0y, float c0z, float c1x, float c1y, float c1z, float t0,
                          float t1, float r, int32_t mat) {
  TPT_BAD(b);
  if (!b->valid_mat(mat)) return -TPT_ERR_BAD_HANDLE;
  HNode n;
  n.kind = H_MSPHERE;
  n.c0 = mk(c0x, c0y, c0z);
  n.c1 = mk(c1x, c1y, c1z);
  n.t0 = t0;
  n.t1 = t1;
  n.r = r;
  n.mat = mat;
  return b->add_node(n);
}
static int32_t add_rect(tpt_builder *b, int kind, float a0, float a1, float b0, float b1, float k, int32_t mat) {
  TPT_BAD(b);
  if (!b->valid_mat(mat)) return -TPT_ERR_BAD_HANDLE;
  HNode n;
  n.kind = kind;
  n.a0 = a0; n.a1 = a1; n.b0 = b0; n.b1 = b1; n.k = k;
  n.mat = mat;
  return b->add_node(n);
}
int32_t tpt_xy_rect(tpt_builder *b, float x0, float x1, float y0, float y1, float k, int32_t mat) {
  return add_rect(b, H_XY, x0, x1, y0, y1, k, mat);
}
int32_t tpt_xz_rect(tpt_builder *b, float x0, float x1, float z0, float z1, float k, int32_t mat) {
  return add_rect(b, H_XZ, x0, x1, z0, z1, k, mat);
}
int32_t tpt_yz_rect(tpt_builder *b, float y0, float y1, float z0, float z1, float k, int32_t mat) {
  return add_rect(b, H_YZ, y0, y1, z0, z1, k, mat);
}
int32_t tpt_flip_normal(tpt_builder *b, int32_t child) {
  TPT_BAD(b);
  if (!b->valid_node(child)) return -TPT_ERR_BAD_HANDLE;
  HNode n;
  n.kind = H_FLIP;
  n.child = child;
  return b->add_node(n);
}
int32_t tpt_box(tpt_builder *b, float x0, float y0, float z0, float x1, float y1, float z1, int32_t mat) {
  TPT_BAD(b);
  if (!b->valid_mat(mat)) return -TPT_ERR_BAD_HANDLE;
  HNode n;
  n.kind = H_BOX;
  n.pmin = mk(x0, y0, z0);
  n.pmax = mk(x1, y1, z1);
  n.mat = mat;
  return b->add_node(n);
}
int32_t tpt_translate(tpt_builder *b, int32_t child, float ox, float oy, float oz) {
  TPT_BAD(b);
  if (!b->valid_node(child)) return -TPT_ERR_BAD_HANDLE;
  HNode n;
  n.kind = H_TRANSLATE;
  n.child = child;
  n.off = mk(ox, oy, oz);
  return b->add_node(n);
}
int32_t tpt_rotate_y(tpt_builder *b, int32_t child, float angle) {
  TPT_BAD(b);
  if (!b->valid_node(child)) return -TPT_ERR_BAD_HANDLE;
  HNode n;
  n.kind = H_ROTY;
  n.child = child;
  init_rotate(*b, n, angle);
  return b->add_node(n);
}
int32_t tpt_constant_medium(tpt_builder *b, int32_t boundary, float density, int32_t tex) {
  TPT_BAD(b);
  if (!b->valid_node(boundary) || !b->valid_tex(tex)) return -TPT_ERR_BAD_HANDLE;
  HNode n;
  n.kind = H_MEDIUM;
  n.child = boundary;
  n.density = density;
  n.phase_tex = tex;
  return b->add_node(n);
}
int32_t tpt_hitable_list(tpt_builder *b, const int32_t *items, int32_t n) {
  TPT_BAD(b);
  if (n < 0 || (n > 0 && !items)) return -TPT_ERR_INVALID_ARGUMENT;
  HNode nd;
  nd.kind = H_LIST;
  for (int i = 0; i < n; i++) {
    if (!b->valid_node(items[i])) return -TPT_ERR_BAD_HANDLE;
    nd.items.push_back(items[i]);
  }
  return b->add_node(nd);
}
int32_t tpt_bvh_node(tpt_builder *b, const int32_t *items, int32_t n, float t0, float t1) {
  TPT_BAD(b);
  if (n < 1 || !items) return -TPT_ERR_INVALID_ARGUMENT;
  std::vector<int> l(items, items + n);
  for (int h : l)
    if (!b->valid_node(h)) return -TPT_ERR_BAD_HANDLE;
  int root = build_bvh(*b, l.data(), n, t0, t1);
  if (root < 0) return root;
  // the root becomes a user-visible hitable; it keeps the shutter interval
  // and its items, in the caller's order, for rebuilds of its topology
  // (TPT_BVH_SAH, TPT_BVH_LBVH)
  b->nodes[root].internal = false;
  b->nodes[root].t0 = t0;
  b->nodes[root].t1 = t1;
  b->nodes[root].items = l;
  if (b->auto_user) b->set_user(root, root);
  return root;
}

tpt_status tpt_builder_set_bvh_build(tpt_builder *b, int32_t mode) {
  if (!b || (mode != TPT_BVH_REFERENCE && mode != TPT_BVH_SAH && mode != TPT_BVH_LBVH))
    return TPT_ERR_INVALID_ARGUMENT;
  b->bvh_build = mode;
  return TPT_OK;
}

double tpt_builder_drand(tpt_builder *b, double min, double max) { return b ? b->drand(min, max) : 0.0; }

tpt_status tpt_builder_set_world(tpt_builder *b, int32_t world) {
  if (!b) return TPT_ERR_INVALID_ARGUMENT;
  if (!b->valid_node(world)) return TPT_ERR_BAD_HANDLE;
  b->world = world;
  return TPT_OK;
}
tpt_status tpt_builder_set_light_shape(tpt_builder *b, int32_t ls) {
  if (!b) return TPT_ERR_INVALID_ARGUMENT;
  if (ls != -1 && !b->valid_node(ls)) return TPT_ERR_BAD_HANDLE;
  b->lights = ls;
  return TPT_OK;
}
}  // extern "C"

// camera_with_blur::camera_with_blur (camera.cc:2-21), precomputed on the host.
static Camera make_camera(const float lf[3], const float la[3], const float up[3], float vfov, float aspect,
                          float aperture, float focus, float t0, float t1) {
  Camera c{};
  c.t0 = t0;
  c.t1 = t1;
  c.lens_radius = aperture / 2;
  float theta = vfov * M_PI / 180;
  float hh = ::tan(theta / 2);
  float hw = aspect * hh;
  v3 from = mk(lf[0], lf[1], lf[2]), at = mk(la[0], la[1], la[2]), vup = mk(up[0], up[1], up[2]);
  v3 w = unit(sub(from, at));
  v3 u = unit(crs(vup, w));
  v3 v = unit(crs(w, u));
  v3 ll = sub(sub(sub(from, scl(u, hw * focus)), scl(v, hh * focus)), scl(w, focus));
  v3 hz = scl(scl(u, 2 * hw), focus);
  v3 vt = scl(scl(v, 2 * hh), focus);
  for (int i = 0; i < 3; i++) {
    c.origin[i] = from.e[i];
    c.lower_left[i] = ll.e[i];
    c.horizontal[i] = hz.e[i];
    c.vertical[i] = vt.e[i];
    c.u[i] = u.e[i];
    c.v[i] = v.e[i];
  }
  return c;
}

static void camera_inputs(const float lf[3], const float la[3], const float up[3], float vfov, float aspect,
                          float aperture, float focus, float t0, float t1, float out[15]) {
  for (int i = 0; i < 3; i++) {
    out[i] = lf[i];
    out[3 + i] = la[i];
    out[6 + i] = up[i];
  }
  out[9] = vfov;
  out[10] = aspect;
  out[11] = aperture;
  out[12] = focus;
  out[13] = t0;
  out[14] = t1;
}

extern "C" {

tpt_status tpt_builder_set_camera(tpt_builder *b, const float lf[3], const float la[3], const float up[3], float vfov,
                                  float aspect, float aperture, float focus, float t0, float t1) {
  if (!b || !lf || !la || !up) return TPT_ERR_INVALID_ARGUMENT;
  b->cam = make_camera(lf, la, up, vfov, aspect, aperture, focus, t0, t1);
  camera_inputs(lf, la, up, vfov, aspect, aperture, focus, t0, t1, b->cam_in);
  b->has_cam = true;
  return TPT_OK;
}

}  // extern "C"

// ============================================================ compiler ====
namespace {

struct Compiler {
  const tpt_builder &B;
  HostScene &S;
  std::unordered_map<int, int> blas_root;  // builder handle -> node index
  tpt_status st = TPT_OK;
  std::string why;

  Compiler(const tpt_builder &b, HostScene &s) : B(b), S(s) {}

  int fail(tpt_status code, const std::string &msg) {
    if (st == TPT_OK) {
      st = code;
      why = msg;
    }
    return -1;
  }

  int push_data(const f4 &v) {
    S.leaf_data.push_back(v);
    return (int)S.leaf_data.size() - 1;
  }

  // Primitive leaf for builder node h with the accumulated flip parity.
  int prim_leaf(int h, int flip) {
    const HNode &n = B.nodes[h];
    i4 hdr{0, (int32_t)S.leaf_data.size(), n.mat, -1};
    switch (n.kind) {
      case H_SPHERE:
        hdr.x = LT_SPHERE;
        push_data(f4{n.c0.e[0], n.c0.e[1], n.c0.e[2], n.r});
        break;
      case H_MSPHERE:
        hdr.x = LT_MSPHERE;
        push_data(f4{n.c0.e[0], n.c0.e[1], n.c0.e[2], n.r});
        push_data(f4{n.c1.e[0], n.c1.e[1], n.c1.e[2], n.t0});
        push_data(f4{n.t1, 0, 0, 0});
        break;
      case H_XY:
      case H_XZ:
      case H_YZ: {
        int axis = n.kind == H_XY ? 2 : n.kind == H_XZ ? 1 : 0;
        hdr.x = LT_RECT | (axis << LEAF_AXIS_SHIFT);
        push_data(f4{n.a0, n.a1, n.b0, n.b1});
        push_data(f4{n.k, 0, 0, 0});
        break;
      }
      case H_BOX:
        hdr.x = LT_BOX;
        push_data(f4{n.pmin.e[0], n.pmin.e[1], n.pmin.e[2], 0});
        push_data(f4{n.pmax.e[0], n.pmax.e[1], n.pmax.e[2], 0});
        break;
      default:
        return fail(TPT_ERR_UNSUPPORTED, "not a primitive");
    }
    if (flip & 1) hdr.x |= LEAF_FLIP;
    S.leaf_hdr.push_back(hdr);
    S.leaf_user.push_back(n.user);
    return (int)S.leaf_hdr.size() - 1;
  }

  // Flattens the BVH rooted at builder node h into pre-order nodes; leaves
  // are created in left-to-right order.  in_blas: leaves must be primitives.
  // Whether texture t (a checker: either of its children) reads (u, v):
  // only image textures do (texture.cc:27-42).
  bool tex_reads_uv(int t, int guard = 0) const {
    if (t < 0 || t >= (int)B.texs.size() || guard > 16) return false;
    const HTex &x = B.texs[t];
    if (x.kind == TT_IMAGE) return true;
    if (x.kind == TT_CHECKER) return tex_reads_uv(x.odd, guard + 1) || tex_reads_uv(x.even, guard + 1);
    return false;
  }

  int flatten_bvh(int h, bool in_blas, int depth, int &max_depth) {
    if (B.bvh_build == TPT_BVH_SAH) return flatten_sah(h, in_blas, depth, max_depth);
    if (B.bvh_build == TPT_BVH_LBVH) return flatten_lbvh(h, in_blas, depth, max_depth);
    if (depth > max_depth) max_depth = depth;
    const HNode &n = B.nodes[h];
    int me = (int)S.node_lo.size();
    S.node_lo.push_back(f4{n.bbox.mn.e[0], n.bbox.mn.e[1], n.bbox.mn.e[2], 0});
    S.node_hi.push_back(f4{n.bbox.mx.e[0], n.bbox.mx.e[1], n.bbox.mx.e[2], 0});
    S.node_skip.push_back(0);
    int refs[2];
    int ch[2] = {n.left, n.right};
    for (int c = 0; c < 2; c++) {
      if (c == 1 && n.right == n.left) {
        refs[1] = refs[0];
        break;
      }
      const HNode &cn = B.nodes[ch[c]];
      if (cn.kind == H_BVH) {
        refs[c] = flatten_bvh(ch[c], in_blas, depth + 1, max_depth);
      } else {
        int leaf = in_blas ? blas_leaf(ch[c]) : any_leaf(ch[c], 0);
        if (leaf < 0) return -1;
        refs[c] = ~leaf;
      }
      if (st != TPT_OK) return -1;
    }
    int32_t lref = refs[0], rref = refs[1];
    std::memcpy(&S.node_lo[me].w, &lref, 4);
    std::memcpy(&S.node_hi[me].w, &rref, 4);
    S.node_skip[me] = (int32_t)S.node_lo.size();  // subtree = [me, skip)
    return me;
  }

  // ---- alternative topology: binned surface-area-heuristic rebuild of a
  // bvh_node's primitives (Wald 2007, "On fast Construction of SAH-based
  // Bounding Volume Hierarchies"), flattened in the same pre-order layout.
  struct SahLeaf {
    int h;
    box3 box;
    float c[3];
  };

  void sah_collect(int h, float t0, float t1, std::vector<SahLeaf> &out) {
    const HNode &n = B.nodes[h];
    if (n.kind == H_BVH) {
      sah_collect(n.left, t0, t1, out);
      if (n.right != n.left) sah_collect(n.right, t0, t1, out);
      return;
    }
    SahLeaf l;
    l.h = h;
    if (!hbox(B, h, t0, t1, l.box)) {
      fail(TPT_ERR_NO_BOUNDING_BOX, "primitive without a bounding box under bvh_node");
      return;
    }
    for (int a = 0; a < 3; a++) l.c[a] = 0.5f * (l.box.mn.e[a] + l.box.mx.e[a]);
    out.push_back(l);
  }

  static float half_area(const box3 &b) {
    const float x = b.mx.e[0] - b.mn.e[0], y = b.mx.e[1] - b.mn.e[1], z = b.mx.e[2] - b.mn.e[2];
    return x * y + y * z + z * x;
  }

  int sah_leaf_ref(const SahLeaf &l, bool in_blas) {
    const int leaf = in_blas ? blas_leaf(l.h) : any_leaf(l.h, 0);
    return leaf < 0 ? INT32_MIN : ~leaf;
  }

  int flatten_sah(int h, bool in_blas, int depth, int &max_depth) {
    std::vector<SahLeaf> leaves;
    sah_collect(h, B.nodes[h].t0, B.nodes[h].t1, leaves);
    if (st != TPT_OK || leaves.empty()) return -1;
    return sah_emit(leaves, 0, (int)leaves.size(), in_blas, depth, max_depth);
  }

  // SAH splits down to depth 16, then halving by count: a 5000-primitive
  // tree stays within the device traversal stack.
  int sah_emit(std::vector<SahLeaf> &sah_leaves, int b, int e, bool in_blas, int depth, int &max_depth) {
    if (depth > max_depth) max_depth = depth;
    box3 bb = sah_leaves[b].box, cb{};
    for (int a = 0; a < 3; a++) cb.mn.e[a] = cb.mx.e[a] = sah_leaves[b].c[a];
    for (int i = b + 1; i < e; i++) {
      bb = surround(bb, sah_leaves[i].box);
      for (int a = 0; a < 3; a++) {
        cb.mn.e[a] = std::min(cb.mn.e[a], sah_leaves[i].c[a]);
        cb.mx.e[a] = std::max(cb.mx.e[a], sah_leaves[i].c[a]);
      }
    }
    const int me = (int)S.node_lo.size();
    S.node_lo.push_back(f4{bb.mn.e[0], bb.mn.e[1], bb.mn.e[2], 0});
    S.node_hi.push_back(f4{bb.mx.e[0], bb.mx.e[1], bb.mx.e[2], 0});
    S.node_skip.push_back(0);
    int mid = b + 1;
    if (e - b > 1) {
      // 16 bins per axis on the centroid bounds; cost = A_l N_l + A_r N_r
      enum { BINS = 16 };
      float best = std::numeric_limits<float>::infinity();
      int best_axis = -1, best_bin = 0;
      for (int a = 0; a < 3 && depth < 16; a++) {
        const float lo = cb.mn.e[a], ext = cb.mx.e[a] - lo;
        if (!(ext > 0.f)) continue;
        int cnt[BINS] = {};
        box3 bx[BINS];
        for (int i = b; i < e; i++) {
          int k = (int)((sah_leaves[i].c[a] - lo) / ext * BINS);
          k = std::min(std::max(k, 0), BINS - 1);
          bx[k] = cnt[k] ? surround(bx[k], sah_leaves[i].box) : sah_leaves[i].box;
          cnt[k]++;
        }
        float right_area[BINS];
        int right_n[BINS];
        box3 acc{};
        int n = 0;
        for (int k = BINS - 1; k > 0; k--) {
          if (cnt[k]) acc = n ? surround(acc, bx[k]) : bx[k];
          n += cnt[k];
          right_area[k] = n ? half_area(acc) : 0.f;
          right_n[k] = n;
        }
        acc = box3{};
        n = 0;
        for (int k = 0; k < BINS - 1; k++) {
          if (cnt[k]) acc = n ? surround(acc, bx[k]) : bx[k];
          n += cnt[k];
          if (n == 0 || right_n[k + 1] == 0) continue;
          const float cost = half_area(acc) * n + right_area[k + 1] * right_n[k + 1];
          if (cost < best) {
            best = cost;
            best_axis = a;
            best_bin = k;
          }
        }
      }
      if (best_axis >= 0) {
        const float lo = cb.mn.e[best_axis], ext = cb.mx.e[best_axis] - lo;
        auto it = std::stable_partition(sah_leaves.begin() + b, sah_leaves.begin() + e, [&](const SahLeaf &l) {
          int k = (int)((l.c[best_axis] - lo) / ext * BINS);
          return std::min(std::max(k, 0), (int)BINS - 1) <= best_bin;
        });
        mid = (int)(it - sah_leaves.begin());
      }
      if (best_axis < 0 || mid <= b || mid >= e) {  // coincident centroids or too deep: halve by count
        int a = 0;
        for (int k = 1; k < 3; k++)
          if (cb.mx.e[k] - cb.mn.e[k] > cb.mx.e[a] - cb.mn.e[a]) a = k;
        std::stable_sort(sah_leaves.begin() + b, sah_leaves.begin() + e,
                         [a](const SahLeaf &x, const SahLeaf &y) { return x.c[a] < y.c[a]; });
        mid = b + (e - b) / 2;
      }
    }
    int refs[2];
    const int rb[2] = {b, mid}, re[2] = {mid, e};
    for (int c = 0; c < 2; c++) {
      if (e - b == 1) {  // a single primitive: left == right, as bvh_node with n == 1
        refs[1] = refs[0] = sah_leaf_ref(sah_leaves[b], in_blas);
        break;
      }
      refs[c] = re[c] - rb[c] == 1 ? sah_leaf_ref(sah_leaves[rb[c]], in_blas)
                                   : sah_emit(sah_leaves, rb[c], re[c], in_blas, depth + 1, max_depth);
      if (st != TPT_OK) return -1;
    }
    if (st != TPT_OK) return -1;
    std::memcpy(&S.node_lo[me].w, &refs[0], 4);
    std::memcpy(&S.node_hi[me].w, &refs[1], 4);
    S.node_skip[me] = (int32_t)S.node_lo.size();
    return me;
  }

  // ---- alternative topology built on the GPU (lbvh.cu): the primitives'
  // leaves in the caller's order, their boxes and max(n - 1, 1) reserved
  // node slots become one build job.
  void lbvh_collect(int h, float t0, float t1, std::vector<SahLeaf> &out, int guard = 0) {
    const HNode &n = B.nodes[h];
    if (n.kind == H_BVH && !n.items.empty() && guard < 64) {
      for (int c : n.items) lbvh_collect(c, t0, t1, out, guard + 1);
      return;
    }
    sah_collect(h, t0, t1, out);
  }

  int flatten_lbvh(int h, bool in_blas, int depth, int &max_depth) {
    if (depth > max_depth) max_depth = depth;  // the device build reports the rest
    std::vector<SahLeaf> leaves;
    lbvh_collect(h, B.nodes[h].t0, B.nodes[h].t1, leaves);
    if (st != TPT_OK || leaves.empty()) return -1;
    const int n = (int)leaves.size();
    std::vector<int32_t> refs(n);
    for (int i = 0; i < n; i++) {  // leaves before nodes: the job's slots stay contiguous
      refs[i] = sah_leaf_ref(leaves[i], in_blas);
      if (st != TPT_OK) return -1;
    }
    const int me = (int)S.node_lo.size(), slots = n > 1 ? n - 1 : 1;
    S.node_lo.resize(me + slots, f4{0, 0, 0, 0});
    S.node_hi.resize(me + slots, f4{0, 0, 0, 0});
    S.node_skip.resize(me + slots, 0);
    const int32_t job = (int32_t)S.lbvh_jobs.size();
    const int64_t pad = lbvh_pad(n);
    S.lbvh_jobs.push_back(i4{me, n, (int32_t)(S.lbvh_prims.size() / 2), (int32_t)S.lbvh_keys});
    S.lbvh_keys += pad;
    S.lbvh_max_pad = std::max(S.lbvh_max_pad, (int32_t)pad);
    S.lbvh_blas.push_back(in_blas ? 1 : 0);
    for (int i = 0; i < n; i++) {
      f4 lo{leaves[i].box.mn.e[0], leaves[i].box.mn.e[1], leaves[i].box.mn.e[2], 0};
      f4 hi{leaves[i].box.mx.e[0], leaves[i].box.mx.e[1], leaves[i].box.mx.e[2], 0};
      std::memcpy(&lo.w, &refs[i], 4);
      std::memcpy(&hi.w, &job, 4);
      S.lbvh_prims.push_back(lo);
      S.lbvh_prims.push_back(hi);
    }
    return me;
  }

  int blas_leaf(int h) {
    int flip = 0;
    while (B.nodes[h].kind == H_FLIP) {
      flip ^= 1;
      h = B.nodes[h].child;
    }
    int k = B.nodes[h].kind;
    if (k == H_SPHERE || k == H_MSPHERE || k == H_XY || k == H_XZ || k == H_YZ || k == H_BOX) return prim_leaf(h, flip);
    return fail(TPT_ERR_UNSUPPORTED, "instanced BVH may only hold primitives");
  }

  // Leaf for any non-list, non-BVH hitable reached from the top level or from
  // a top-level BVH.
  int any_leaf(int h, int flip) {
    const HNode &n = B.nodes[h];
    switch (n.kind) {
      case H_SPHERE:
      case H_MSPHERE:
      case H_XY:
      case H_XZ:
      case H_YZ:
      case H_BOX:
        return prim_leaf(h, flip);
      case H_FLIP:
        return any_leaf(n.child, flip ^ 1);
      case H_TRANSLATE:
      case H_ROTY:
        return instance_leaf(h, flip);
      case H_MEDIUM: {
        int bnd = boundary_leaf(n.child);
        if (bnd < 0) return -1;
        i4 hdr{LT_MEDIUM, (int32_t)S.leaf_data.size(), -1, bnd};
        push_data(f4{n.density, 0, 0, 0});
        // the phase function: isotropic(texture) (hitable.cc:92-96)
        i4 mi{MT_ISOTROPIC, n.phase_tex, 0, tex_reads_uv(n.phase_tex) ? 1 : 0};
        S.mat_i.push_back(mi);
        S.mat_f.push_back(f4{0, 0, 0, 0});
        hdr.z = (int)S.mat_i.size() - 1;
        S.leaf_hdr.push_back(hdr);
        S.leaf_user.push_back(n.user);
        return (int)S.leaf_hdr.size() - 1;
      }
      case H_LIST:
        return fail(TPT_ERR_UNSUPPORTED, "hitable_list below a bvh_node or transform");
      case H_BVH:
        return fail(TPT_ERR_UNSUPPORTED, "bvh_node as a leaf");
    }
    return fail(TPT_ERR_UNSUPPORTED, "unknown hitable");
  }

  int boundary_leaf(int h) {
    int flip = 0;
    while (B.nodes[h].kind == H_FLIP) {
      flip ^= 1;
      h = B.nodes[h].child;
    }
    int k = B.nodes[h].kind;
    if (k == H_TRANSLATE || k == H_ROTY) {
      int leaf = instance_leaf(h, flip);
      if (leaf < 0) return -1;
      int child = S.leaf_hdr[leaf].w;
      if (child >= 0) return fail(TPT_ERR_UNSUPPORTED, "medium boundary must be a single primitive");
      return leaf;
    }
    if (k == H_SPHERE || k == H_MSPHERE || k == H_XY || k == H_XZ || k == H_YZ || k == H_BOX) return prim_leaf(h, flip);
    return fail(TPT_ERR_UNSUPPORTED, "medium boundary must be a primitive or a transformed primitive");
  }

  // translate / rotate_y chains become one instance leaf whose ops are
  // applied to the ray in world-to-object order.
  int instance_leaf(int h, int flip) {
    std::vector<f4> ops;
    int cur = h;
    for (;;) {
      const HNode &n = B.nodes[cur];
      if (n.kind == H_TRANSLATE) {
        ops.push_back(f4{(float)OP_TRANSLATE, n.off.e[0], n.off.e[1], n.off.e[2]});
        cur = n.child;
      } else if (n.kind == H_ROTY) {
        ops.push_back(f4{(float)OP_ROTATE_Y, n.sn, n.cs, 0});
        cur = n.child;
      } else if (n.kind == H_FLIP) {
        flip ^= 1;
        cur = n.child;
      } else {
        break;
      }
    }
    if ((int)ops.size() > MAX_INSTANCE_OPS) return fail(TPT_ERR_UNSUPPORTED, "transform chain longer than 4");
    const HNode &child = B.nodes[cur];
    int32_t child_ref;
    if (child.kind == H_BVH) {
      auto it = blas_root.find(cur);
      if (it != blas_root.end()) {
        child_ref = it->second;
      } else {
        int md = 0;
        int root = flatten_bvh(cur, true, 1, md);
        if (root < 0) return -1;
        blas_root[cur] = root;
        S.blas_depth = std::max(S.blas_depth, md);
        S.n_blas++;
        child_ref = root;
      }
    } else {
      int leaf = blas_leaf(cur);
      if (leaf < 0) return -1;
      child_ref = ~leaf;
    }
    i4 hdr{LT_INSTANCE | ((flip & 1) ? LEAF_FLIP : 0), (int32_t)S.leaf_data.size(), -1, child_ref};
    push_data(f4{(float)ops.size(), 0, 0, 0});
    for (const f4 &o : ops) push_data(o);
    S.leaf_hdr.push_back(hdr);
    S.leaf_user.push_back(B.nodes[h].user);
    return (int)S.leaf_hdr.size() - 1;
  }

  // Instanced BVHs are flattened before the top level so that every BVH
  // owns a contiguous pre-order range (the stackless walk relies on it).
  void flatten_instanced(int h, std::vector<char> &seen) {
    if (seen[h]) return;
    seen[h] = 1;
    const HNode &n = B.nodes[h];
    switch (n.kind) {
      case H_TRANSLATE:
      case H_ROTY: {
        int cur = n.child;
        while (B.nodes[cur].kind == H_TRANSLATE || B.nodes[cur].kind == H_ROTY || B.nodes[cur].kind == H_FLIP)
          cur = B.nodes[cur].child;
        if (B.nodes[cur].kind == H_BVH && !blas_root.count(cur)) {
          int md = 0;
          int root = flatten_bvh(cur, true, 1, md);
          if (root < 0) return;
          blas_root[cur] = root;
          S.blas_depth = std::max(S.blas_depth, md);
          S.n_blas++;
        }
        return;
      }
      case H_FLIP:
      case H_MEDIUM:
        flatten_instanced(n.child, seen);
        return;
      case H_LIST:
        for (int it : n.items) flatten_instanced(it, seen);
        return;
      case H_BVH:
        flatten_instanced(n.left, seen);
        flatten_instanced(n.right, seen);
        return;
      default:
        return;
    }
  }

  void flatten_list(int h, std::vector<int> &out) {
    const HNode &n = B.nodes[h];
    for (int it : n.items) {
      if (B.nodes[it].kind == H_LIST)
        flatten_list(it, out);  // sequential semantics compose: nested lists flatten exactly
      else
        out.push_back(it);
    }
  }

  // light_shape -> flat item table with pick weights (hitable_list.cc:24-36).
  void add_light(int h, float weight) {
    const HNode &n = B.nodes[h];
    if (n.kind == H_LIST) {
      if (n.items.empty()) return;
      float w = 1.0 / n.items.size();
      for (int it : n.items) add_light(it, weight * w);
      return;
    }
    i4 li{LS_NONE, 0, 0, 0};
    f4 a{0, 0, 0, 0};
    if (n.kind == H_XZ) {
      li.x = LS_XZ_RECT;
      a = f4{n.a0, n.a1, n.b0, n.b1};
    } else if (n.kind == H_SPHERE) {
      li.x = LS_SPHERE;
      a = f4{n.c0.e[0], n.c0.e[1], n.c0.e[2], n.r};
    }
    S.light_i.push_back(li);
    S.light_f.push_back(a);
    S.light_f.push_back(f4{n.k, weight, 0, 0});
  }

  tpt_status run() {
    if (B.world < 0) return fail(TPT_ERR_INVALID_ARGUMENT, "no world"), st;
    // textures
    for (const HTex &t : B.texs) {
      i4 ti{t.kind, 0, 0, 0};
      f4 tf{0, 0, 0, 0};
      if (t.kind == TT_CONST) tf = f4{t.c[0], t.c[1], t.c[2], 0};
      if (t.kind == TT_CHECKER) { ti.y = t.odd; ti.z = t.even; }
      if (t.kind == TT_PERLIN) tf.x = t.scale;
      if (t.kind == TT_IMAGE) {
        ti.y = t.w;
        ti.z = t.h;
        ti.w = (int32_t)S.images.size();
        S.images.insert(S.images.end(), t.px.begin(), t.px.end());
      }
      S.tex_i.push_back(ti);
      S.tex_f.push_back(tf);
    }
    // materials
    for (const HMat &m : B.mats) {
      i4 mi{m.kind, m.tex, 0, tex_reads_uv(m.tex) ? 1 : 0};
      f4 mf{m.albedo[0], m.albedo[1], m.albedo[2], m.fuzz};
      if (m.kind == MT_DIELECTRIC) mf = f4{m.ior, 0, 0, 0};
      S.mat_i.push_back(mi);
      S.mat_f.push_back(mf);
    }
    for (int i = 0; i < 256; i++)
      S.perlin_grad.push_back(f4{B.pgrad[3 * i], B.pgrad[3 * i + 1], B.pgrad[3 * i + 2], 0});
    S.perlin_perm.assign(B.pperm, B.pperm + 768);
    // world
    std::vector<int> items;
    if (B.nodes[B.world].kind == H_LIST)
      flatten_list(B.world, items);
    else
      items.push_back(B.world);
    int top_depth = 0;
    {
      std::vector<char> seen(B.nodes.size(), 0);
      for (int h : items) flatten_instanced(h, seen);
      if (st != TPT_OK) return st;
    }
    for (int h : items) {
      if (B.nodes[h].kind == H_BVH) {
        int md = 0;
        int root = flatten_bvh(h, false, 1, md);
        if (root < 0) return st == TPT_OK ? TPT_ERR_UNSUPPORTED : st;
        top_depth = std::max(top_depth, md);
        S.items.push_back(i2{ITEM_BVH, root});
      } else {
        int leaf = any_leaf(h, 0);
        if (leaf < 0) return st == TPT_OK ? TPT_ERR_UNSUPPORTED : st;
        S.items.push_back(i2{ITEM_LEAF, leaf});
      }
    }
    // child boxes of every node, for the stack walk: one 64-byte load per
    // popped node gives both children's boxes and references
    S.node_kids.assign(4 * S.node_lo.size(), f4{0, 0, 0, 0});
    for (size_t i = 0; i < S.node_lo.size(); i++) {
      int32_t ref[2];
      std::memcpy(&ref[0], &S.node_lo[i].w, 4);
      std::memcpy(&ref[1], &S.node_hi[i].w, 4);
      for (int c = 0; c < 2; c++) {
        f4 lo{0, 0, 0, 0}, hi{0, 0, 0, 0};
        if (ref[c] >= 0) {
          lo = S.node_lo[ref[c]];
          hi = S.node_hi[ref[c]];
          // the box's size term of the pruning bound, in the device's order
          // of float operations (prune_key)
          hi.w = ((hi.x - lo.x) + (hi.y - lo.y)) + (hi.z - lo.z);
        } else if ((S.leaf_hdr[~ref[c]].x & LEAF_TYPE_MASK) == LT_SPHERE) {
          // a sphere leaf carries its {center, radius} (flag hi.y = 1): the
          // stack walk tests it without loading the leaf
          const f4 sp = S.leaf_data[S.leaf_hdr[~ref[c]].y];
          lo = f4{sp.x, sp.y, sp.z, 0};
          hi = f4{sp.w, 1.f, 0, 0};
        }
        std::memcpy(&lo.w, &ref[c], 4);
        S.node_kids[4 * i + 2 * c] = lo;
        S.node_kids[4 * i + 2 * c + 1] = hi;
      }
    }
    // stack bound: both children of every level plus the instance marker
    S.max_stack = top_depth + 2 + (S.n_blas ? S.blas_depth + 2 : 0);
    if (S.max_stack > TRAVERSAL_STACK)
      return fail(TPT_ERR_STACK_OVERFLOW, "BVH deeper than the device traversal stack"), st;
    // lights
    S.light_is_list = 0;
    S.has_lights = B.lights >= 0;
    if (B.lights >= 0) {
      S.light_is_list = B.nodes[B.lights].kind == H_LIST;
      add_light(B.lights, 1.0f);
      float cdf = 0;
      for (size_t i = 0; i < S.light_i.size(); i++) {
        cdf += S.light_f[2 * i + 1].y;
        S.light_f[2 * i + 1].z = cdf;
      }
      if (S.light_i.empty()) S.has_lights = 0;  // empty list: reference UB; treated as no lights
    }
    if (!B.has_cam) return fail(TPT_ERR_INVALID_ARGUMENT, "no camera"), st;
    {
      box3 wb;
      if (hbox(B, B.world, 0, 0, wb))
        for (int i = 0; i < 3; i++) {
          S.world_lo[i] = wb.mn.e[i];
          S.world_hi[i] = wb.mx.e[i];
        }
    }
    S.cam = B.cam;
    std::memcpy(S.cam_in, B.cam_in, sizeof(S.cam_in));
    // keep the BVH trees for topology dumps
    return st;
  }
};

}  // namespace

// ============================================================ scene API ===
struct tpt_scene {
  HostScene S;
  std::shared_ptr<tpt_builder> builder;  // for topology dumps
};

static void dump_tree(const tpt_builder &B, int h, std::vector<float> &boxes, std::vector<int> &kids) {
  const HNode &n = B.nodes[h];
  int me = (int)kids.size() / 2;
  kids.push_back(0);
  kids.push_back(0);
  for (int i = 0; i < 3; i++) boxes.push_back(n.bbox.mn.e[i]);
  for (int i = 0; i < 3; i++) boxes.push_back(n.bbox.mx.e[i]);
  int ch[2] = {n.left, n.right};
  for (int c = 0; c < 2; c++) {
    const HNode &cn = B.nodes[ch[c]];
    int ref;
    if (cn.kind == H_BVH && cn.internal) {
      ref = (int)kids.size() / 2;
      dump_tree(B, ch[c], boxes, kids);
    } else {
      ref = -(1 + cn.user);
    }
    kids[2 * me + c] = ref;
  }
}

namespace tpt {
const HostScene *host_scene(const tpt_scene *s) { return s ? &s->S : nullptr; }
}  // namespace tpt

extern "C" {

tpt_status tpt_scene_compile(const tpt_builder *b, tpt_scene **out) {
  if (!b || !out) return TPT_ERR_INVALID_ARGUMENT;
  auto *sc = new tpt_scene();
  Compiler C(*b, sc->S);
  tpt_status st = C.run();
  if (st != TPT_OK) {
    delete sc;
    return st;
  }
  sc->builder = std::make_shared<tpt_builder>(*b);
  *out = sc;
  return TPT_OK;
}

void tpt_scene_destroy(tpt_scene *s) { delete s; }

tpt_status tpt_scene_get_info(const tpt_scene *s, tpt_scene_info *o) {
  if (!s || !o) return TPT_ERR_INVALID_ARGUMENT;
  const HostScene &S = s->S;
  o->n_nodes = (int32_t)S.node_lo.size();
  o->n_leaves = (int32_t)S.leaf_hdr.size();
  o->n_items = (int32_t)S.items.size();
  o->n_blas = S.n_blas;
  o->n_materials = (int32_t)S.mat_i.size();
  o->n_textures = (int32_t)S.tex_i.size();
  o->n_lights = (int32_t)S.light_i.size();
  o->max_stack = S.max_stack;
  o->arena_bytes = (int64_t)arena_bytes(S);
  return TPT_OK;
}

int32_t tpt_scene_bvh_dump(const tpt_scene *s, int32_t user, float *boxes, int32_t *kids, int32_t cap) {
  if (!s) return -TPT_ERR_INVALID_ARGUMENT;
  const tpt_builder &B = *s->builder;
  auto it = B.handle_of_user.find(user);
  if (it == B.handle_of_user.end() || B.nodes[it->second].kind != H_BVH) return -TPT_ERR_BAD_HANDLE;
  std::vector<float> bx;
  std::vector<int> kd;
  dump_tree(B, it->second, bx, kd);
  int n = (int)kd.size() / 2;
  if (n > cap) return n;
  std::memcpy(boxes, bx.data(), bx.size() * sizeof(float));
  std::memcpy(kids, kd.data(), kd.size() * sizeof(int));
  return n;
}

// Scene-description text (one statement per line; format in the package's
// loader documentation): builder calls in file order, SD ids kept as the
// user ids reported for hits and dumps.
tpt_status tpt_scene_from_text(const char *text, tpt_scene **out, char *err, size_t errlen) {
  return tpt_scene_from_text_opt(text, TPT_BVH_REFERENCE, out, err, errlen);
}

tpt_status tpt_scene_from_text_opt(const char *text, int32_t bvh_build, tpt_scene **out, char *err, size_t errlen) {
  if (!text || !out) return TPT_ERR_INVALID_ARGUMENT;
  tpt_builder *b = nullptr;
  tpt_builder_create(&b);
  std::unique_ptr<tpt_builder> guard(b);
  if (tpt_builder_set_bvh_build(b, bvh_build) != TPT_OK) return TPT_ERR_INVALID_ARGUMENT;
  b->perlin_draws = false;  // scene text carries explicit perlin tables
  b->auto_user = false;     // hits and dumps report SD ids
  std::unordered_map<int, int> tex, mat, node;
  std::istringstream in(text);
  std::string ln, msg;
  int lineno = 0;
  tpt_status st = TPT_OK;
  auto bad = [&](tpt_status code, const std::string &m) {
    st = code;
    msg = m;
  };
  while (st == TPT_OK && std::getline(in, ln)) {
    lineno++;
    std::istringstream is(ln);
    std::string kw;
    if (!(is >> kw) || kw[0] == '#') continue;
    bool ok = true;
    auto F = [&]() -> float {
      std::string s;
      if (!(is >> s)) { ok = false; return 0.f; }
      char *end = nullptr;
      float v = std::strtof(s.c_str(), &end);
      if (end == s.c_str()) ok = false;
      return v;
    };
    auto I = [&]() -> int {
      long v = 0;
      if (!(is >> v)) ok = false;
      return (int)v;
    };
    auto look = [&](std::unordered_map<int, int> &m, int id) -> int {
      auto it = m.find(id);
      if (it == m.end()) { ok = false; return -1; }
      return it->second;
    };
    int32_t h = 0;
    if (kw == "tex") {
      int id = I();
      std::string ty;
      is >> ty;
      if (ty == "const") { float r = F(), g = F(), bl = F(); h = tpt_constant_texture(b, r, g, bl); }
      else if (ty == "checker") { int o = look(tex, I()), e = look(tex, I()); if (ok) h = tpt_checker_texture(b, o, e); }
      else if (ty == "perlin") { h = tpt_perlin_noise_texture(b, F()); }
      else if (ty == "image") {
        int w = I(), hh = I();
        uint32_t seed = (uint32_t)I();
        if (ok && w > 0 && hh > 0) {
          std::vector<uint8_t> px((size_t)w * hh * 3);
          procedural_image(w, hh, seed, px.data());
          h = tpt_image_texture(b, px.data(), w, hh);
        } else {
          ok = false;
        }
      } else { ok = false; }
      if (ok && h >= 0) tex[id] = h;
    } else if (kw == "perlin_tables") {
      std::vector<float> g(768);
      std::vector<int32_t> p(768);
      for (float &x : g) x = F();
      for (int32_t &x : p) x = I();
      if (ok) tpt_perlin_tables(b, g.data(), p.data());
    } else if (kw == "mat") {
      int id = I();
      std::string ty;
      is >> ty;
      if (ty == "lambertian") { int t = look(tex, I()); if (ok) h = tpt_lambertian(b, t); }
      else if (ty == "metal") { float r = F(), g = F(), bl = F(), f = F(); h = tpt_metal(b, r, g, bl, f); }
      else if (ty == "dielectric") { h = tpt_dielectric(b, F()); }
      else if (ty == "diffuse_light") { int t = look(tex, I()); if (ok) h = tpt_diffuse_light(b, t); }
      else if (ty == "isotropic") { int t = look(tex, I()); if (ok) h = tpt_isotropic(b, t); }
      else { ok = false; }
      if (ok && h >= 0) mat[id] = h;
    } else if (kw == "node") {
      int id = I();
      std::string ty;
      is >> ty;
      if (ty == "sphere") {
        float x = F(), y = F(), z = F(), r = F();
        int m = look(mat, I());
        if (ok) h = tpt_sphere(b, x, y, z, r, m);
      } else if (ty == "moving_sphere") {
        float v[9];
        for (float &x : v) x = F();
        int m = look(mat, I());
        if (ok) h = tpt_moving_sphere(b, v[0], v[1], v[2], v[3], v[4], v[5], v[6], v[7], v[8], m);
      } else if (ty == "xy_rect" || ty == "xz_rect" || ty == "yz_rect") {
        float a0 = F(), a1 = F(), b0 = F(), b1 = F(), k = F();
        int m = look(mat, I());
        if (ok) {
          if (ty == "xy_rect") h = tpt_xy_rect(b, a0, a1, b0, b1, k, m);
          else if (ty == "xz_rect") h = tpt_xz_rect(b, a0, a1, b0, b1, k, m);
          else h = tpt_yz_rect(b, a0, a1, b0, b1, k, m);
        }
      } else if (ty == "flip_normal") {
        int c = look(node, I());
        if (ok) h = tpt_flip_normal(b, c);
      } else if (ty == "box") {
        float v[6];
        for (float &x : v) x = F();
        int m = look(mat, I());
        if (ok) h = tpt_box(b, v[0], v[1], v[2], v[3], v[4], v[5], m);
      } else if (ty == "translate") {
        int c = look(node, I());
        float x = F(), y = F(), z = F();
        if (ok) h = tpt_translate(b, c, x, y, z);
      } else if (ty == "rotate_y") {
        int c = look(node, I());
        float a = F();
        if (ok) h = tpt_rotate_y(b, c, a);
      } else if (ty == "constant_medium") {
        int c = look(node, I());
        float d = F();
        int t = look(tex, I());
        if (ok) h = tpt_constant_medium(b, c, d, t);
      } else if (ty == "hitable_list" || ty == "bvh_node") {
        float t0 = 0, t1 = 0;
        if (ty == "bvh_node") { t0 = F(); t1 = F(); }
        int n = I();
        std::vector<int32_t> l;
        for (int i = 0; ok && i < n; i++) l.push_back(look(node, I()));
        if (ok) h = ty == "bvh_node" ? tpt_bvh_node(b, l.data(), n, t0, t1) : tpt_hitable_list(b, l.data(), n);
      } else {
        ok = false;
      }
      if (ok && h >= 0) {
        node[id] = h;
        b->set_user(h, id);  // the SD id becomes the user id of the hitable
      }
    } else if (kw == "world") {
      int w = look(node, I());
      if (ok) h = tpt_builder_set_world(b, w);
      if (h > 0) h = -h;
    } else if (kw == "lights") {
      int l = look(node, I());
      if (ok) h = tpt_builder_set_light_shape(b, l);
      if (h > 0) h = -h;
    } else if (kw == "camera") {
      float v[15];
      for (float &x : v) x = F();
      if (ok) h = -tpt_builder_set_camera(b, v, v + 3, v + 6, v[9], v[10], v[11], v[12], v[13], v[14]);
    } else {
      ok = false;
    }
    if (!ok) bad(TPT_ERR_PARSE, "line " + std::to_string(lineno) + ": cannot parse '" + kw + "'");
    else if (h < 0) bad(-h, "line " + std::to_string(lineno) + ": " + tpt_status_string(-h));
  }
  if (st == TPT_OK) {
    st = tpt_scene_compile(b, out);
    if (st != TPT_OK) msg = std::string("compile: ") + tpt_status_string(st);
  }
  if (st != TPT_OK && err && errlen) std::snprintf(err, errlen, "%s", msg.c_str());
  return st;
}

void tpt_quantize(const float *mean_rgb, int64_t n_pixels, uint8_t *rgb8) {
  for (int64_t i = 0; i < 3 * n_pixels; i++) {
    float c = std::sqrt(mean_rgb[i]);
    int q = int(255.99f * c);  // main.cpp:137-139
    if (q < 0) q = 0;          // main.cpp:176-182
    if (q > 255) q = 255;
    rgb8[i] = (uint8_t)q;
  }
}

tpt_status tpt_scene_get_camera(const tpt_scene *s, float out[15]) {
  if (!s || !out) return TPT_ERR_INVALID_ARGUMENT;
  std::memcpy(out, s->S.cam_in, sizeof(s->S.cam_in));
  return TPT_OK;
}

tpt_status tpt_scene_set_camera(tpt_scene *s, const float lf[3], const float la[3], const float up[3], float vfov,
                                float aspect, float aperture, float focus, float t0, float t1) {
  if (!s || !lf || !la || !up) return TPT_ERR_INVALID_ARGUMENT;
  s->S.cam = make_camera(lf, la, up, vfov, aspect, aperture, focus, t0, t1);
  camera_inputs(lf, la, up, vfov, aspect, aperture, focus, t0, t1, s->S.cam_in);
  return TPT_OK;
}

tpt_status tpt_write_ppm(const char *path, const uint8_t *rgb8, int32_t w, int32_t h) {
  if (!path || !rgb8 || w <= 0 || h <= 0) return TPT_ERR_INVALID_ARGUMENT;
  FILE *f = std::fopen(path, "w");
  if (!f) return TPT_ERR_INVALID_ARGUMENT;
  std::fprintf(f, "P3\n%d %d\n255\n", w, h);  // main.cpp:69
  for (int64_t i = 0; i < (int64_t)w * h; i++)
    std::fprintf(f, "%d %d %d \n", rgb8[3 * i], rgb8[3 * i + 1], rgb8[3 * i + 2]);
  std::fclose(f);
  return TPT_OK;
}

}  // extern "C"
