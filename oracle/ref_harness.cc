// ref_harness.cc - drives the UNMODIFIED reference sources (compiled from the
// reference checkout by oracle/Makefile, never copied) through their own
// public classes, for pinning the oracle and for the CPU baseline.
//
// TEST INFRASTRUCTURE ONLY.  Scenes come from the same SD text the oracle and
// the product read (format in oracle.h).  Every primitive gets its own copy of
// its material, so rec.mat_ptr identifies the primitive that was hit: the
// reference's hit_record carries no primitive id.  Scene construction runs on
// a fresh std::thread so that bvh_node draws its axes from a drand_r stream in
// its default state (utils.cc:28-32), exactly like the oracle and the product.
#include <atomic>
#include <cfloat>
#include <chrono>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <future>
#include <limits>
#include <map>
#include <mutex>
#include <sstream>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "camera.h"
#include "inipp.h"
#include "hitable.h"
#include "hitable_list.h"
#include "material.h"
#include "rect_box.h"
#include "sphere.h"
#include "texture.h"
#include "utils.h"
#include "vec3.h"

extern "C" void oracle_procedural_image(int32_t w, int32_t h, uint32_t seed, uint8_t *rgb);

namespace {

enum { MK_LAMB = 1, MK_METAL, MK_DIEL, MK_LIGHT, MK_ISO };

struct RefScene {
  std::unordered_map<int, texture *> tex;
  std::unordered_map<int, material *> mat;
  std::unordered_map<int, int> mat_kind;
  std::unordered_map<int, hitable *> node;
  std::unordered_map<const hitable *, int> sd_of_node;
  std::unordered_map<const material *, int> prim_of_mat;
  std::unordered_map<const hitable *, int> bvh_roots;  // SD-level bvh_node objects
  std::vector<std::vector<uint8_t> *> images;
  hitable *world = nullptr;
  hitable *lights = nullptr;
  camera *cam = nullptr;
  bool has_perlin = false;
  vec3 pgrad[256];
  int pperm[3][256];
  std::string err;
};

material *copy_material(RefScene &R, int sd_mat, int prim) {
  auto it = R.mat.find(sd_mat);
  if (it == R.mat.end()) {
    R.err = "undefined material";
    return nullptr;
  }
  material *m = it->second, *c = nullptr;
  switch (R.mat_kind[sd_mat]) {
    case MK_LAMB: c = new lambertian(*static_cast<lambertian *>(m)); break;
    case MK_METAL: c = new metal(*static_cast<metal *>(m)); break;
    case MK_DIEL: c = new dielectric(*static_cast<dielectric *>(m)); break;
    case MK_LIGHT: c = new diffuse_light(*static_cast<diffuse_light *>(m)); break;
    case MK_ISO: c = new isotropic(*static_cast<isotropic *>(m)); break;
  }
  R.prim_of_mat[c] = prim;
  return c;
}

bool parse_line(RefScene &R, const std::string &ln) {
  std::istringstream is(ln);
  std::string kw;
  if (!(is >> kw) || kw[0] == '#') return true;
  auto F = [&is]() -> float {
    std::string s;
    is >> s;
    return std::strtof(s.c_str(), nullptr);
  };
  auto I = [&is]() -> int {
    long v = -1;
    is >> v;
    return (int)v;
  };
  auto N = [&R](int id) -> hitable * {
    auto it = R.node.find(id);
    if (it == R.node.end()) {
      R.err = "undefined node";
      return nullptr;
    }
    return it->second;
  };
  auto T = [&R](int id) -> texture * {
    auto it = R.tex.find(id);
    if (it == R.tex.end()) {
      R.err = "undefined texture";
      return nullptr;
    }
    return it->second;
  };
  if (kw == "tex") {
    int id = I();
    std::string ty;
    is >> ty;
    if (ty == "const") {
      float r = F(), g = F(), b = F();
      R.tex[id] = new constant_texture(vec3(r, g, b));
    } else if (ty == "checker") {
      texture *o = T(I()), *e = T(I());
      R.tex[id] = new checker_texture(o, e);
    } else if (ty == "perlin") {
      float sc = F();
      // The constructor refills the shared static tables from drand_r and a
      // clock-seeded shuffle (perlin_noise.cc:3-21).  Run it on a throwaway
      // thread so the scene thread's drand_r stream is untouched; the SD
      // tables are written back after the scene is built.
      perlin_noise_texture *pt = nullptr;
      std::thread th([&pt, sc]() { pt = new perlin_noise_texture(sc); });
      th.join();
      R.tex[id] = pt;
    } else if (ty == "image") {
      int w = I(), h = I();
      uint32_t seed = (uint32_t)I();
      auto *buf = new std::vector<uint8_t>((size_t)w * h * 3);
      oracle_procedural_image(w, h, seed, buf->data());
      R.images.push_back(buf);
      R.tex[id] = new image_texture(buf->data(), w, h);
    } else {
      R.err = "unknown texture";
      return false;
    }
  } else if (kw == "perlin_tables") {
    for (int i = 0; i < 256; i++) {
      float x = F(), y = F(), z = F();
      R.pgrad[i] = vec3(x, y, z);
    }
    for (int a = 0; a < 3; a++)
      for (int i = 0; i < 256; i++) R.pperm[a][i] = I() & 255;
    R.has_perlin = true;
  } else if (kw == "mat") {
    int id = I();
    std::string ty;
    is >> ty;
    if (ty == "lambertian") {
      R.mat[id] = new lambertian(T(I()));
      R.mat_kind[id] = MK_LAMB;
    } else if (ty == "metal") {
      float r = F(), g = F(), b = F(), f = F();
      R.mat[id] = new metal(vec3(r, g, b), f);
      R.mat_kind[id] = MK_METAL;
    } else if (ty == "dielectric") {
      R.mat[id] = new dielectric(F());
      R.mat_kind[id] = MK_DIEL;
    } else if (ty == "diffuse_light") {
      R.mat[id] = new diffuse_light(T(I()));
      R.mat_kind[id] = MK_LIGHT;
    } else if (ty == "isotropic") {
      R.mat[id] = new isotropic(T(I()));
      R.mat_kind[id] = MK_ISO;
    } else {
      R.err = "unknown material";
      return false;
    }
  } else if (kw == "node") {
    int id = I();
    std::string ty;
    is >> ty;
    hitable *h = nullptr;
    if (ty == "sphere") {
      float x = F(), y = F(), z = F(), r = F();
      h = new sphere(vec3(x, y, z), r, copy_material(R, I(), id));
    } else if (ty == "moving_sphere") {
      float x0 = F(), y0 = F(), z0 = F(), x1 = F(), y1 = F(), z1 = F(), t0 = F(), t1 = F(), r = F();
      h = new moving_sphere(vec3(x0, y0, z0), vec3(x1, y1, z1), t0, t1, r, copy_material(R, I(), id));
    } else if (ty == "xy_rect" || ty == "xz_rect" || ty == "yz_rect") {
      float a0 = F(), a1 = F(), b0 = F(), b1 = F(), k = F();
      material *m = copy_material(R, I(), id);
      if (ty == "xy_rect") h = new xy_rect(a0, a1, b0, b1, k, m);
      else if (ty == "xz_rect") h = new xz_rect(a0, a1, b0, b1, k, m);
      else h = new yz_rect(a0, a1, b0, b1, k, m);
    } else if (ty == "flip_normal") {
      h = new flip_normal(N(I()));
    } else if (ty == "box") {
      float x0 = F(), y0 = F(), z0 = F(), x1 = F(), y1 = F(), z1 = F();
      h = new box(vec3(x0, y0, z0), vec3(x1, y1, z1), copy_material(R, I(), id));
    } else if (ty == "translate") {
      hitable *c = N(I());
      float x = F(), y = F(), z = F();
      h = new translate(c, vec3(x, y, z));
    } else if (ty == "rotate_y") {
      hitable *c = N(I());
      h = new rotate_y(c, F());
    } else if (ty == "constant_medium") {
      hitable *b = N(I());
      float d = F();
      auto *cm = new constant_medium(b, d, T(I()));
      R.prim_of_mat[cm->phase_funcion_] = id;
      h = cm;
    } else if (ty == "hitable_list") {
      int n = I();
      hitable **l = new hitable *[n > 0 ? n : 1];
      for (int i = 0; i < n; i++) l[i] = N(I());
      h = new hitable_list(l, n);
    } else if (ty == "bvh_node") {
      float t0 = F(), t1 = F();
      int n = I();
      hitable **l = new hitable *[n > 0 ? n : 1];
      for (int i = 0; i < n; i++) l[i] = N(I());
      h = new bvh_node(l, n, t0, t1);
      R.bvh_roots[h] = id;
    } else {
      R.err = "unknown node";
      return false;
    }
    R.node[id] = h;
    R.sd_of_node[h] = id;
  } else if (kw == "world") {
    R.world = N(I());
  } else if (kw == "lights") {
    R.lights = N(I());
  } else if (kw == "camera") {
    float v[15];
    for (float &x : v) x = F();
    R.cam = new camera(vec3(v[0], v[1], v[2]), vec3(v[3], v[4], v[5]), vec3(v[6], v[7], v[8]), v[9], v[10],
                       v[11], v[12], v[13], v[14]);
  } else {
    R.err = "unknown statement";
    return false;
  }
  return R.err.empty();
}

void install_perlin(const RefScene &R) {
  if (!R.has_perlin) return;
  for (int i = 0; i < 256; i++) {
    perlin_noise::random_vec3_[i] = R.pgrad[i];
    perlin_noise::permute_x_[i] = R.pperm[0][i];
    perlin_noise::permute_y_[i] = R.pperm[1][i];
    perlin_noise::permute_z_[i] = R.pperm[2][i];
  }
}

void dump(const RefScene &R, const bvh_node *n, std::vector<float> &boxes, std::vector<int> &kids) {
  int me = (int)kids.size() / 2;
  kids.push_back(0);
  kids.push_back(0);
  for (int i = 0; i < 3; i++) boxes.push_back(n->box_.min()[i]);
  for (int i = 0; i < 3; i++) boxes.push_back(n->box_.max()[i]);
  const hitable *ch[2] = {n->left_, n->right_};
  for (int c = 0; c < 2; c++) {
    auto *bn = dynamic_cast<const bvh_node *>(ch[c]);
    int ref;
    if (bn && !R.bvh_roots.count(ch[c])) {
      ref = (int)kids.size() / 2;
      dump(R, bn, boxes, kids);
    } else {
      auto it = R.sd_of_node.find(ch[c]);
      ref = -(1 + (it == R.sd_of_node.end() ? -2 : it->second));
    }
    kids[2 * me + c] = ref;
  }
}

}  // namespace

extern "C" {

typedef struct {
  int32_t width, height, spp, max_depth;
  int32_t lean;        // 1: skip the per-pixel unordered_map insert (main.cpp:144-148)
  int32_t burn_run;    // burn-in selector: each row discards burn_run*B1 + row*B2 draws
  int32_t burn_row;
  int32_t row_begin, row_end;  // image rows (0 = top) to render; end<=0: all
} ref_render_params;

void *ref_scene_load(const char *sd_text, char *err, int errlen) {
  auto *R = new RefScene();
  std::string text(sd_text ? sd_text : "");
  bool ok = true;
  int bad_line = 0;
  std::thread th([&]() {  // fresh thread: fresh drand_r stream for bvh_node
    std::istringstream in(text);
    std::string ln;
    int k = 0;
    while (std::getline(in, ln)) {
      k++;
      if (!parse_line(*R, ln)) {
        ok = false;
        bad_line = k;
        return;
      }
    }
  });
  th.join();
  if (ok && !R->world) {
    ok = false;
    R->err = "no world";
  }
  if (!ok) {
    if (err && errlen > 0) std::snprintf(err, errlen, "line %d: %s", bad_line, R->err.c_str());
    delete R;
    return nullptr;
  }
  install_perlin(*R);
  return R;
}

int32_t ref_bvh_dump(void *sp, int32_t sd_id, float *boxes, int32_t *kids, int32_t cap) {
  auto *R = static_cast<RefScene *>(sp);
  auto it = R->node.find(sd_id);
  if (it == R->node.end()) return -1;
  auto *bn = dynamic_cast<const bvh_node *>(it->second);
  if (!bn) return -1;
  std::vector<float> b;
  std::vector<int> k;
  // the root is always expanded, even though it is an SD-level node
  k.push_back(0);
  k.push_back(0);
  for (int i = 0; i < 3; i++) b.push_back(bn->box_.min()[i]);
  for (int i = 0; i < 3; i++) b.push_back(bn->box_.max()[i]);
  const hitable *ch[2] = {bn->left_, bn->right_};
  for (int c = 0; c < 2; c++) {
    auto *cb = dynamic_cast<const bvh_node *>(ch[c]);
    int ref;
    if (cb && !R->bvh_roots.count(ch[c])) {
      ref = (int)k.size() / 2;
      dump(*R, cb, b, k);
    } else {
      auto jt = R->sd_of_node.find(ch[c]);
      ref = -(1 + (jt == R->sd_of_node.end() ? -2 : jt->second));
    }
    k[c] = ref;
  }
  int n = (int)k.size() / 2;
  if (n > cap) return n;
  std::memcpy(boxes, b.data(), b.size() * sizeof(float));
  std::memcpy(kids, k.data(), k.size() * sizeof(int));
  return n;
}

// world->hit(r, 0.001, FLT_MAX, rec) for each ray, in order, on one fresh
// thread (constant_medium consumes that thread's drand_r stream).
int32_t ref_trace(void *sp, const float *rays, int64_t n, float *out_f, int32_t *out_i) {
  auto *R = static_cast<RefScene *>(sp);
  std::thread th([&]() {
    for (int64_t i = 0; i < n; i++) {
      const float *q = rays + 7 * i;
      ray r(vec3(q[0], q[1], q[2]), vec3(q[3], q[4], q[5]), q[6]);
      hit_record rec;
      bool h = R->world->hit(r, 0.001, std::numeric_limits<float>::max(), rec);
      float *o = out_f + 9 * i;
      if (h) {
        o[0] = rec.t; o[1] = rec.u; o[2] = rec.v;
        for (int k = 0; k < 3; k++) {
          o[3 + k] = rec.point[k];
          o[6 + k] = rec.normal[k];
        }
        auto it = R->prim_of_mat.find(rec.mat_ptr);
        out_i[2 * i] = 1;
        out_i[2 * i + 1] = it == R->prim_of_mat.end() ? -2 : it->second;
      } else {
        for (int k = 0; k < 9; k++) o[k] = 0.f;
        out_i[2 * i] = 0;
        out_i[2 * i + 1] = -1;
      }
    }
  });
  th.join();
  return 0;
}

// Replays main.cpp:109-175: one std::async task per image row, ns samples
// per pixel through camera::get_ray and color(), de_nan, running sum, mean.
// mean_rgb (row 0 = top) receives the mean before gamma.  Returns seconds.
double ref_render(void *sp, const ref_render_params *p, float *mean_rgb) {
  auto *R = static_cast<RefScene *>(sp);
  int nx = p->width, ny = p->height, ns = p->spp, depth = p->max_depth;
  int rb = p->row_begin < 0 ? 0 : p->row_begin;
  int re = p->row_end <= 0 || p->row_end > ny ? ny : p->row_end;
  camera cam = *R->cam;
  std::mutex mtx, mtx2;
  std::map<int, std::vector<int>> result;
  std::unordered_map<std::string, std::vector<vec3>> pixel_sample_cols;
  auto start = std::chrono::high_resolution_clock::now();
  auto row_task = [&](int index) {
    int row = ny - 1 - index;
    int64_t burn = (int64_t)p->burn_run * 400009 + (int64_t)index * (int64_t)p->burn_row;
    for (int64_t b = 0; b < burn; b++) drand_r();
    std::vector<int> row_colors;
    for (int i = 0; i < nx; i++) {
      std::vector<vec3> sample_cols;
      vec3 col(0.0, 0.0, 0.0);
      for (int k = 0; k < ns; k++) {
        float u = ((float)i + drand_r()) / (float)nx;
        float v = ((float)index + drand_r()) / (float)ny;
        ray r = cam.get_ray(u, v);
        col += de_nan(color(r, R->world, R->lights, 0, depth));
        if ((k + 1) % ns == 0) sample_cols.push_back(col);
      }
      col /= float(ns);
      float *o = mean_rgb + 3 * ((size_t)row * nx + i);
      o[0] = col[0]; o[1] = col[1]; o[2] = col[2];
      vec3 g(sqrt(col.r()), sqrt(col.g()), sqrt(col.b()));
      row_colors.push_back(int(255.99f * g.r()));
      row_colors.push_back(int(255.99f * g.g()));
      row_colors.push_back(int(255.99f * g.b()));
      if (!p->lean) {
        std::lock_guard<std::mutex> lock(mtx2);
        auto key = std::to_string(i) + "+" + std::to_string(index);
        pixel_sample_cols.insert({key, sample_cols});
      }
    }
    std::lock_guard<std::mutex> lock(mtx);
    result.insert({index, row_colors});
  };
  std::vector<std::future<void>> futures;
  for (int row = re - 1; row >= rb; row--) {
    int j = ny - 1 - row;
    futures.emplace_back(std::async(std::launch::deferred | std::launch::async, row_task, j));
  }
  for (auto &f : futures) f.wait();
  auto end = std::chrono::high_resolution_clock::now();
  return std::chrono::duration<double>(end - start).count();
}

int32_t ref_hardware_concurrency(void) { return (int32_t)std::thread::hardware_concurrency(); }

static void frontend_boxes(const bvh_node *bn, std::vector<float> &out) {
  for (int i = 0; i < 3; i++) out.push_back(bn->box_.min()[i]);
  for (int i = 0; i < 3; i++) out.push_back(bn->box_.max()[i]);
  const hitable *ch[2] = {bn->left_, bn->right_};
  for (int c = 0; c < 2; c++) {
    if (c == 1 && ch[1] == ch[0]) break;
    if (auto *cb = dynamic_cast<const bvh_node *>(ch[c])) frontend_boxes(cb, out);
  }
}

// The reference side of tests/frontend/random_bvh.cc: the same n spheres
// drawn with the reference's drand_r, then bvh_node, on a fresh thread
// (default drand_r stream); writes the pre-order node boxes (6 floats each)
// and returns the node count.
int32_t ref_frontend_bvh(int32_t n, float *boxes, int32_t cap) {
  std::vector<float> out;
  std::thread th([&]() {
    material *m = new lambertian(new constant_texture(vec3(0.5f, 0.5f, 0.5f)));
    std::vector<hitable *> list;
    for (int i = 0; i < n; i++) {
      const float x = (float)drand_r(-10, 10);
      const float z = (float)drand_r(-10, 10);
      const float r = (float)(0.1 + 0.3 * drand_r(0, 1));
      list.push_back(new sphere(vec3(x, r, z), r, m));
    }
    frontend_boxes(new bvh_node(list.data(), n, 0.0f, 1.0f), out);
  });
  th.join();
  const int nodes = (int)out.size() / 6;
  for (int i = 0; i < 6 * nodes && i < 6 * cap; i++) boxes[i] = out[i];
  return nodes;
}

}  // extern "C"

hitable *two_checker_spheres();  // defined in utils.cc without a declaration in utils.h

namespace {

// Pre-order dump of one bvh_node tree: per node its box and, per child, the
// child's pre-order index, or -1 for a leaf.
void dump_preorder(const bvh_node *n, std::vector<float> &boxes, std::vector<int> &kids) {
  const int me = (int)kids.size() / 2;
  kids.push_back(-1);
  kids.push_back(-1);
  for (int i = 0; i < 3; i++) boxes.push_back(n->box_.min()[i]);
  for (int i = 0; i < 3; i++) boxes.push_back(n->box_.max()[i]);
  const hitable *ch[2] = {n->left_, n->right_};
  for (int c = 0; c < 2; c++)
    if (auto *b = dynamic_cast<const bvh_node *>(ch[c])) {
      kids[2 * me + c] = (int)kids.size() / 2;
      dump_preorder(b, boxes, kids);
    }
}

// The bvh_nodes a scene function built itself (not their inner nodes), in
// the order it built them: a depth-first walk of lists and wrappers.
void find_bvh_roots(const hitable *h, std::vector<const bvh_node *> &out) {
  if (!h) return;
  if (auto *b = dynamic_cast<const bvh_node *>(h)) {
    out.push_back(b);
  } else if (auto *l = dynamic_cast<const hitable_list *>(h)) {
    for (int i = 0; i < l->list_size_; i++) find_bvh_roots(l->list_[i], out);
  } else if (auto *t = dynamic_cast<const translate *>(h)) {
    find_bvh_roots(t->ptr_, out);
  } else if (auto *r = dynamic_cast<const rotate_y *>(h)) {
    find_bvh_roots(r->ptr_, out);
  } else if (auto *f = dynamic_cast<const flip_normal *>(h)) {
    find_bvh_roots(f->ptr_, out);
  } else if (auto *m = dynamic_cast<const constant_medium *>(h)) {
    find_bvh_roots(m->boundary_, out);
  }
}

}  // namespace

extern "C" {

// Runs one of the reference's own scene functions (utils.cc:96-414) on a
// fresh thread (drand_r in its default state) and dumps the bvh_nodes it
// built, concatenated: boxes (6 floats per node), kids (2 per node, see
// dump_preorder), tree_nodes[k] = node count of tree k.  Returns the total
// node count (the arrays are filled when it is <= cap), *n_trees the trees;
// -1 for an unknown name.
int32_t ref_scene_function_bvhs(const char *name, float *boxes, int32_t *kids, int32_t *tree_nodes, int32_t cap,
                                int32_t *n_trees) {
  const std::string nm(name ? name : "");
  hitable *(*fn)() = nm == "random_scene"          ? random_scene
                     : nm == "two_checker_spheres" ? two_checker_spheres
                     : nm == "two_perlin_spheres"  ? two_perlin_spheres
                     : nm == "light_spheres"       ? light_spheres
                     : nm == "sphere_cornell_box"  ? sphere_cornell_box
                     : nm == "cornell_box"         ? cornell_box
                     : nm == "cornell_box_smoke"   ? cornell_box_smoke
                     : nm == "oneweek_final"       ? oneweek_final
                                                   : nullptr;
  if (!fn) return -1;
  std::vector<float> b;
  std::vector<int> k, sizes;
  std::thread th([&]() {
    std::vector<const bvh_node *> roots;
    find_bvh_roots(fn(), roots);
    for (const bvh_node *r : roots) {
      std::vector<float> tb;
      std::vector<int> tk;
      dump_preorder(r, tb, tk);
      sizes.push_back((int)tk.size() / 2);
      b.insert(b.end(), tb.begin(), tb.end());
      k.insert(k.end(), tk.begin(), tk.end());
    }
  });
  th.join();
  const int n = (int)k.size() / 2;
  *n_trees = (int32_t)sizes.size();
  if (n <= cap) {
    std::memcpy(boxes, b.data(), b.size() * sizeof(float));
    std::memcpy(kids, k.data(), k.size() * sizeof(int));
    std::memcpy(tree_nodes, sizes.data(), sizes.size() * sizeof(int));
  }
  return n;
}

// config.ini through the reference's own parser and the extraction calls of
// main.cpp:42-56, from main.cpp:31-40's defaults.  out: width, height,
// sample, recur_depth, fov, allow_bonus_pic, bonus_pic, aperture,
// start_time, end_time.
void ref_config_parse(const char *text, double out[10]) {
  int nx = 400, ny = 200, ns = 10, depth = 50, allow = 0, bonus = 10;
  float aperture = 0.2f, time0 = 0.0f, time1 = 1.0f, fov = 90.0f;
  std::istringstream is{std::string(text)};
  inipp::Ini<char> ini;
  ini.parse(is);
  inipp::extract(ini.sections["DEFAULT"]["width"], nx);
  inipp::extract(ini.sections["DEFAULT"]["height"], ny);
  inipp::extract(ini.sections["DEFAULT"]["sample"], ns);
  inipp::extract(ini.sections["DEFAULT"]["recur_depth"], depth);
  inipp::extract(ini.sections["DEFAULT"]["fov"], fov);
  inipp::extract(ini.sections["DEFAULT"]["bonus_pic"], bonus);
  inipp::extract(ini.sections["DEFAULT"]["allow_bonus_pic"], allow);
  inipp::extract(ini.sections["BLUR"]["aperture"], aperture);
  inipp::extract(ini.sections["CAM_MOTION"]["start_time"], time0);
  inipp::extract(ini.sections["CAM_MOTION"]["end_time"], time1);
  const double v[10] = {(double)nx, (double)ny, (double)ns, (double)depth, fov, (double)allow, (double)bonus,
                        aperture, time0, time1};
  for (int i = 0; i < 10; i++) out[i] = v[i];
}

}  // extern "C"
