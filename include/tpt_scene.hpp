/* tpt_scene.hpp - C++ scene front end with the reference's class names and
 * constructor signatures (headers/texture.h, material.h, sphere.h,
 * rect_box.h, hitable.h, hitable_list.h, camera.h), so that scene-building
 * code written against the reference compiles unchanged against this header
 * and produces a tpt_scene for the GPU path.
 *
 * Every object records itself in a per-thread tpt_builder as it is
 * constructed; tpt::compile_scene() flattens the graph and starts a fresh
 * builder.  drand_r() draws from that builder's stream, which bvh_node also
 * uses, so a scene whose layout is drawn with drand_r gets the reference's
 * BVH topology bit for bit (the reference shares one thread-local mt19937
 * between scene code and bvh_node, utils.cc:28-32, hitable.cc:33).
 *
 * The objects are handles: they hold no geometry and cannot be hit-tested on
 * the host (tpt_trace_closest does that on the GPU).  Like the reference,
 * objects are created with `new` and never freed; they are a few bytes each.
 * Header-only, C++14; link libtpt.so.  (No counterpart in the reference: it
 * is the reference's own interface, rebound.) */
#ifndef TPT_SCENE_HPP
#define TPT_SCENE_HPP

#include <algorithm>
#include <cmath>
#include <iostream>
#include <stdexcept>
#include <string>
#include <vector>

#include "tpt.h"

namespace tpt {

// The builder that objects of this thread record into.
inline tpt_builder *&current_builder() {
  static thread_local tpt_builder *b = nullptr;
  if (!b && tpt_builder_create(&b) != TPT_OK) throw std::runtime_error("tpt_builder_create failed");
  return b;
}

// A negative handle is a negated tpt_status.
inline int32_t checked(int32_t h, const char *what) {
  if (h < 0) throw std::runtime_error(std::string(what) + ": " + tpt_status_string((tpt_status)-h));
  return h;
}

// vec3 (headers/vec3.h:6-157): three floats with the reference's
// interface, so scene code that computes positions, offsets and colours
// (utils.cc:96-414) compiles and gets the same floats.  Every operation is
// evaluated in float, component by component, in the reference's order
// (length: sqrt((x*x + y*y) + z*z); make_unit_vector scales by 1.0 / length
// rounded from double to float); the scene layout, and with it the BVH that
// bvh_node builds, depends on those bits.
struct vec3 {
  float e[3];
  vec3() : e{0, 0, 0} {}
  vec3(float x, float y, float z) : e{x, y, z} {}
  vec3(float s) : e{s, s, s} {}  // NOLINT: implicit, as the reference's
  float x() const { return e[0]; }
  float y() const { return e[1]; }
  float z() const { return e[2]; }
  float r() const { return e[0]; }
  float g() const { return e[1]; }
  float b() const { return e[2]; }
  float operator[](int i) const { return e[i]; }
  float &operator[](int i) { return e[i]; }
  const vec3 &operator+() const { return *this; }
  vec3 operator-() const { return vec3(-e[0], -e[1], -e[2]); }
  vec3 &operator+=(const vec3 &o) { return each(o, [](float &a, float b) { a += b; }); }
  vec3 &operator-=(const vec3 &o) { return each(o, [](float &a, float b) { a -= b; }); }
  vec3 &operator*=(const vec3 &o) { return each(o, [](float &a, float b) { a *= b; }); }
  vec3 &operator/=(const vec3 &o) { return each(o, [](float &a, float b) { a /= b; }); }
  vec3 &operator*=(const float t) { return each(vec3(t), [](float &a, float b) { a *= b; }); }
  vec3 &operator/=(const float t) { return each(vec3(t), [](float &a, float b) { a /= b; }); }
  float squared_length() const { return e[0] * e[0] + e[1] * e[1] + e[2] * e[2]; }
  float length() const { return std::sqrt(squared_length()); }
  void make_unit_vector() { *this *= (float)(1.0 / length()); }
  void normalize() { make_unit_vector(); }

 private:
  template <class F>
  vec3 &each(const vec3 &o, F f) {
    for (int i = 0; i < 3; i++) f(e[i], o.e[i]);
    return *this;
  }
};

inline vec3 operator+(vec3 a, const vec3 &b) { return a += b; }
inline vec3 operator-(vec3 a, const vec3 &b) { return a -= b; }
inline vec3 operator*(vec3 a, const vec3 &b) { return a *= b; }
inline vec3 operator/(vec3 a, const vec3 &b) { return a /= b; }
inline vec3 operator*(vec3 a, float t) { return a *= t; }
inline vec3 operator*(float t, vec3 a) { return a *= t; }
inline vec3 operator/(vec3 a, float t) { return a /= t; }
inline float dot(const vec3 &a, const vec3 &b) { return a.e[0] * b.e[0] + a.e[1] * b.e[1] + a.e[2] * b.e[2]; }
inline vec3 cross(const vec3 &a, const vec3 &b) {
  return vec3(a.e[1] * b.e[2] - b.e[1] * a.e[2], a.e[2] * b.e[0] - b.e[2] * a.e[0], a.e[0] * b.e[1] - b.e[0] * a.e[1]);
}
inline vec3 normalize(vec3 v) { return v / v.length(); }
inline vec3 unit_vector(vec3 v) { return normalize(v); }
inline vec3 vec_min(const vec3 &a, const vec3 &b) {
  return vec3(std::min(a.e[0], b.e[0]), std::min(a.e[1], b.e[1]), std::min(a.e[2], b.e[2]));
}
inline vec3 vec_max(const vec3 &a, const vec3 &b) {
  return vec3(std::max(a.e[0], b.e[0]), std::max(a.e[1], b.e[1]), std::max(a.e[2], b.e[2]));
}
inline std::istream &operator>>(std::istream &is, vec3 &v) { return is >> v.e[0] >> v.e[1] >> v.e[2]; }
inline std::ostream &operator<<(std::ostream &os, const vec3 &v) {
  return os << v.e[0] << " " << v.e[1] << " " << v.e[2];
}

// ---- textures (headers/texture.h)
class texture {
 public:
  int32_t handle = -1;
  virtual ~texture() {}
};
class constant_texture : public texture {
 public:
  constant_texture(vec3 c) {
    handle = checked(tpt_constant_texture(current_builder(), c[0], c[1], c[2]), "constant_texture");
  }
};
class checker_texture : public texture {
 public:
  checker_texture(texture *t0, texture *t1) {
    handle = checked(tpt_checker_texture(current_builder(), t0->handle, t1->handle), "checker_texture");
  }
};
class perlin_noise_texture : public texture {
 public:
  perlin_noise_texture(float scale = 1.0) {
    handle = checked(tpt_perlin_noise_texture(current_builder(), scale), "perlin_noise_texture");
  }
};
class image_texture : public texture {
 public:
  image_texture(unsigned char *pixels, int width, int height) {
    handle = checked(tpt_image_texture(current_builder(), pixels, width, height), "image_texture");
  }
};

// ---- materials (headers/material.h)
class material {
 public:
  int32_t handle = -1;
  virtual ~material() {}
};
class lambertian : public material {
 public:
  lambertian(texture *albedo) { handle = checked(tpt_lambertian(current_builder(), albedo->handle), "lambertian"); }
};
class metal : public material {
 public:
  metal(const vec3 &albedo, float fuzz) {
    handle = checked(tpt_metal(current_builder(), albedo[0], albedo[1], albedo[2], fuzz), "metal");
  }
};
class dielectric : public material {
 public:
  dielectric(float ri) { handle = checked(tpt_dielectric(current_builder(), ri), "dielectric"); }
};
class diffuse_light : public material {
 public:
  diffuse_light(texture *a) { handle = checked(tpt_diffuse_light(current_builder(), a->handle), "diffuse_light"); }
};
class isotropic : public material {
 public:
  isotropic(texture *t) { handle = checked(tpt_isotropic(current_builder(), t->handle), "isotropic"); }
};

// ---- hitables (headers/sphere.h, rect_box.h, hitable.h, hitable_list.h)
class hitable {
 public:
  int32_t handle = -1;
  virtual ~hitable() {}
};
class sphere : public hitable {
 public:
  sphere(vec3 center, float radius, material *m) {
    handle = checked(tpt_sphere(current_builder(), center[0], center[1], center[2], radius, m->handle), "sphere");
  }
};
class moving_sphere : public hitable {
 public:
  moving_sphere(vec3 center0, vec3 center1, float t0, float t1, float radius, material *m) {
    handle = checked(tpt_moving_sphere(current_builder(), center0[0], center0[1], center0[2], center1[0], center1[1],
                                       center1[2], t0, t1, radius, m->handle),
                     "moving_sphere");
  }
};
class xy_rect : public hitable {
 public:
  xy_rect(float x0, float x1, float y0, float y1, float k, material *mat) {
    handle = checked(tpt_xy_rect(current_builder(), x0, x1, y0, y1, k, mat->handle), "xy_rect");
  }
};
class xz_rect : public hitable {
 public:
  xz_rect(float x0, float x1, float z0, float z1, float k, material *mat) {
    handle = checked(tpt_xz_rect(current_builder(), x0, x1, z0, z1, k, mat->handle), "xz_rect");
  }
};
class yz_rect : public hitable {
 public:
  yz_rect(float y0, float y1, float z0, float z1, float k, material *mat) {
    handle = checked(tpt_yz_rect(current_builder(), y0, y1, z0, z1, k, mat->handle), "yz_rect");
  }
};
class flip_normal : public hitable {
 public:
  flip_normal(hitable *p) { handle = checked(tpt_flip_normal(current_builder(), p->handle), "flip_normal"); }
};
class box : public hitable {
 public:
  box(vec3 pmin, vec3 pmax, material *mat) {
    handle = checked(tpt_box(current_builder(), pmin[0], pmin[1], pmin[2], pmax[0], pmax[1], pmax[2], mat->handle),
                     "box");
  }
};
class translate : public hitable {
 public:
  translate(hitable *p, const vec3 &offset) {
    handle = checked(tpt_translate(current_builder(), p->handle, offset[0], offset[1], offset[2]), "translate");
  }
};
class rotate_y : public hitable {
 public:
  rotate_y(hitable *p, float angle) {
    handle = checked(tpt_rotate_y(current_builder(), p->handle, angle), "rotate_y");
  }
};
class constant_medium : public hitable {
 public:
  constant_medium(hitable *boundary, float density, texture *t) {
    handle = checked(tpt_constant_medium(current_builder(), boundary->handle, density, t->handle),
                     "constant_medium");
  }
};
class hitable_list : public hitable {
 public:
  hitable_list(hitable **l, int n) {
    std::vector<int32_t> h(n > 0 ? n : 0);
    for (int i = 0; i < n; i++) h[i] = l[i]->handle;
    handle = checked(tpt_hitable_list(current_builder(), h.data(), n), "hitable_list");
  }
};
class bvh_node : public hitable {
 public:
  bvh_node(hitable **l, int n, float time0, float time1) {
    std::vector<int32_t> h(n > 0 ? n : 0);
    for (int i = 0; i < n; i++) h[i] = l[i]->handle;
    handle = checked(tpt_bvh_node(current_builder(), h.data(), n, time0, time1), "bvh_node");
  }
};

// ---- camera (headers/camera.h)
class camera_with_blur {
 public:
  vec3 lookfrom, lookat, vup;
  float vfov, aspect, aperture, focus_dist, t0, t1;
  camera_with_blur(vec3 lookfrom_, vec3 lookat_, vec3 vup_, float vfov_, float aspect_, float aperture_,
                   float focus_dist_, float t0_, float t1_)
      : lookfrom(lookfrom_), lookat(lookat_), vup(vup_), vfov(vfov_), aspect(aspect_), aperture(aperture_),
        focus_dist(focus_dist_), t0(t0_), t1(t1_) {}
};

using camera = camera_with_blur;  // camera.h:23

// drand_r (utils.cc:28-32) on the current builder's stream.
inline double drand_r(double min = 0.0, double max = 1.0) { return tpt_builder_drand(current_builder(), min, max); }

// Flattens the current builder's graph with `world`, the light_shape of
// color() (nullptr: none) and the camera into a compiled scene; the thread
// starts a fresh builder (and drand_r stream) for its next scene.
inline tpt_scene *compile_scene(hitable *world, hitable *light_shape, const camera_with_blur &cam,
                                int32_t bvh_build = TPT_BVH_REFERENCE) {
  tpt_builder *b = current_builder();
  if (tpt_builder_set_world(b, world->handle) != TPT_OK ||
      tpt_builder_set_light_shape(b, light_shape ? light_shape->handle : -1) != TPT_OK ||
      tpt_builder_set_bvh_build(b, bvh_build) != TPT_OK)
    throw std::runtime_error("compile_scene: bad world or light_shape");
  tpt_builder_set_camera(b, cam.lookfrom.e, cam.lookat.e, cam.vup.e, cam.vfov, cam.aspect, cam.aperture,
                         cam.focus_dist, cam.t0, cam.t1);
  tpt_scene *s = nullptr;
  const tpt_status st = tpt_scene_compile(b, &s);
  tpt_builder_destroy(b);
  current_builder() = nullptr;  // the next object starts a new builder
  if (st != TPT_OK) throw std::runtime_error(std::string("tpt_scene_compile: ") + tpt_status_string(st));
  return s;
}

}  // namespace tpt

#endif
