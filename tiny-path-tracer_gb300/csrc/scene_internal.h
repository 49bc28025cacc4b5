// scene_internal.h - host-side compiled scene (the arena before upload).
#ifndef TPT_SCENE_INTERNAL_H
#define TPT_SCENE_INTERNAL_H
#include <stddef.h>
#include <stdint.h>

#include <vector>

#include "../../include/tpt.h"
#include "arena.h"
#include "lbvh.h"

namespace tpt {

struct HostScene {
  std::vector<f4> node_lo, node_hi;
  std::vector<int32_t> node_skip;  // pre-order index just past each node's subtree
  std::vector<f4> node_kids;       // per node: {left lo, ref}, {left hi, ext}, {right lo, ref}, {right hi, ext};
                                   // a sphere leaf child: {center, ref}, {radius, 1, 0, 0}
  std::vector<i4> leaf_hdr;
  std::vector<int32_t> leaf_user;
  std::vector<f4> leaf_data;
  std::vector<i2> items;
  std::vector<i4> mat_i;
  std::vector<f4> mat_f;
  std::vector<i4> tex_i;
  std::vector<f4> tex_f;
  std::vector<uint8_t> images;
  std::vector<f4> perlin_grad;
  std::vector<int32_t> perlin_perm;
  std::vector<i4> light_i;
  std::vector<f4> light_f;
  int32_t light_is_list = 0, has_lights = 0;
  int32_t n_blas = 0, blas_depth = 0, max_stack = 0;
  float world_lo[3] = {0, 0, 0}, world_hi[3] = {0, 0, 0};  // world bounding box (0 if none)
  Camera cam{};
  float cam_in[15] = {};  // the camera's inputs: lookfrom, lookat, vup, vfov, aspect, aperture, focus, t0, t1
  // TPT_BVH_LBVH: one device build job per bvh_node (lbvh.h); its node slots
  // stay zero on the host and are filled after upload
  std::vector<i4> lbvh_jobs;
  std::vector<f4> lbvh_prims;
  std::vector<uint8_t> lbvh_blas;  // per job: 1 if the BVH is instanced
  int64_t lbvh_keys = 0;
  int32_t lbvh_max_pad = 0;
};

// Sections of the device arena, each 256-byte aligned, in DevScene order,
// then the LBVH build inputs and scratch (a section with null data is
// reserved, not copied).
enum { ARENA_SECTIONS = 20, ARENA_LBVH_JOBS = 17, ARENA_LBVH_PRIMS = 18, ARENA_LBVH_WORK = 19 };
struct ArenaSection {
  const void *data;
  size_t bytes;
};
inline void arena_sections(const HostScene &S, ArenaSection out[ARENA_SECTIONS]) {
  const ArenaSection t[ARENA_SECTIONS] = {
      {S.node_lo.data(), S.node_lo.size() * sizeof(f4)},
      {S.node_hi.data(), S.node_hi.size() * sizeof(f4)},
      {S.node_skip.data(), S.node_skip.size() * sizeof(int32_t)},
      {S.leaf_hdr.data(), S.leaf_hdr.size() * sizeof(i4)},
      {S.leaf_user.data(), S.leaf_user.size() * sizeof(int32_t)},
      {S.leaf_data.data(), S.leaf_data.size() * sizeof(f4)},
      {S.items.data(), S.items.size() * sizeof(i2)},
      {S.mat_i.data(), S.mat_i.size() * sizeof(i4)},
      {S.mat_f.data(), S.mat_f.size() * sizeof(f4)},
      {S.tex_i.data(), S.tex_i.size() * sizeof(i4)},
      {S.tex_f.data(), S.tex_f.size() * sizeof(f4)},
      {S.images.data(), S.images.size()},
      {S.perlin_grad.data(), S.perlin_grad.size() * sizeof(f4)},
      {S.perlin_perm.data(), S.perlin_perm.size() * sizeof(int32_t)},
      {S.light_i.data(), S.light_i.size() * sizeof(i4)},
      {S.light_f.data(), S.light_f.size() * sizeof(f4)},
      {S.node_kids.data(), S.node_kids.size() * sizeof(f4)},
      {S.lbvh_jobs.data(), S.lbvh_jobs.size() * sizeof(i4)},
      {S.lbvh_prims.data(), S.lbvh_prims.size() * sizeof(f4)},
      {nullptr, S.lbvh_jobs.empty() ? 0
                                    : lbvh_work_bytes((int64_t)S.lbvh_prims.size() / 2, (int32_t)S.lbvh_jobs.size(),
                                                      S.lbvh_keys)}};
  for (int i = 0; i < ARENA_SECTIONS; i++) out[i] = t[i];
}

struct ArenaLayout {
  size_t off[ARENA_SECTIONS];
  size_t total;
};

inline size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

inline ArenaLayout arena_layout(const HostScene &S) {
  ArenaSection sec[ARENA_SECTIONS];
  arena_sections(S, sec);
  ArenaLayout L;
  size_t at = 0;
  for (int i = 0; i < ARENA_SECTIONS; i++) {
    L.off[i] = at;
    at += align256(sec[i].bytes ? sec[i].bytes : 16);
  }
  L.total = at;
  return L;
}

inline size_t arena_bytes(const HostScene &S) { return arena_layout(S).total; }

const HostScene *host_scene(const tpt_scene *s);

}  // namespace tpt
#endif
