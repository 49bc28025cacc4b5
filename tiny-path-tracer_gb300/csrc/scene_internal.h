// scene_internal.h - host-side compiled scene (the arena before upload).
#ifndef TPT_SCENE_INTERNAL_H
#define TPT_SCENE_INTERNAL_H
#include <stddef.h>
#include <stdint.h>

#include <vector>

#include "../../include/tpt.h"
#include "arena.h"

namespace tpt {

struct HostScene {
  std::vector<f4> node_lo, node_hi;
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
  Camera cam{};
};

// Sections of the device arena, each 256-byte aligned.
struct ArenaLayout {
  size_t off[15];
  size_t total;
};

inline size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

inline ArenaLayout arena_layout(const HostScene &S) {
  size_t sizes[15] = {
      S.node_lo.size() * sizeof(f4),     S.node_hi.size() * sizeof(f4),   S.leaf_hdr.size() * sizeof(i4),
      S.leaf_user.size() * sizeof(int32_t), S.leaf_data.size() * sizeof(f4), S.items.size() * sizeof(i2),
      S.mat_i.size() * sizeof(i4),       S.mat_f.size() * sizeof(f4),     S.tex_i.size() * sizeof(i4),
      S.tex_f.size() * sizeof(f4),       S.images.size(),                 S.perlin_grad.size() * sizeof(f4),
      S.perlin_perm.size() * sizeof(int32_t), S.light_i.size() * sizeof(i4), S.light_f.size() * sizeof(f4)};
  ArenaLayout L;
  size_t at = 0;
  for (int i = 0; i < 15; i++) {
    L.off[i] = at;
    at += align256(sizes[i] ? sizes[i] : 16);
  }
  L.total = at;
  return L;
}

inline size_t arena_bytes(const HostScene &S) { return arena_layout(S).total; }

const HostScene *host_scene(const tpt_scene *s);

}  // namespace tpt
#endif
