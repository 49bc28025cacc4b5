// arena.h - device layout of a compiled scene, shared by the host compiler
// (scene.cc) and the CUDA kernels.  Plain-old-data only.
//
// HBM layout (one contiguous allocation per uploaded scene, 256-byte aligned
// sections):
//   node_skip[n]             pre-order index just past the node's subtree
//                            (stackless walk: on a box miss jump there)
//   node_lo[n], node_hi[n]   BVH2 nodes as two SoA float4 arrays:
//                            {min.x,min.y,min.z,left}, {max.x,max.y,max.z,right}
//                            (children stored as int bits; >= 0 internal node,
//                            < 0 leaf ~index).  Every BVH of the scene (top
//                            level and instanced) lives in the same array,
//                            flattened in pre-order, so a parent and its
//                            left child are adjacent.
//   leaf_hdr[m]              int4 {type | flip<<4 | axis<<5, data offset,
//                            material, aux}; leaves of one BVH are numbered in
//                            left-to-right order, which is the reference's tie
//                            order (ties go right, hitable.cc:71).
//   leaf_user[m]             user id (builder handle / SD id) of the leaf
//   leaf_data[]              float4 pool of primitive parameters
//   items[k]                 top-level list: int2 {kind, ref}; a world that
//                            is a hitable_list is evaluated item by item with
//                            the list's shrinking t_max (hitable_list.cc:38-51)
//   mat_i/mat_f, tex_i/tex_f material and texture tables
//   images                   RGB8 texels of all image textures
//   perlin_grad[256], perlin_perm[768]
//   light_i/light_f          flattened light_shape items with pick weights
#ifndef TPT_ARENA_H
#define TPT_ARENA_H
#include <stdint.h>

namespace tpt {

struct f4 { float x, y, z, w; };
struct i4 { int32_t x, y, z, w; };
struct i2 { int32_t x, y; };

enum LeafType : int32_t {
  LT_SPHERE = 1,    // data[0] = {c.xyz, r}
  LT_MSPHERE = 2,   // data[0] = {c0.xyz, r}, data[1] = {c1.xyz, t0}, data[2] = {t1,0,0,0}
  LT_RECT = 3,      // axis = plane axis; data[0] = {a0,a1,b0,b1}, data[1] = {k,0,0,0}
  LT_BOX = 4,       // data[0] = {pmin.xyz,0}, data[1] = {pmax.xyz,0}
  LT_INSTANCE = 5,  // data[0] = {n_ops,0,0,0}; data[1..n] = {op, a, b, c}; aux = child ref
  LT_MEDIUM = 6     // data[0] = {density,0,0,0}; aux = boundary leaf; mat = phase material
};
enum { LEAF_TYPE_MASK = 15, LEAF_FLIP = 16, LEAF_AXIS_SHIFT = 5 };
enum { OP_TRANSLATE = 0, OP_ROTATE_Y = 1 };  // op a,b,c: offset | sin, cos
enum { MAX_INSTANCE_OPS = 4 };

enum ItemKind : int32_t { ITEM_BVH = 0, ITEM_LEAF = 1 };

enum MatType : int32_t { MT_LAMBERTIAN = 1, MT_METAL = 2, MT_DIELECTRIC = 3, MT_LIGHT = 4, MT_ISOTROPIC = 5 };
// mat_i = {type, tex, 0, reads_uv (1 if the texture tree holds an image)}; mat_f = {albedo.xyz, fuzz} (metal) | {ior,0,0,0}

enum TexType : int32_t { TT_CONST = 1, TT_CHECKER = 2, TT_PERLIN = 3, TT_IMAGE = 4 };
// tex_i = {type, a, b, c}: checker {odd, even}; image {w, h, byte offset}
// tex_f = {r,g,b,0} (const) | {scale,0,0,0} (perlin)

enum LightType : int32_t { LS_NONE = 0, LS_XZ_RECT = 1, LS_SPHERE = 2 };
// light_i = {type, 0, 0, 0}; light_f[2*i] = {a0,a1,b0,b1} | {c.xyz, r};
// light_f[2*i+1] = {k, weight, cdf, 0}

struct Camera {  // camera.cc:2-21, precomputed on the host
  float origin[3], lower_left[3], horizontal[3], vertical[3], u[3], v[3];
  float lens_radius, t0, t1;
};

// Traversal stack depth (entries per thread in shared memory).
enum { TRAVERSAL_STACK = 32 };

struct DevScene {
  const f4 *node_lo;
  const f4 *node_hi;
  const int32_t *node_skip;
  const i4 *leaf_hdr;
  const int32_t *leaf_user;
  const f4 *leaf_data;
  const i2 *items;
  const i4 *mat_i;
  const f4 *mat_f;
  const i4 *tex_i;
  const f4 *tex_f;
  const uint8_t *images;
  const f4 *perlin_grad;
  const int32_t *perlin_perm;
  const i4 *light_i;
  const f4 *light_f;
  const f4 *node_kids;  // 4 per node: both children's boxes, refs in lo.w; a sphere leaf child
                        // carries {center, ref}, {radius, 1, 0, 0}
  int32_t n_nodes, n_leaves, n_items, n_mats, n_texs, n_lights;
  int32_t light_is_list;  // 0: single light_shape hitable; 1: hitable_list
  int32_t has_lights;
  int32_t flat_max;  // BVH items of at most this many nodes use the stackless walk
  int32_t feat;      // FEAT_* (device.cuh): the leaf kinds present, for kernel specialisation
  Camera cam;
};

// float4 per entry of the path-guiding lobe table: 8 lobes + 2 of weight sums.
enum { GUIDE_ENTRY = 10 };

// Default size limit of the stackless pre-order walk (tuned per render).
enum { DEFAULT_FLAT_MAX = 48 };

}  // namespace tpt
#endif
