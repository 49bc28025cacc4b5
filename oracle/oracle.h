/*
 * oracle.h - C API of the CPU oracle for the tiny-path-tracer hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is a plain C++ restatement of the
 * reference's algorithm (BlurryLight/tiny-path-tracer, its src/ and
 * headers/ directories); every function in oracle.cc cites the reference file:line it
 * follows.  It exists to check the CUDA product: only tests/, the smoke()
 * entry point and bench.py's cpu_baseline / reference legs may load it.  The
 * product library never links, loads or calls it.
 *
 * Parity pinning: the reference ships no tests and no golden vectors.  The
 * oracle is pinned against outputs of the reference itself, compiled from its
 * unmodified sources by oracle/Makefile into oracle/_ref/ (see ref_harness.cc)
 * and frozen as fixtures under tests/golden/ by tests/golden/gen_golden.py.
 *
 * Scene description ("SD") text format, shared by the oracle, the reference
 * harness and the product's loader.  One statement per line, '#' comments.
 * Ids are small non-negative integers, unique per kind, defined before use.
 *
 *   tex ID const R G B
 *   tex ID checker ODD_TEX EVEN_TEX
 *   tex ID perlin SCALE                    (uses the scene's perlin tables)
 *   tex ID image W H SEED                  (procedural RGB8 image, see
 *                                           oracle_procedural_image)
 *   perlin_tables G0x G0y G0z ... G255z P0x..P255x P0y..P255y P0z..P255z
 *   mat ID lambertian TEX
 *   mat ID metal R G B FUZZ
 *   mat ID dielectric IOR
 *   mat ID diffuse_light TEX
 *   mat ID isotropic TEX
 *   node ID sphere CX CY CZ R MAT
 *   node ID moving_sphere C0X C0Y C0Z C1X C1Y C1Z T0 T1 R MAT
 *   node ID xy_rect X0 X1 Y0 Y1 K MAT      (likewise xz_rect, yz_rect)
 *   node ID flip_normal CHILD
 *   node ID box X0 Y0 Z0 X1 Y1 Z1 MAT
 *   node ID translate CHILD OX OY OZ
 *   node ID rotate_y CHILD ANGLE_DEGREES
 *   node ID constant_medium BOUNDARY DENSITY TEX
 *   node ID hitable_list N CHILD...
 *   node ID bvh_node T0 T1 N CHILD...      (built when the line is read,
 *                                           consuming the scene's drand_r)
 *   world NODE
 *   lights NODE                            (the light_shape of color())
 *   camera FX FY FZ AX AY AZ UX UY UZ VFOV ASPECT APERTURE FOCUS T0 T1
 *
 * Each scene load starts the drand_r stream (std::mt19937, default seed)
 * afresh, so BVH topology depends only on the text.
 */
#ifndef TPT_ORACLE_H
#define TPT_ORACLE_H
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

typedef struct oracle_scene oracle_scene;

typedef struct {
  int32_t width, height, spp, max_depth;
  int32_t semantics;     /* 0 = reference quirks, 1 = physical */
  int32_t background;    /* 0 = black, 1 = sky gradient */
  float sky_scale;
  int32_t nthreads;      /* worker threads (rows are distributed) */
  uint64_t seed;
  int32_t row_begin, row_end; /* image rows (0 = top) to render; end<=0: all */
} oracle_render_params;

typedef struct {
  int64_t segments;      /* rays traced by color() */
  int64_t aabb_tests, sphere_tests, rect_tests, instance_xforms, medium_tests;
  int64_t lambertian, metal, dielectric, light_pdf_evals;
} oracle_counters;

/* Scene */
oracle_scene *oracle_scene_load(const char *sd_text, char *err, int errlen);
void oracle_scene_free(oracle_scene *s);
/* out[0..7] = n_nodes, n_leaves, n_bvh_internal, n_mats, n_texs, world, lights, has_camera */
void oracle_scene_info(const oracle_scene *s, int32_t *out);
/* Pre-order dump of the BVH built for SD node `sd_id` (a bvh_node line).
 * Per internal node: box (6 floats) into boxes, and (left, right) into kids,
 * where a child >= 0 is the pre-order index of an internal node and a child
 * < 0 is -(1 + SD id of the leaf).  Returns the node count, or -1. */
int32_t oracle_bvh_dump(const oracle_scene *s, int32_t sd_id, float *boxes,
                        int32_t *kids, int32_t cap);
/* World bounding box (6 floats); returns 0 if the world has none. */
int32_t oracle_world_box(const oracle_scene *s, float *box6);

/* Closest hit of world->hit(r, 0.001, FLT_MAX) for n rays given as
 * (ox,oy,oz,dx,dy,dz,time).  out_f: (t,u,v,px,py,pz,nx,ny,nz) per ray,
 * out_i: (hit, prim SD id) per ray.  media_mode 0: the free-flight uniform of
 * a constant_medium is philox(seed, ray index, medium SD id); media_mode 1:
 * a single std::mt19937 stream consumed in the reference's order. */
int32_t oracle_trace(const oracle_scene *s, const float *rays, int64_t n,
                     uint64_t seed, int32_t media_mode, float *out_f,
                     int32_t *out_i, int32_t nthreads, oracle_counters *cnt);

/* Deterministic seeded ray batch: a fraction `frac_camera` are camera rays
 * of the scene's camera, the rest have origins uniform in the world box and
 * uniform directions of random length; `frac_axis` of the random rays have
 * one or two direction components set to exactly zero. */
void oracle_make_rays(const oracle_scene *s, int64_t n, uint64_t seed,
                      float frac_camera, float frac_axis, float *rays);

/* Path-traced render.  mean_rgb: width*height*3 floats, row 0 = top image
 * row, holding the per-pixel mean of de_nan(color()).  Returns 0 on success. */
int32_t oracle_render(const oracle_scene *s, const oracle_render_params *p,
                      float *mean_rgb, oracle_counters *cnt);

/* Reference output quantisation (main.cpp:135-142,176-182): gamma 2,
 * int(255.99*c), clamp to [0,255]. */
void oracle_quantize(const float *mean_rgb, int64_t n_pixels, uint8_t *rgb8);

/* Linear BVH over n boxes (6 floats each: min xyz, max xyz), the CPU
 * restatement of the GPU builder of TPT_BVH_LBVH (lbvh.cc).  keys: the
 * n unsorted 64-bit keys (Morton code of the centroid, then the index);
 * returns the Morton bits per axis. */
int32_t oracle_lbvh_keys(const float *boxes, int32_t n, uint64_t *keys);
/* The tree: max(n - 1, 1) internal nodes in pre-order; per node its box
 * (6 floats), children (>= 0: node, < 0: ~box index) and the pre-order index
 * just past its subtree; *out_depth = levels of internal nodes.  Returns the
 * node count, or -1 for n < 1. */
int32_t oracle_lbvh_build(const float *boxes, int32_t n, float *out_boxes, int32_t *out_kids,
                          int32_t *out_skip, int32_t *out_depth);

/* Philox-4x32-10 block (Salmon et al., SC'11). */
void oracle_philox(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);

/* Procedural RGB8 image texture, deterministic integer arithmetic only. */
void oracle_procedural_image(int32_t w, int32_t h, uint32_t seed, uint8_t *rgb);

#ifdef __cplusplus
}
#endif
#endif
