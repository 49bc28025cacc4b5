/*
 * tpt.h - C ABI of the GB300 (sm_103a) path tracer: the drop-in boundary for
 * the hot path of BlurryLight/tiny-path-tracer (camera rays -> BVH closest
 * hit -> material scatter -> mixture-pdf light sampling -> per-pixel
 * accumulation).
 *
 * The reference exposes no FFI: its boundary is the C++ virtual object model
 * (hitable / material / texture / camera, the free function color()) and the
 * config.ini keys.  This header maps each of those onto plain C entry points:
 *
 *   - scene construction mirrors the reference constructors one to one
 *     (tpt_sphere <-> sphere::sphere, tpt_bvh_node <-> bvh_node::bvh_node ...)
 *     and returns integer handles instead of raw pointers;
 *   - tpt_trace_closest replaces world->hit(r, 0.001, FLT_MAX, rec) for a
 *     batch of rays;
 *   - tpt_render replaces the per-row sample loop of main.cpp:109-159 with
 *     color() (utils.cc:58-94) inside it;
 *   - tpt_render_params carries the config.ini keys (main.cpp:42-56).
 *
 * Conventions: every entry point returns a tpt_status (0 = TPT_OK) or, for
 * constructors, a non-negative handle / a negative tpt_status.  Buffers are
 * caller-owned; nothing is retained after a call returns unless stated.  No
 * entry point exits the process or throws across the ABI.  One tpt_context
 * per host thread.  There is no CPU fallback: device entry points return
 * TPT_ERR_NO_DEVICE when no CUDA device is usable.
 */
#ifndef TPT_H
#define TPT_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int32_t tpt_status;
enum {
  TPT_OK = 0,
  TPT_ERR_INVALID_ARGUMENT = 1,
  TPT_ERR_PARSE = 2,
  TPT_ERR_UNSUPPORTED = 3,      /* scene shape the device layout cannot express */
  TPT_ERR_NO_BOUNDING_BOX = 4,  /* reference: exit(-1) in box_axis_compare (hitable.cc:20-23) */
  TPT_ERR_CUDA = 5,
  TPT_ERR_OUT_OF_MEMORY = 6,
  TPT_ERR_DEVICE_TIMEOUT = 7,   /* a device loop hit its iteration limit */
  TPT_ERR_STACK_OVERFLOW = 8,   /* traversal stack deeper than the device stack */
  TPT_ERR_NO_DEVICE = 9,
  TPT_ERR_BAD_HANDLE = 10
};

/* Human-readable name of a status code (static storage). */
const char *tpt_status_string(tpt_status s);
/* Library version, e.g. "tpt-gb300 0.1". */
const char *tpt_version(void);
/* Detail of the last failing CUDA call on this host thread ("" if none). */
const char *tpt_last_error(void);

/* ------------------------------------------------------------------------
 * Scene construction.  A builder holds a scene graph made of the reference's
 * classes.  Handles are per-kind integers (textures, materials, hitables).
 * ---------------------------------------------------------------------- */
typedef struct tpt_builder tpt_builder;

tpt_status tpt_builder_create(tpt_builder **out);
void tpt_builder_destroy(tpt_builder *b);

/* Textures: headers/texture.h:15-51. */
int32_t tpt_constant_texture(tpt_builder *b, float r, float g, float bl);          /* texture.h:15-24 */
int32_t tpt_checker_texture(tpt_builder *b, int32_t odd, int32_t even);           /* texture.cc:4-16 */
int32_t tpt_perlin_noise_texture(tpt_builder *b, float scale);                    /* texture.cc:18-25 */
/* Shared perlin tables (perlin_noise.h:13-16): 256 gradients (x,y,z) and the
 * x, y, z permutations of 0..255.  Without this call the builder fills them
 * from its drand_r stream like perlin_noise.cc:3-21 (the permutation shuffle
 * uses a fixed-seed engine instead of the reference's clock seed). */
tpt_status tpt_perlin_tables(tpt_builder *b, const float *gradients768, const int32_t *perm768);
/* image_texture (texture.cc:27-42): RGB8, width*height*3 bytes, copied. */
int32_t tpt_image_texture(tpt_builder *b, const uint8_t *rgb, int32_t width, int32_t height);

/* Materials: headers/material.h:27-79. */
int32_t tpt_lambertian(tpt_builder *b, int32_t albedo_tex);                       /* material.cc:3-17 */
int32_t tpt_metal(tpt_builder *b, float r, float g, float bl, float fuzz);        /* material.h:39-50 */
int32_t tpt_dielectric(tpt_builder *b, float ref_idx);                            /* material.cc:19-70 */
int32_t tpt_diffuse_light(tpt_builder *b, int32_t emit_tex);                      /* material.cc:79-86 */
int32_t tpt_isotropic(tpt_builder *b, int32_t albedo_tex);                        /* material.h:72-79 */

/* Hitables: headers/sphere.h, rect_box.h, hitable.h, hitable_list.h. */
int32_t tpt_sphere(tpt_builder *b, float cx, float cy, float cz, float radius, int32_t mat);   /* sphere.h:6-21 */
int32_t tpt_moving_sphere(tpt_builder *b, float c0x, float c0y, float c0z, float c1x, float c1y, float c1z,
                          float t0, float t1, float radius, int32_t mat);                      /* sphere.h:23-40 */
int32_t tpt_xy_rect(tpt_builder *b, float x0, float x1, float y0, float y1, float k, int32_t mat); /* rect_box.h:5-15 */
int32_t tpt_xz_rect(tpt_builder *b, float x0, float x1, float z0, float z1, float k, int32_t mat); /* rect_box.h:17-30 */
int32_t tpt_yz_rect(tpt_builder *b, float y0, float y1, float z0, float z1, float k, int32_t mat); /* rect_box.h:32-42 */
int32_t tpt_flip_normal(tpt_builder *b, int32_t child);                                       /* rect_box.h:44-60 */
int32_t tpt_box(tpt_builder *b, float x0, float y0, float z0, float x1, float y1, float z1, int32_t mat); /* rect_box.h:62-74 */
int32_t tpt_translate(tpt_builder *b, int32_t child, float ox, float oy, float oz);           /* rect_box.h:77-99 */
int32_t tpt_rotate_y(tpt_builder *b, int32_t child, float angle_degrees);                     /* rect_box.h:101-116 */
int32_t tpt_constant_medium(tpt_builder *b, int32_t boundary, float density, int32_t tex);   /* hitable.h:58-69 */
int32_t tpt_hitable_list(tpt_builder *b, const int32_t *items, int32_t n);                   /* hitable_list.h:4-19 */
/* bvh_node (hitable.cc:32-56): built immediately, drawing its split axes from
 * the builder's drand_r stream (std::mt19937 in its default state when the
 * builder is created), so topology matches the reference bit for bit.
 * Returns TPT_ERR_NO_BOUNDING_BOX (negated) where the reference would exit. */
int32_t tpt_bvh_node(tpt_builder *b, const int32_t *items, int32_t n, float t0, float t1);

/* drand_r(min, max) (utils.cc:28-32) on the builder's stream: scene code that
 * draws its random layout through this shares one mt19937 stream with
 * bvh_node, exactly as the reference's scene functions share drand_r with
 * the bvh_node constructor on their thread. */
double tpt_builder_drand(tpt_builder *b, double min, double max);

tpt_status tpt_builder_set_world(tpt_builder *b, int32_t world);
/* light_shape argument of color() (utils.h:26-27); -1 = none (pure cosine). */
tpt_status tpt_builder_set_light_shape(tpt_builder *b, int32_t light_shape);
/* camera_with_blur constructor (camera.cc:2-21). */
tpt_status tpt_builder_set_camera(tpt_builder *b, const float lookfrom[3], const float lookat[3], const float vup[3],
                                  float vfov, float aspect, float aperture, float focus_dist, float t0, float t1);

/* ------------------------------------------------------------------------
 * Compiled scenes: the builder graph flattened into the device layout
 * (BVH nodes as 32-byte {min.xyz,left}{max.xyz,right} SoA records, leaf and
 * material tables).  Host memory; immutable.
 * ---------------------------------------------------------------------- */
typedef struct tpt_scene tpt_scene;

tpt_status tpt_scene_compile(const tpt_builder *b, tpt_scene **out);
/* Parse scene-description text (the statement format documented in
 * docs of the package loader) into a builder and compile it. */
tpt_status tpt_scene_from_text(const char *sd_text, tpt_scene **out, char *err, size_t errlen);
/* BVH topology the compiler flattens for every bvh_node.  REFERENCE (the
 * default) is the reference's own tree (random axis, median split,
 * hitable.cc:32-56), required for closest-hit parity.  SAH rebuilds each
 * bvh_node's primitives with a binned surface-area heuristic on the host;
 * LBVH leaves them to a linear BVH built on the GPU when the scene is
 * uploaded (Morton-ordered primitives, Karras 2012 radix tree; the build
 * runs again on every tpt_render_noalloc call).  Neither has a counterpart
 * in the reference: they give the same closest hits except which of several
 * primitives at exactly equal t wins, and renders that agree statistically,
 * usually faster on large scenes.  An LBVH tree's depth is known only after
 * the build: tpt_scene_upload fails with TPT_ERR_STACK_OVERFLOW if it
 * exceeds the traversal stack (tpt_scene_info.max_stack counts its BVHs as
 * one level).  tpt_scene_bvh_dump always reports the reference tree. */
enum { TPT_BVH_REFERENCE = 0, TPT_BVH_SAH = 1, TPT_BVH_LBVH = 2 };
tpt_status tpt_builder_set_bvh_build(tpt_builder *b, int32_t mode);
tpt_status tpt_scene_from_text_opt(const char *sd_text, int32_t bvh_build, tpt_scene **out, char *err,
                                   size_t errlen);
void tpt_scene_destroy(tpt_scene *s);

typedef struct {
  int32_t n_nodes, n_leaves, n_items, n_blas;
  int32_t n_materials, n_textures, n_lights, max_stack;
  int64_t arena_bytes;
} tpt_scene_info;
tpt_status tpt_scene_get_info(const tpt_scene *s, tpt_scene_info *out);

/* Pre-order dump of the BVH built for builder hitable `handle` (a
 * tpt_bvh_node).  Per node: box (6 floats) and (left, right), a child >= 0
 * being a pre-order node index and a child < 0 being -(1 + hitable handle of
 * the leaf).  Returns the node count (call with cap 0 to size), or < 0. */
int32_t tpt_scene_bvh_dump(const tpt_scene *s, int32_t handle, float *boxes, int32_t *kids, int32_t cap);

/* ------------------------------------------------------------------------
 * Device context.
 * ---------------------------------------------------------------------- */
typedef struct tpt_context tpt_context;

tpt_status tpt_context_create(int32_t device, tpt_context **out);
void tpt_context_destroy(tpt_context *ctx);
/* Use this cudaStream_t (passed as void*) for all later work; NULL = the
 * context's own stream. */
tpt_status tpt_context_set_stream(tpt_context *ctx, void *stream);
/* Copy a compiled scene into device memory (and build its BVHs there if it
 * was compiled with TPT_BVH_LBVH); returns a slot id. */
tpt_status tpt_scene_upload(tpt_context *ctx, const tpt_scene *s, int32_t *slot);
tpt_status tpt_scene_release(tpt_context *ctx, int32_t slot);

/* The GPU linear-BVH builder of TPT_BVH_LBVH over n boxes (host buffers,
 * 6 floats each: min xyz, max xyz).  Writes m = max(n - 1, 1) nodes in
 * pre-order: node_boxes (m x 6), node_kids (m x 2: >= 0 a node, < 0 ~box
 * index), node_skip (m: the pre-order index just past the node's subtree),
 * and *depth = levels of internal nodes.  Synchronous. */
tpt_status tpt_bvh_build_boxes(tpt_context *ctx, const float *boxes, int32_t n, float *node_boxes,
                               int32_t *node_kids, int32_t *node_skip, int32_t *depth);

/* Context options (tpt_context_set_option). */
enum {
  TPT_OPT_FLAT_NODES = 1  /* BVHs of at most this many nodes use the stackless walk
                             (default 48); applies to tpt_trace_closest and to renders
                             whose flat_nodes parameter is 0 */
};
tpt_status tpt_context_set_option(tpt_context *ctx, int32_t option, int64_t value);

/* Memory location flags for caller buffers. */
enum { TPT_MEM_HOST = 0, TPT_MEM_DEVICE = 1 };

/* Batched world->hit(r, 0.001, FLT_MAX, rec) (hitable.h:30-39).
 * rays: n x 7 floats (ox,oy,oz,dx,dy,dz,time).  hit_f: n x 9 floats
 * (t,u,v,px,py,pz,nx,ny,nz); hit_i: n x 2 int32 (hit flag, hitable handle of
 * the primitive hit, -1 on a miss).  The free-flight uniform of a
 * constant_medium is Philox-4x32-10 of (ray index, medium handle) keyed by
 * `seed`.  mem = TPT_MEM_HOST or TPT_MEM_DEVICE for all three buffers. */
tpt_status tpt_trace_closest(tpt_context *ctx, int32_t slot, const float *rays, int64_t n, uint64_t seed,
                             float *hit_f, int32_t *hit_i, int32_t mem);

/* Render parameters: the config.ini keys (main.cpp:42-56) plus the
 * integrator switches. */
enum { TPT_SEMANTICS_REFERENCE = 0, TPT_SEMANTICS_PHYSICAL = 1 };
enum { TPT_BACKGROUND_BLACK = 0, TPT_BACKGROUND_SKY = 1 };
/* AUTO = PERSISTENT: measured fastest on the Cornell workload. */
enum { TPT_ENGINE_AUTO = 0, TPT_ENGINE_WAVEFRONT = 1, TPT_ENGINE_PERSISTENT = 2 };
typedef struct {
  int32_t width, height;    /* [DEFAULT] width, height */
  int32_t spp;              /* [DEFAULT] sample */
  int32_t max_depth;        /* [DEFAULT] recur_depth */
  int32_t semantics;        /* TPT_SEMANTICS_* */
  int32_t background;       /* TPT_BACKGROUND_* */
  float sky_scale;          /* sky gradient scale (utils.cc:87-90 uses 0.1) */
  uint64_t seed;            /* RNG key */
  int32_t engine;           /* TPT_ENGINE_* */
  int32_t block;            /* threads per block, 0 = tuned (persistent engine: <= 128) */
  int32_t wave;             /* wavefront: path slots (0 = 1M); persistent: register
                               variant, minimum resident blocks 4 (default), 5, 6 or 8 */
  int32_t accumulate_fp64;  /* 1: also accumulate in double (out_rgb is the FP64 mean) */
  int32_t profile;          /* 1: time each traverse/shade launch with CUDA events */
  int32_t flat_nodes;       /* stackless-walk size limit; 0 = the context option */
  int32_t refill;           /* persistent engines: a warp's finished lanes take new camera
                               samples once at least this many are idle (1..32; 0 = 1) */
} tpt_render_params;

typedef struct {
  int64_t samples;          /* camera samples traced */
  int64_t segments;         /* rays traced (all bounces) */
  int32_t iterations;       /* wavefront iterations / persistent launches */
  int32_t kernel_launches;  /* kernels this library launched */
  double device_ms;         /* device time of the render, CUDA events */
  double traverse_ms;       /* profile=1: summed device time of the traversal launches */
  double shade_ms;          /* profile=1: summed device time of the shading launches */
  int32_t traverse_launches;
  int32_t shade_launches;
} tpt_render_stats;

void tpt_render_params_default(tpt_render_params *p);

/* Render the scene in `slot`.  out_rgb: width*height*3 floats, row 0 = top
 * image row, each the mean of de_nan(color()) over spp samples (linear, before
 * the gamma of main.cpp:136).  mem = TPT_MEM_HOST or TPT_MEM_DEVICE.
 * stats may be NULL. */
tpt_status tpt_render(tpt_context *ctx, int32_t slot, const tpt_render_params *p, float *out_rgb, int32_t mem,
                      tpt_render_stats *stats);

/* Render without allocating any memory (no counterpart in the reference).
 * For callers that cannot call cudaMalloc: a plugin inside a host program
 * that owns all device memory through its own pool (an allocation behind the
 * pool's back breaks its accounting or fails under its memory cap), or a
 * real-time loop that must not take the implicit device synchronisation of
 * an allocation.  The caller passes, in memory it owns:
 *   arena_dev    device buffer of at least tpt_scene_info.arena_bytes bytes;
 *                each call copies the compiled scene into it (host-to-device
 *                copies only),
 *   out_rgb_dev  device buffer of width*height*3 floats (the mean radiance,
 *                row 0 = top, as tpt_render writes it),
 *   stream       the cudaStream_t to run on (NULL = the legacy default).
 * The per-pixel accumulators and counters live in one file-scope device
 * array of TPT_NOALLOC_MAX_PIXELS*16 + 256 bytes (16 MiB), which every GPU
 * that loads the library holds until the process exits; images of more than
 * TPT_NOALLOC_MAX_PIXELS pixels are rejected with TPT_ERR_INVALID_ARGUMENT.
 * The persistent engine renders.  The call is synchronous: it waits for
 * `stream` before it returns (it reads the kernels' error flag back).  The
 * first call on a device looks up the array's device address
 * (cudaGetSymbolAddress), so make that first call before any stream capture.
 * All calls share the array, which keeps the last call's contents (each call
 * clears what it uses): calls that overlap on the GPU (other threads, other
 * streams) race and corrupt each other's images.  Fields of
 * tpt_render_params this call ignores: engine (always persistent), profile;
 * accumulate_fp64 = 1 is rejected with TPT_ERR_INVALID_ARGUMENT.  Every
 * TPT_ERR_INVALID_ARGUMENT return leaves its reason in tpt_last_error(). */
#define TPT_NOALLOC_MAX_PIXELS (1 << 20)
tpt_status tpt_render_noalloc(const tpt_scene *scene, void *arena_dev, int64_t arena_bytes,
                              const tpt_render_params *p, float *out_rgb_dev, void *stream);

/* Batched render: many scenes of uneven size, resolution and spp in one
 * persistent launch (configs of many small jobs).  Each item names an
 * uploaded scene, its frame size and spp, and its output (width*height*3
 * floats, TPT_MEM_HOST or TPT_MEM_DEVICE for all items).  `common` supplies
 * the remaining parameters (max_depth, semantics, background, seed, block,
 * wave = register variant, flat_nodes, profile); an item's image equals what
 * tpt_render would produce for it with the same parameters.  The launch
 * sequence (clear, persistent kernel, resolves) is captured once into a CUDA
 * graph and replayed while the items and parameters stay the same. */
typedef struct {
  int32_t slot;
  int32_t width, height, spp;
  float *out_rgb;
} tpt_batch_item;
enum { TPT_MAX_BATCH = 256 };
tpt_status tpt_render_batch(tpt_context *ctx, const tpt_batch_item *items, int32_t n, const tpt_render_params *common,
                            int32_t mem, tpt_render_stats *stats);

/* Autotuner: renders `probe_spp` samples per pixel (raised so that a probe
 * has at least 16 M samples: smaller probes measure launch tails) with each candidate
 * configuration - engine, threads per block, register variant, wavefront
 * queue size, stackless-walk threshold - times them with CUDA events, times
 * the three fastest again on a probe of ~0.1 s (at least 4x longer;
 * fastest of three runs: the leaders are often within a percent or two, and
 * a short probe's launch tail hides differences a full frame shows), writes
 * the winner into *p
 * (engine, block, wave, flat_nodes; the other fields are kept) and remembers
 * it for the slot, so later renders of that slot with engine =
 * TPT_ENGINE_AUTO use it.  best_msps (may be NULL) receives the winner's
 * Msamples/s. */
tpt_status tpt_autotune(tpt_context *ctx, int32_t slot, tpt_render_params *p, int32_t probe_spp, double *best_msps);
/* Autotuner of a batch: renders the batch with every item's spp divided by
 * spp_divisor (at least 1) for each candidate block size, register variant
 * and stackless-walk threshold of the batched persistent launch - and, when
 * every item is sphere-only, the stepped-walk kernel (wave 14-16) with 16 or
 * 24 waiting lanes per shading round (refill) - times them with CUDA
 * events, times the three fastest again (fastest of three runs) and writes
 * the winner into p (block, wave, flat_nodes, refill) for tpt_render_batch.
 * best_msps (may be NULL) receives its Msamples/s.
 * In tpt_render_batch, wave 14, 15 or 16 selects the stepped walk for
 * sphere-only batches (4, 5 or 6 resident blocks per SM): each lane advances
 * its BVH walk a few nodes per round and the lanes that finished shade
 * together once `refill` of them wait; other batches ignore it. */
tpt_status tpt_autotune_batch(tpt_context *ctx, const tpt_batch_item *items, int32_t n, tpt_render_params *p,
                              int32_t spp_divisor, double *best_msps);

/* ------------------------------------------------------------------------
 * Learned parts: fully fused FP16 MLPs on the 5th-generation tensor cores
 * (tcgen05.mma, FP32 accumulators in tensor memory; training and inference
 * alike), in -> [64, ReLU] x n_hidden -> out, no biases, weights
 * row-major [out][in] per layer, concatenated.  Supported shapes:
 * (112, 3, 48) path-guiding network, (64, 5, 16) radiance cache,
 * (32, 2, 16) test network.  Batches are device buffers of `rows` rows,
 * rows a multiple of 16; x is row-major f16 [rows][in], y f32 [rows][out].
 * (No counterpart in the reference.)
 * ---------------------------------------------------------------------- */
typedef struct tpt_mlp tpt_mlp;
tpt_status tpt_mlp_create(int32_t device, int32_t in_dim, int32_t n_hidden, int32_t out_dim, uint64_t seed,
                          tpt_mlp **out);
void tpt_mlp_destroy(tpt_mlp *m);
int64_t tpt_mlp_param_count(const tpt_mlp *m);
tpt_status tpt_mlp_set_params(tpt_mlp *m, const float *host_params);
tpt_status tpt_mlp_get_params(const tpt_mlp *m, float *host_params);
/* f32 weight gradients accumulated since the last Adam step (loss-scaled). */
tpt_status tpt_mlp_get_grad(const tpt_mlp *m, float *host_grad);
tpt_status tpt_mlp_forward(tpt_mlp *m, const void *x_f16, int64_t rows, float *y, void *stream);
/* Accumulates the weight gradient of sum(scale * dy * y) (dy: f32 [rows][out]). */
tpt_status tpt_mlp_backward_given(tpt_mlp *m, const void *x_f16, const float *dy, int64_t rows, float scale,
                                  void *stream);
/* Guiding network only: accumulates the weight gradient of the weighted vMF
 * mixture negative log-likelihood, sum_rows w * -log q(omega), times `scale`;
 * target: f32 [rows][4] = (omega.xyz unit, w).  loss_out (host, may be NULL)
 * receives the unscaled loss sum. */
tpt_status tpt_mlp_backward_vmf(tpt_mlp *m, const void *x_f16, const float *target, int64_t rows, float scale,
                                float *loss_out, void *stream);
/* Radiance-cache network only: accumulates the weight gradient of the
 * relative L2 loss of Mueller et al. 2021, sum_rows sum_rgb
 * (y - t)^2 / (sg(y)^2 + 0.01) with the denominator held constant, times
 * `scale`; target: f32 [rows][4] = (rgb, unused).  loss_out (host, may be
 * NULL) receives the unscaled loss sum. */
tpt_status tpt_mlp_backward_rel_l2(tpt_mlp *m, const void *x_f16, const float *target, int64_t rows, float scale,
                                   float *loss_out, void *stream);
/* The radiance cache's training step as the cached renderer runs it: row r
 * of the `rows`-row batch is record h(r) mod count of `records` (device, 5
 * float4 per record: the four feature float4 of tpt_nrc_encode, then the
 * target radiance), h the 32-bit mix of r, `step` and `key` the renderer
 * uses; the rows are encoded inside the training kernel (no input matrix in
 * memory) and the gradient of the relative L2 loss is accumulated as
 * tpt_mlp_backward_rel_l2 would for the same rows. */
tpt_status tpt_mlp_backward_rel_l2_records(tpt_mlp *m, const float *records, int64_t count, uint32_t key,
                                           uint32_t step, const float *lo, const float *extent, int64_t rows,
                                           float scale, float *loss_out, void *stream);
/* The learned parts' input encodings, one row per record (device buffers).
 * tpt_guide_encode: records of 3 float4 (position, weight), (normal, -),
 * (sampled direction, -) -> f16 rows of 112: the position normalised to the
 * box [lo, lo + extent] as a one-blob of 32 bins per axis, then the normal;
 * target (may be NULL) receives (direction, weight) per row, an unusable
 * record (non-finite or negative weight) a zero weight.
 * tpt_nrc_encode: records of `stride` float4 (>= 4; the first four are
 * (position, roughness), (outgoing direction, -), (normal, -), (albedo, -))
 * -> f16 rows of 64: a 12-octave triangle wave per position axis, spherical
 * one-blobs (4 + 4 bins) of the direction and the normal, a 4-bin roughness
 * one-blob, the albedo. */
tpt_status tpt_guide_encode(const float *records, int64_t count, const float *lo, const float *extent, void *x_f16,
                            float *target, void *stream);
tpt_status tpt_nrc_encode(const float *records, int64_t count, int32_t stride, const float *lo, const float *extent,
                          void *x_f16, void *stream);
/* Radiance-cache network only: the cached renderer's query evaluation.
 * queries: device, 6 float4 each - the four feature float4 of
 * tpt_nrc_encode, then (throughput rgb, pixel index as int32 bits), then
 * unused; accum: device, n_pixels float4.  For every query, encodes its
 * features (box [lo, lo + extent]), evaluates the network on the tensor
 * cores and adds throughput x max(output rgb, 0) (NaN components as 0) to
 * accum[pixel].xyz, in one kernel.  Queries naming a pixel >= n_pixels are
 * skipped and the call returns TPT_ERR_INVALID_ARGUMENT after the others
 * were added.  Synchronises the stream. */
tpt_status tpt_mlp_cache_accumulate(tpt_mlp *m, const float *queries, int64_t count, const float *lo,
                                    const float *extent, float *accum, int64_t n_pixels, void *stream);
/* Adam step (lr, beta 0.9/0.999, eps 1e-8) on the accumulated gradient
 * multiplied by inv_loss_scale; clears the gradient. */
tpt_status tpt_mlp_adam(tpt_mlp *m, float lr, float inv_loss_scale, void *stream);
const char *tpt_mlp_last_error(void);

/* Learned path guiding (no counterpart in the reference).  The image is
 * rendered in `passes` passes of spp/passes samples per pixel; after each
 * pass the guiding network (one-blob position + normal -> 8-lobe vMF mixture,
 * shape (112, 3, 48)) takes `train_steps` Adam steps on records of the
 * paths' first diffuse vertices (position, normal, sampled direction,
 * weight = the sample's contribution f L cos / pdf), and is then evaluated on
 * a grid_res^3 x 6-normal table.  From the second pass on, diffuse vertices
 * sample the table's mixture with probability alpha and the plain mixture
 * (light + cosine) otherwise, weighting by the one-sample MIS density
 * alpha q + (1 - alpha) p_plain, so the estimator stays unbiased.  Requires
 * TPT_SEMANTICS_PHYSICAL.  out_rgb as tpt_render. */
typedef struct {
  int32_t passes;       /* >= 1 */
  int32_t train_steps;  /* Adam steps after each pass */
  int32_t batch;        /* training rows per step (multiple of 16) */
  float lr;             /* Adam learning rate (1e-3) */
  int32_t grid_res;     /* table cells per axis (16) */
  float alpha;          /* guide probability at a diffuse vertex (0.5) */
  int32_t record_cap;   /* training records kept per pass (1 to 2^28) */
  uint64_t seed;        /* network initialisation and record sampling */
  float light_share;    /* probability of light sampling within the non-guide part
                           (0.5: the plain tracer's light/cosine mixture; 0: cosine
                           only, the guide then carries all light sampling) */
  int32_t warm_start;   /* 0: a fresh network (seed); 1: continue from the context's
                           network (the last guided render's, or tpt_learned_load's),
                           guiding from the first pass */
} tpt_guide_params;
typedef struct {
  double render_ms, train_ms;  /* device time spent rendering / training + table refresh */
  float final_loss;            /* mean training loss of the last step */
  int64_t records;             /* training records collected (all passes) */
} tpt_guide_stats;
void tpt_guide_params_default(tpt_guide_params *g);
tpt_status tpt_render_guided(tpt_context *ctx, int32_t slot, const tpt_render_params *p, const tpt_guide_params *g,
                             float *out_rgb, int32_t mem, tpt_render_stats *stats, tpt_guide_stats *gstats);
/* Training records of the last pass of the last tpt_render_guided call on
 * this context, copied to host memory: up to `cap` records of 12 floats,
 * (position, weight), (normal, 0), (sampled direction, 0).  *count receives
 * the number available.  For tests and diagnostics (no counterpart in the
 * reference). */
tpt_status tpt_guide_records(tpt_context *ctx, float *out, int64_t cap, int64_t *count);

/* Neural radiance cache (no counterpart in the reference).  Rendered in
 * `passes` passes; in every pass after the first, a path stops at its first
 * diffuse vertex (lambertian, or isotropic in physical semantics) whose
 * vertex number is at least terminate_depth (0 = camera hit), or earlier
 * (past the camera hit) once its path spread exceeds spread_c x the camera
 * vertex's, and adds throughput x cache(position, outgoing direction,
 * normal, albedo, roughness), the cache being an MLP of shape (64, 5, 16)
 * evaluated on the tensor cores for all such vertices at once; specular
 * vertices and lights are traced through.  Every train_stride-th path is a
 * training path: it is traced to full depth (contributing its unbiased
 * estimate) and records its first three diffuse vertices with their
 * measured outgoing radiance; after each pass the cache takes train_steps
 * Adam steps on them (relative L2 loss).  The first pass, first_pass_spp
 * samples per pixel, traces every path to full depth.
 * The estimator is biased by the cache's error; the plain tracer is its
 * fallback and the yardstick for that error.  Defaults in parentheses. */
typedef struct {
  int32_t passes;           /* >= 1 (3) */
  int32_t train_steps;      /* Adam steps after each pass (512) */
  int32_t batch;            /* training rows per step (16384) */
  float lr;                 /* Adam learning rate (3e-3) */
  int32_t terminate_depth;  /* the latest vertex a path ends at into the cache (3) */
  int32_t train_stride;     /* every n-th path trains the cache (16) */
  int32_t record_cap;       /* training records per pass */
  int32_t query_cap;        /* cache queries per launch (paths are launched in chunks) */
  uint64_t seed;
  int32_t warm_start;       /* 0: a fresh cache (seed); 1: continue from the context's
                               cache (the last cached render's, or tpt_learned_load's),
                               querying it from the first pass */
  int32_t first_pass_spp;   /* spp of the uncached first pass (8; 0: spp / passes, like
                               the others); the other passes share the rest */
  int32_t first_train_steps; /* Adam steps after the first pass (0: train_steps) */
  float spread_c;           /* > 0: a path also ends into the cache at a diffuse vertex
                               past the camera hit once its path spread (Mueller et
                               al. 2021, section 5) exceeds spread_c x the camera
                               vertex's; terminate_depth stays the latest end (0.01;
                               0: off) */
} tpt_nrc_params;
typedef struct {
  double render_ms, infer_ms, train_ms;
  float final_loss;
  int64_t records, queries;
} tpt_nrc_stats;
void tpt_nrc_params_default(tpt_nrc_params *n);
/* Chooses the engine of the slot's cached renders (TPT_ENGINE_AUTO): traces
 * a short cached render of p's size and settings (probe_spp >= 2 samples per
 * pixel, an untrained cache) on the wavefront engine and on the persistent
 * engine at 64 or 128 threads and 4 or 5 resident blocks per SM, and keeps
 * the one with the shortest tracing time (*engine_out, may be NULL).  The cache's own
 * training and inference cost the same on both engines.  The probes render
 * with fresh caches, so the context's cache is replaced (load a checkpoint
 * for a warm start afterwards). */
tpt_status tpt_autotune_nrc(tpt_context *ctx, int32_t slot, const tpt_render_params *p, int32_t probe_spp,
                            int32_t *engine_out);
tpt_status tpt_render_nrc(tpt_context *ctx, int32_t slot, const tpt_render_params *p, const tpt_nrc_params *n,
                          float *out_rgb, int32_t mem, tpt_render_stats *stats, tpt_nrc_stats *nstats);

/* Checkpoint and resume of the learned parts (no counterpart in the
 * reference, which has no learned state): the context's guiding network
 * (TPT_NET_GUIDE) or radiance cache (TPT_NET_CACHE) as 3 P + 1 floats -
 * weights, Adam first and second moments (P each), and the Adam step count.
 * tpt_learned_save with out = NULL (or cap too small) only reports *count;
 * it fails with TPT_ERR_BAD_HANDLE before the context has rendered with that
 * network.  tpt_learned_load restores a checkpoint into a context (creating
 * the network), so that the next render with warm_start = 1 continues from
 * it; a network's inputs are positions normalised to the scene's world box,
 * so a checkpoint carries over between scenes with the same box. */
enum { TPT_NET_GUIDE = 0, TPT_NET_CACHE = 1 };
tpt_status tpt_learned_save(tpt_context *ctx, int32_t which, float *out, int64_t cap, int64_t *count);
tpt_status tpt_learned_load(tpt_context *ctx, int32_t which, const float *in, int64_t count);

/* ------------------------------------------------------------------------
 * The formats on either side of the render loop of main.cpp.
 * ---------------------------------------------------------------------- */
/* config.ini (main.cpp:29-56): section/key per field. */
typedef struct {
  int32_t width;            /* [DEFAULT] width (400) */
  int32_t height;           /* [DEFAULT] height (200) */
  int32_t sample;           /* [DEFAULT] sample: samples per pixel (10) */
  int32_t recur_depth;      /* [DEFAULT] recur_depth: max depth (50) */
  float fov;                /* [DEFAULT] fov, degrees (90) */
  int32_t allow_bonus_pic;  /* [DEFAULT] allow_bonus_pic (0) */
  int32_t bonus_pic;        /* [DEFAULT] bonus_pic: snapshots (10) */
  float aperture;           /* [BLUR] aperture (0.2) */
  float start_time;         /* [CAM_MOTION] start_time (0) */
  float end_time;           /* [CAM_MOTION] end_time (1) */
} tpt_config;
/* The defaults of main.cpp:31-40. */
void tpt_config_default(tpt_config *c);
/* Parses INI text with the grammar of the reference's inipp: trimmed lines,
 * ';' comments, [sections], key = value (the first definition of a key in a
 * section wins); a field changes only when its key is present and its whole
 * value converts (else it keeps its current value). */
tpt_status tpt_config_parse(const char *text, tpt_config *c);
/* tpt_config_parse of a file; an unreadable file leaves *c unchanged and
 * returns TPT_OK, as main.cpp:29 never checks its stream. */
tpt_status tpt_config_load(const char *path, tpt_config *c);
/* The camera inputs of a compiled scene, tpt_builder_set_camera's arguments
 * in order: lookfrom[3], lookat[3], vup[3], vfov, aspect, aperture, focus,
 * time0, time1. */
tpt_status tpt_scene_get_camera(const tpt_scene *s, float out[15]);
/* Replaces a compiled scene's camera (main.cpp:86-90 builds it from the
 * config's fov, aperture and shutter); takes effect at the next upload. */
tpt_status tpt_scene_set_camera(tpt_scene *s, const float lookfrom[3], const float lookat[3], const float vup[3],
                                float vfov, float aspect, float aperture, float focus, float time0, float time1);
/* allow_bonus_pic (main.cpp:111-131,192-216): renders spp samples per pixel
 * and also the running means after every slice = spp / bonus_pic samples:
 * snapshots_rgb holds bonus_pic images (width*height*3 floats each), image k
 * the mean of each pixel's first (k+1)*slice samples, identical to what
 * tpt_render gives at spp = (k+1)*slice.  out_rgb receives the mean of all
 * spp samples.  bonus_pic > spp is TPT_ERR_INVALID_ARGUMENT (the reference
 * divides by zero).  Persistent engine; physical or reference semantics. */
tpt_status tpt_render_snapshots(tpt_context *ctx, int32_t slot, const tpt_render_params *p, int32_t bonus_pic,
                                float *out_rgb, float *snapshots_rgb, int32_t mem, tpt_render_stats *stats);
/* A frame split across GPUs (the reference renders one frame in row tasks,
 * main.cpp:157-159; here the split is over samples, so every rank renders
 * the whole image).  tpt_render_range renders samples [sample_begin,
 * sample_end) of every pixel (p->spp is ignored) with the persistent engine
 * and writes the per-pixel SUMS, not the mean, into accum_dev: device
 * memory of width*height float4 (16-byte aligned; xyz = radiance sum, w
 * unused), cleared first.  Each sample draws from its own (pixel, sample
 * index) stream, so the shares of any partition of [0, spp) add up - after
 * a sum-reduce of the accumulators across ranks - to what one GPU
 * accumulates for the whole frame, up to float summation order.
 * tpt_resolve_sums turns summed accumulators of spp samples per pixel into
 * the mean image (TPT_MEM_HOST or TPT_MEM_DEVICE output).  Both wait for the
 * context's stream.  (No counterpart in the reference.) */
tpt_status tpt_render_range(tpt_context *ctx, int32_t slot, const tpt_render_params *p, int32_t sample_begin,
                            int32_t sample_end, float *accum_dev, tpt_render_stats *stats);
tpt_status tpt_resolve_sums(tpt_context *ctx, const float *accum_dev, int32_t width, int32_t height, int32_t spp,
                            float *out_rgb, int32_t mem);
/* Reads a PPM image (P3 or P6, maxval <= 255, '#' comments) for
 * tpt_image_texture: the stand-in for the stb_image decode of
 * utils.cc:236-240.  Call with rgb8 = NULL to get the size; then with a
 * buffer of cap >= width*height*3 bytes (row 0 = top). */
tpt_status tpt_read_ppm(const char *path, uint8_t *rgb8, int64_t cap, int32_t *width, int32_t *height);
/* `count` quantised images side by side in one PPM P3 file: the strip
 * main.cpp:222-243 asks ImageMagick's `convert +append` for. */
tpt_status tpt_write_ppm_strip(const char *path, const uint8_t *const *images, int32_t count, int32_t width,
                               int32_t height);

/* Host helpers: reference output quantisation (main.cpp:135-142,176-182) and
 * the PPM P3 writer of main.cpp:69,183-189. */
void tpt_quantize(const float *mean_rgb, int64_t n_pixels, uint8_t *rgb8);
tpt_status tpt_write_ppm(const char *path, const uint8_t *rgb8, int32_t width, int32_t height);

#ifdef __cplusplus
}
#endif
#endif /* TPT_H */
