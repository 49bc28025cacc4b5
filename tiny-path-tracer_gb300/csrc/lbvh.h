// lbvh.h - GPU linear-BVH build (TPT_BVH_LBVH), shared by the scene upload
// paths (kernels.cu) and the builder kernels (lbvh.cu).
//
// The host compiler leaves every bvh_node of a TPT_BVH_LBVH scene as a build
// job: its primitives' leaves and boxes are in the arena, and max(n - 1, 1)
// node slots are reserved at the job's node base.  After the arena is on the
// device, lbvh_build() fills those slots (node_lo/hi, node_kids, node_skip) in
// the same pre-order layout the host flattener writes.
#ifndef TPT_LBVH_H
#define TPT_LBVH_H
#include <cuda_runtime.h>
#include <stdint.h>

#include "arena.h"

namespace tpt {

// lbvh_jobs[j] = {node base, primitive count n, first primitive, first key}
// lbvh_prims[2 p]     = {min.xyz, leaf ref of the primitive (int bits, < 0)}
// lbvh_prims[2 p + 1] = {max.xyz, job index (int bits)}
// Keys of job j occupy the padded range [first key, first key + pow2ceil(n)).
struct LbvhArgs {
  const i4 *jobs;
  int32_t n_jobs;
  const f4 *prims;
  int32_t n_prims;
  int64_t n_keys;   // sum of the jobs' padded key ranges
  int32_t max_pad;  // largest padded key range
  f4 *node_lo, *node_hi, *node_kids;
  int32_t *node_skip;
  int32_t n_leaves;  // leaf records of the scene (bound of the leaf references)
  const i4 *leaf_hdr;   // the scene's leaves (null: no scene), for sphere
  const f4 *leaf_data;  // leaves' data carried in node_kids
  void *work;        // lbvh_work_bytes(n_prims, n_jobs, n_keys)
};

inline size_t lbvh_align(size_t x) { return (x + 255) & ~(size_t)255; }

// Bytes of build scratch: keys (8 B per padded key), per internal node its
// range (16 B) and children (8 B), parent links, positions and counters
// (4 x 4 B per primitive), per job its depth, then one counter.
inline size_t lbvh_work_bytes(int64_t n_prims, int32_t n_jobs, int64_t n_keys) {
  return lbvh_align((size_t)n_keys * 8) + lbvh_align((size_t)n_prims * 16) + lbvh_align((size_t)n_prims * 8) +
         4 * lbvh_align((size_t)n_prims * 4) + lbvh_align((size_t)(n_jobs + 1) * 4);
}

// Inside the work area, valid after lbvh_build(): the per-job tree depth
// (levels of internal nodes), followed by the number of nodes whose child or
// skip reference left the job's range (0 unless the build is broken; the
// upload then fails instead of handing the tree to the traversal).
int32_t *lbvh_depths(void *work, int64_t n_prims, int32_t n_jobs, int64_t n_keys);

// Enqueues the build on `s` (no allocation, no synchronisation).
cudaError_t lbvh_build(const LbvhArgs &a, cudaStream_t s);

#ifdef __CUDACC__
#define TPT_LBVH_HD __host__ __device__
#else
#define TPT_LBVH_HD
#endif

// Padded key range of a job of n primitives.
TPT_LBVH_HD inline int64_t lbvh_pad(int64_t n) {
  int64_t p = 1;
  while (p < n) p <<= 1;
  return p;
}

}  // namespace tpt
#endif
