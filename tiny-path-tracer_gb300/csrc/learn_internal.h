// learn_internal.h - host interface between the renderer (kernels.cu) and
// the learned parts (learn.cu).
#ifndef TPT_LEARN_INTERNAL_H
#define TPT_LEARN_INTERNAL_H
#include <cuda_runtime.h>

#include "../../include/tpt.h"

namespace tpt {
struct GuideNet;
tpt_status guide_create(int device, uint64_t seed, GuideNet **out);
void guide_destroy(GuideNet *g);
tpt_status guide_train(GuideNet *g, const float4 *records, int count, int steps, int batch, float lr, float3 lo,
                       float3 ext, uint64_t seed, cudaStream_t s);
tpt_status guide_refresh(GuideNet *g, int res, float4 *table, cudaStream_t s);
float guide_last_loss(const GuideNet *g);

struct CacheNet;
tpt_status cache_create(int device, uint64_t seed, CacheNet **out);
void cache_destroy(CacheNet *g);
tpt_status cache_train(CacheNet *g, const float4 *records, int count, int steps, int batch, float lr, float3 lo,
                       float3 ext, uint32_t key, cudaStream_t s);
// Evaluates the cache at `count` queries (6 float4 each: vertex features,
// then throughput and pixel) and adds throughput x max(cache, 0) to accum
// (one float4 per pixel), in one tensor-core kernel.
tpt_status cache_infer(CacheNet *g, const float4 *queries, int count, float3 lo, float3 ext, float4 *accum,
                       cudaStream_t s);
// TPT_ERR_CUDA if an MMA completion wait of the cache's kernels timed out.
tpt_status cache_check(CacheNet *g, cudaStream_t s);
float cache_last_loss(const CacheNet *g);

// Checkpoint of a network's training state: weights, Adam moments, step
// count (3 P + 1 floats); loading also refreshes the FP16 weights.
tpt_mlp *guide_mlp(GuideNet *g);
tpt_mlp *cache_mlp(CacheNet *g);
int64_t mlp_state_count(const tpt_mlp *m);
tpt_status mlp_save_state(const tpt_mlp *m, float *out);
tpt_status mlp_load_state(tpt_mlp *m, const float *in);
}  // namespace tpt
#endif
