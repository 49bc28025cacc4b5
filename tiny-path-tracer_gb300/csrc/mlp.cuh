// mlp.cuh - the shape and weight layout of the learned parts' FP16
// multilayer perceptrons (the path-guiding network and the radiance cache),
// and the f16 packing helpers their tensor-core kernels (learn.cu) share.
//
// Shape: in_dim (multiple of 16, <= 128) -> n_hidden layers of width 64
// (ReLU) -> out_dim (multiple of 16, <= 64, linear).  No biases.  Weights are
// stored row-major per layer, [out][in], concatenated layer after layer.
#ifndef TPT_MLP_CUH
#define TPT_MLP_CUH

#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace tpt {
namespace mlp {

constexpr int HID = 64;

struct Net {
  int in_dim, n_hidden, out_dim;
  const __half *w16;  // f16 weights, concatenated [out][in] per layer
  float *grad;        // f32 gradient accumulators, same layout
};

__host__ __device__ inline int n_layers(const Net &n) { return n.n_hidden + 1; }
__host__ __device__ inline int layer_in(const Net &n, int l) { return l == 0 ? n.in_dim : HID; }
__host__ __device__ inline int layer_out(const Net &n, int l) { return l == n.n_hidden ? n.out_dim : HID; }
__host__ __device__ inline int layer_offset(const Net &n, int l) {  // in weights
  int off = 0;
  for (int i = 0; i < l; i++) off += layer_in(n, i) * layer_out(n, i);
  return off;
}
__host__ __device__ inline int param_count(const Net &n) { return layer_offset(n, n_layers(n)); }

__device__ __forceinline__ uint32_t pack2(float lo, float hi) {
  __half2 h = __floats2half2_rn(lo, hi);
  return *reinterpret_cast<uint32_t *>(&h);
}
// Gradients: saturate at the largest finite half instead of overflowing to
// inf (an inf times a zero weight or mask becomes NaN in the next product).
__device__ __forceinline__ uint32_t pack2_sat(float lo, float hi) {
  return pack2(fminf(fmaxf(lo, -65504.f), 65504.f), fminf(fmaxf(hi, -65504.f), 65504.f));
}
__device__ __forceinline__ float2 unpack2(uint32_t v) {
  __half2 h = *reinterpret_cast<__half2 *>(&v);
  return __half22float2(h);
}

}  // namespace mlp
}  // namespace tpt
#endif
