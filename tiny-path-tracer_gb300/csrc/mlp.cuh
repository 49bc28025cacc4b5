// mlp.cuh - fully fused FP16 multilayer perceptrons on the tensor cores
// (mma.sync.m16n8k16, f16 inputs, f32 accumulation) for the learned parts of
// the renderer: the path-guiding network and the radiance cache.
//
// Shape: in_dim (multiple of 16, <= 128) -> n_hidden layers of width 64
// (ReLU) -> out_dim (multiple of 8, <= 64, linear).  No biases.  Weights are
// stored row-major per layer, [out][in], concatenated layer after layer.
//
// One warp owns 16 rows of the batch at a time.  A layer's accumulator tiles
// (16x8, f32) are converted in registers into the next layer's A fragments
// (16x16, f16): accumulator tiles 2k and 2k+1 hold exactly the rows and
// columns of A tile k, so activations never leave registers in the forward
// pass.  Weights live in shared memory with rows padded by 8 halves, which
// makes the B-fragment loads bank-conflict free.
#ifndef TPT_MLP_CUH
#define TPT_MLP_CUH

#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace tpt {
namespace mlp {

constexpr int HID = 64;
constexpr int MAX_IN = 128;
constexpr int MAX_OUT = 64;
constexpr int MAX_HIDDEN = 6;
constexpr int WARPS = 8;  // warps per CTA (128 rows per CTA step)

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
// shared-memory layout: W (padded rows of in+8 halves) for every layer
__host__ __device__ inline int smem_w_offset(const Net &n, int l) {
  int off = 0;
  for (int i = 0; i < l; i++) off += layer_out(n, i) * (layer_in(n, i) + 8);
  return off;
}
__host__ __device__ inline int smem_w_halves(const Net &n) { return smem_w_offset(n, n_layers(n)); }
// transposed copies for the backward pass, layers 1..L-1: [in][out+8]
__host__ __device__ inline int smem_wt_offset(const Net &n, int l) {
  int off = 0;
  for (int i = 1; i < l; i++) off += layer_in(n, i) * (layer_out(n, i) + 8);
  return off;
}
__host__ __device__ inline int smem_wt_halves(const Net &n) { return smem_wt_offset(n, n_layers(n)); }

__device__ __forceinline__ void mma16816(float (&c)[4], uint32_t a0, uint32_t a1, uint32_t a2, uint32_t a3,
                                         uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.f16.f16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

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

// Copies all weights into shared memory (row stride in+8) and, if `wt`,
// the transposed hidden/output layers (row stride out+8).  16-byte loads:
// every layer's row length and offset are multiples of 8 halves, and the
// padded shared rows keep 16-byte alignment.
__device__ inline void load_weights(const Net &n, __half *sw, __half *swt) {
  for (int l = 0; l < n_layers(n); l++) {
    const int K = layer_in(n, l), N = layer_out(n, l);
    const uint4 *g = reinterpret_cast<const uint4 *>(n.w16 + layer_offset(n, l));
    __half *s = sw + smem_w_offset(n, l);
    const int chunks = N * K / 8;
    for (int c = threadIdx.x; c < chunks; c += blockDim.x) {
      const int i = c * 8, o = i / K, k = i - o * K;  // 8 consecutive inputs of output o
      const uint4 v = __ldg(g + c);
      *reinterpret_cast<uint4 *>(s + o * (K + 8) + k) = v;
      if (swt && l > 0) {
        const __half *h = reinterpret_cast<const __half *>(&v);
        __half *t = swt + smem_wt_offset(n, l) + o;
#pragma unroll
        for (int j = 0; j < 8; j++) t[(k + j) * (N + 8)] = h[j];
      }
    }
  }
}

// One layer: acc[N/8][4] = A (16 x K, fragments a[K/16][4]) * W^T.
template <int K, int N>
__device__ __forceinline__ void layer_mma(const uint32_t (&a)[K / 16][4], const __half *w, float (&acc)[N / 8][4]) {
  const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
#pragma unroll
  for (int j = 0; j < N / 8; j++) acc[j][0] = acc[j][1] = acc[j][2] = acc[j][3] = 0.f;
#pragma unroll
  for (int kk = 0; kk < K / 16; kk++) {
#pragma unroll
    for (int j = 0; j < N / 8; j++) {
      const __half *row = w + (j * 8 + g) * (K + 8) + kk * 16 + 2 * t;
      const uint32_t b0 = *reinterpret_cast<const uint32_t *>(row);
      const uint32_t b1 = *reinterpret_cast<const uint32_t *>(row + 8);
      mma16816(acc[j], a[kk][0], a[kk][1], a[kk][2], a[kk][3], b0, b1);
    }
  }
}

// Accumulator tiles -> next layer's A fragments, with ReLU.
template <int N>
__device__ __forceinline__ void relu_to_frag(const float (&acc)[N / 8][4], uint32_t (&a)[N / 16][4]) {
#pragma unroll
  for (int kk = 0; kk < N / 16; kk++) {
    a[kk][0] = pack2(fmaxf(acc[2 * kk][0], 0.f), fmaxf(acc[2 * kk][1], 0.f));
    a[kk][1] = pack2(fmaxf(acc[2 * kk][2], 0.f), fmaxf(acc[2 * kk][3], 0.f));
    a[kk][2] = pack2(fmaxf(acc[2 * kk + 1][0], 0.f), fmaxf(acc[2 * kk + 1][1], 0.f));
    a[kk][3] = pack2(fmaxf(acc[2 * kk + 1][2], 0.f), fmaxf(acc[2 * kk + 1][3], 0.f));
  }
}

// A fragments of 16 rows of a row-major f16 matrix (row stride ld halves).
template <int K>
__device__ __forceinline__ void load_frag_rows(const __half *x, int ld, uint32_t (&a)[K / 16][4]) {
  const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
#pragma unroll
  for (int kk = 0; kk < K / 16; kk++) {
    const __half *r0 = x + g * ld + kk * 16 + 2 * t;
    const __half *r1 = r0 + 8 * ld;
    a[kk][0] = *reinterpret_cast<const uint32_t *>(r0);
    a[kk][1] = *reinterpret_cast<const uint32_t *>(r1);
    a[kk][2] = *reinterpret_cast<const uint32_t *>(r0 + 8);
    a[kk][3] = *reinterpret_cast<const uint32_t *>(r1 + 8);
  }
}

}  // namespace mlp
}  // namespace tpt
#endif
